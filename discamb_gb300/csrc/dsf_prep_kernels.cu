// Resident per-structure tables of the structure-factor kernel.
//
//   RS[h][s]  per (reflection, symmetry operation): h' = R^T h (integer and
//             real), the phase offset h.t (2^32 fixed point and real; exact,
//             translations are multiples of 1/24) and the density-normalised
//             harmonics d_lm of h'/|h'| in the global frame
//             (pre_atom_loop_sf_calc, src/Scattering/HansenCoppens_SF_Engine3.cpp:319-418;
//              getDensityNormalized<4>, include/discamb/MathUtilities/real_spherical_harmonics.h:102-115)
//   TR[t][h]  per (type, reflection): spherical f = f_core + P_val f_val(|h|/kappa)
//             (or the n-Gaussian f0 of IAM types) and the signed radial terms
//             4 pi N_l g_l(|h|/kappa') of the deformation density
//             (pre_atom_loop_sf_calc, same file :365-418)
//   TRM[t][h] f_val, P_val df_val/dkappa and 4 pi N_l dg_l/dkappa' (the
//             multipole-parameter adjoint; no counterpart in the reference)
// Rows past the last reflection (padding to a multiple of 16) are zero.
#include "dsf_device.cuh"
#include "dsf_math.cuh"
#include "dsf_sf_kernel.cuh"

namespace dsf {

template <typename R>
struct SelP;
template <>
struct SelP<float> {
    static __device__ const TypeRadialT<float> *types(const DevStructure &S) { return S.types_f; }
    static __device__ const float *pre(const DevStructure &S) { return S.term_pre_f; }
    static __device__ const float *zexp(const DevStructure &S) { return S.term_exp_f; }
};
template <>
struct SelP<double> {
    static __device__ const TypeRadialT<double> *types(const DevStructure &S) { return S.types_d; }
    static __device__ const double *pre(const DevStructure &S) { return S.term_pre_d; }
    static __device__ const double *zexp(const DevStructure &S) { return S.term_exp_d; }
};

__device__ __forceinline__ float fexp_(float x) { return expf(x); }
__device__ __forceinline__ double fexp_(double x) { return exp(x); }

template <typename R>
__global__ void rs_prep_kernel(DevStructure S, int n_hkl_pad, RsRec<R> *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nS = S.n_sym;
    if (i >= n_hkl_pad * nS) return;
    const int h = i / nS, s = i - h * nS;
    RsRec<R> rec;
    for (int q = 0; q < 28; q++) rec.y[q] = R(0);
    for (int q = 0; q < 4; q++) rec.hf[q] = R(0);
    rec.hi = make_int4(0, 0, 0, 0);
    if (h < S.n_hkl) {
        const int4 hv = S.hkl[h];
        const int *Rm = S.sym_rot + 9 * s;
        const int *t = S.sym_t24 + 3 * s;
        const int hp0 = hv.x * Rm[0] + hv.y * Rm[3] + hv.z * Rm[6];
        const int hp1 = hv.x * Rm[1] + hv.y * Rm[4] + hv.z * Rm[7];
        const int hp2 = hv.x * Rm[2] + hv.y * Rm[5] + hv.z * Rm[8];
        int tr = (hv.x * t[0] + hv.y * t[1] + hv.z * t[2]) % 24;
        if (tr < 0) tr += 24;
        const uint32_t tq = (uint32_t)((((uint64_t)tr << 32) + 12u) / 24u);
        rec.hi = make_int4(hp0, hp1, hp2, (int)tq);
        rec.hf[0] = R(hp0);
        rec.hf[1] = R(hp1);
        rec.hf[2] = R(hp2);
        rec.hf[3] = R(tr / 24.0);
        if (S.model == MODEL_HC) {
            const double cx = S.B[0] * hp0 + S.B[1] * hp1 + S.B[2] * hp2;
            const double cy = S.B[3] * hp0 + S.B[4] * hp1 + S.B[5] * hp2;
            const double cz = S.B[6] * hp0 + S.B[7] * hp1 + S.B[8] * hp2;
            const double n2 = cx * cx + cy * cy + cz * cz;
            if (n2 > 1e-20) {  // F(000): no deformation term
                const double inv = 1.0 / sqrt(n2);
                double v[25];
                harmonic_polys<double>(cx * inv, cy * inv, cz * inv, v);
                for (int q = 0; q < 25; q++) rec.y[q] = R(v[q] * kDensityNorm[q]);
            }
        } else {
            // the ADP quadratic form's monomials of h' (the coset kernels read them instead of forming them per
            // atom), rounded as the kernel's own products in R would be
            const R a = rec.hf[0], b = rec.hf[1], c = rec.hf[2];
            rec.y[0] = a * a; rec.y[1] = b * b; rec.y[2] = c * c;
            rec.y[3] = R(2) * a * b; rec.y[4] = R(2) * a * c; rec.y[5] = R(2) * b * c;
        }
    }
    out[i] = rec;
}

// radial terms of one (type, reflection), see the file comment
template <typename R>
__device__ void radial_terms2(const DevStructure &S, const TypeRadialT<R> &t, R h2, R *base, R *mpv, bool mp)
{
    for (int q = 0; q < 8; q++) {
        base[q] = R(0);
        mpv[q] = R(0);
    }
    const R hl = sqrt(h2);
    const R K = R(2.0 * DSF_PI) * hl;
    if (S.model == MODEL_IAM) {
        R s = t.iam_c;
        const R x2 = h2 * R(0.25);
        for (int q = 0; q < t.iam_n; q++) s += t.iam_a[q] * fexp_(-t.iam_b[q] * x2);
        base[0] = s;
        return;
    }
    if (S.model != MODEL_HC) return;
    const R *pre = SelP<R>::pre(S);
    const R *zx = SelP<R>::zexp(S);
    R fc = R(0);
    for (int q = t.core_begin; q < t.core_end; q++) fc += pre[q] * gcore<R>(0, S.term_m[q], K, zx[q]);
    const R Kv = K * t.inv_kappa, Kd = K * t.inv_kappa_p;
    R fv = R(0), dfv = R(0);
    for (int q = t.val_begin; q < t.val_end; q++) {
        fv += pre[q] * gcore<R>(0, S.term_m[q], Kv, zx[q]);
        if (mp) dfv -= R(2) * pre[q] * gcore<R>(1, S.term_m[q], Kv, zx[q]);  // dG(n,0)/dK = -G(n+1,1)
    }
    base[0] = fc + t.pv * fv;
    mpv[0] = fv;
    mpv[1] = t.pv * dfv * (-Kv * t.inv_kappa);
    for (int l = 0; l < t.n_def; l++) {
        const R g = gcore<R>(l, t.def_m[l], Kd, t.zeta);
        base[1 + l] = t.def_pre[l] * g;
        if (mp && Kd > R(0)) {
            // dG/dK = (l/K) G(n,l) - G(n+1,l+1); the second term's prefactor is 2(l+1) times larger
            const R dg = R(l) / Kd * g - R(2 * (l + 1)) * gcore<R>(l + 1, t.def_m[l], Kd, t.zeta);
            mpv[2 + l] = t.def_pre[l] * dg * (-Kd * t.inv_kappa_p);
        }
    }
}

// Mott-Bethe conversion of the X-ray form factor of an HC type to electron
// scattering, as the reference engine does per term (HansenCoppens_SF_Engine3.cpp:1387-1397):
// f_e = C (Z - f_x) / s^2 with s^2 = |h|^2 / 4 and C = 0.023934 (the anomalous
// term stays additive), f_e(000) = the element's electron f at s = 0.  Linear in
// f_x, so the deformation radial terms and the multipole-adjoint terms scale by
// -C / s^2 (zero at 000).  Evaluated in FP64 for both table precisions: Z - f_x
// cancels at low angle.
__device__ void electron_terms(const DevStructure &S, int t, double h2, double *base, double *mpv, bool mp)
{
    const TypeRadialT<double> &ty = S.types_d[t];
    radial_terms2<double>(S, ty, h2, base, mpv, mp);
    if (h2 > 0.0) {
        const double s2 = 0.25 * h2, c = 0.023934;
        base[0] = c * (ty.e_z - base[0]) / s2;
        for (int q = 1; q < 8; q++) base[q] *= -c / s2;
        for (int q = 0; q < 8; q++) mpv[q] *= -c / s2;
    } else {
        base[0] = ty.e_f000;
        for (int q = 1; q < 8; q++) base[q] = 0.0;
        for (int q = 0; q < 8; q++) mpv[q] = 0.0;
    }
}

template <typename R>
__global__ void tr_prep_kernel(DevStructure S, int n_hkl_pad, R *tr, R *trm, int mp)
{
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (h >= n_hkl_pad) return;
    R base[8], mpv[8];
    if (h < S.n_hkl && S.electron && S.model == MODEL_HC) {
        double bd[8], md[8];
        electron_terms(S, t, S.h2[h], bd, md, mp != 0);
        for (int q = 0; q < 8; q++) {
            base[q] = R(bd[q]);
            mpv[q] = R(md[q]);
        }
    } else if (h < S.n_hkl) {
        const R h2 = R(S.h2[h]);
        radial_terms2<R>(S, SelP<R>::types(S)[t], h2, base, mpv, mp != 0);
    } else {
        for (int q = 0; q < 8; q++) base[q] = mpv[q] = R(0);
    }
    const size_t row = ((size_t)t * n_hkl_pad + h) * 8;
    if (tr)
        for (int q = 0; q < 8; q++) tr[row + q] = base[q];
    if (mp && trm)
        for (int q = 0; q < 8; q++) trm[row + q] = mpv[q];
}

cudaError_t launch_rs_prep(const DevStructure &S, int n_hkl_pad, void *rs_f, void *rs_d, cudaStream_t st)
{
    const int n = n_hkl_pad * S.n_sym;
    if (rs_f) rs_prep_kernel<float><<<(n + 127) / 128, 128, 0, st>>>(S, n_hkl_pad, (RsRec<float> *)rs_f);
    if (rs_d) rs_prep_kernel<double><<<(n + 127) / 128, 128, 0, st>>>(S, n_hkl_pad, (RsRec<double> *)rs_d);
    return cudaGetLastError();
}

cudaError_t launch_tr_prep(const DevStructure &S, int n_hkl_pad, void *tr_f, void *tr_d, void *trm_f, void *trm_d,
                           bool mp, cudaStream_t st)
{
    dim3 grid((n_hkl_pad + 127) / 128, S.n_types);
    float *tf = mp ? nullptr : (float *)tr_f, *mf = mp ? (float *)trm_f : nullptr;
    double *td = mp ? nullptr : (double *)tr_d, *md = mp ? (double *)trm_d : nullptr;
    if (tf || mf) tr_prep_kernel<float><<<grid, 128, 0, st>>>(S, n_hkl_pad, tf, mf, mp);
    if (td || md) tr_prep_kernel<double><<<grid, 128, 0, st>>>(S, n_hkl_pad, td, md, mp);
    return cudaGetLastError();
}

size_t rs_record_bytes(bool fp64) { return fp64 ? sizeof(RsRec<double>) : sizeof(RsRec<float>); }

// Per atom (engine order): the rotation blocks D_l (l = 0..4) of the
// density-normalised real harmonics between the atom's local frame and the
// crystal frame, d(L^T u) = D d(u), fitted over K sample directions
// (D_l^T = pinv_l B_l with B_l the harmonics of the rotated directions), and
// the global-frame populations P_glob = D^T P up to the type's l_max
// (calculateGlobalCoordinatesPlm, src/Scattering/HansenCoppens_SF_Engine3.cpp:594-654).
// fit = [pinv_0 .. pinv_4] ([2l+1][K] each, at offset K l^2) then the K directions [K][3].
__global__ void global_plm_kernel(int n, int K, const int *perm, const int *atom_type, const double *lcs,
                                  const double *type_plm, const int *type_lmax, const double *fit, double *dmat,
                                  double *pg_d, float *pg_f)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int o = perm[a], t = atom_type[o];
    const double *L = lcs + 9 * (size_t)o;
    const double *u = fit + (size_t)K * 25;
    double D[165];
    for (int q = 0; q < 165; q++) D[q] = 0.0;
    for (int k = 0; k < K; k++) {
        double v[3], p[25];
        for (int j = 0; j < 3; j++) v[j] = L[0 + j] * u[3 * k] + L[3 + j] * u[3 * k + 1] + L[6 + j] * u[3 * k + 2];
        harmonic_polys<double>(v[0], v[1], v[2], p);
        int off = 0;
        for (int l = 0; l <= 4; l++) {
            const int nl = 2 * l + 1;
            const double *pinv = fit + (size_t)K * l * l;
            for (int i = 0; i < nl; i++) {
                const double b = p[l * l + i] * kDensityNorm[l * l + i];
                for (int j = 0; j < nl; j++) D[off + i * nl + j] += pinv[j * K + k] * b;
            }
            off += nl * nl;
        }
    }
    double *Dout = dmat + 165 * (size_t)a;
    for (int q = 0; q < 165; q++) Dout[q] = D[q];
    const int lmax = type_lmax[t];
    const double *P = type_plm + 25 * (size_t)t;
    int off = 0;
    for (int l = 0; l <= 4; l++) {
        const int nl = 2 * l + 1;
        for (int j = 0; j < nl; j++) {
            double v = 0.0;
            if (l <= lmax)
                for (int i = 0; i < nl; i++) v += D[off + i * nl + j] * P[l * l + i];
            pg_d[25 * (size_t)a + l * l + j] = v;
            pg_f[25 * (size_t)a + l * l + j] = (float)v;
        }
        off += nl * nl;
    }
}

cudaError_t launch_global_plm(int n, int K, const int *perm, const int *atom_type, const double *lcs,
                              const double *type_plm, const int *type_lmax, const double *fit, double *dmat,
                              double *pg_d, float *pg_f, cudaStream_t st)
{
    global_plm_kernel<<<(n + 63) / 64, 64, 0, st>>>(n, K, perm, atom_type, lcs, type_plm, type_lmax, fit, dmat,
                                                     pg_d, pg_f);
    return cudaGetLastError();
}

// Form factors of every atom at one reciprocal vector (Cartesian hc), in the
// caller's atom order, without anomalous dispersion; excluded atoms get 0.
// HC: f_core + P_val f_val(|h|/kappa) + sum_l i^l 4 pi N_l g_l(|h|/kappa')
// sum_m P_lm d_lm(h/|h|) with the crystal-frame P_lm (no deformation term at
// h = 0), as HansenCoppens_SF_Engine::calculateFormFactors
// (src/Scattering/HansenCoppens_SF_Engine.cpp:383-500, which interpolates the
// spherical part from splines where this evaluates it); IAM: the n-Gaussian
// f0(|h|) (IamFormFactorCalculationsManager::calculateCart,
// src/Scattering/IamFormFactorCalculationsManager.cpp:147-161).
__global__ void form_factor_kernel(DevStructure S, double hx, double hy, double hz, const int *include,
                                   double2 *out)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;  // engine (sorted) atom
    if (a >= S.n_atoms) return;
    const int orig = S.atom_orig[a];
    if (include && !include[orig]) {
        out[orig] = make_double2(0.0, 0.0);
        return;
    }
    int lo = 0, hi = S.n_tiles - 1;  // the atom's tile: last with tile_begin <= a
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (S.tile_begin[mid] <= a) lo = mid;
        else hi = mid - 1;
    }
    const int t = S.tile_types[lo * kMaxTileTypes + S.atom_ltype[a]];
    const double h2 = hx * hx + hy * hy + hz * hz;
    double base[8], mpv[8];
    radial_terms2<double>(S, S.types_d[t], h2, base, mpv, false);
    double fre = base[0], fim = 0.0;
    if (S.model == MODEL_HC && h2 > 1e-20) {
        const double inv = 1.0 / sqrt(h2);
        double v[25];
        harmonic_polys<double>(hx * inv, hy * inv, hz * inv, v);
        const double *pg = S.atom_pg_d + 25 * (size_t)a;
        double A[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int q = 0; q < 25; q++) A[q < 1 ? 0 : q < 4 ? 1 : q < 9 ? 2 : q < 16 ? 3 : 4] += pg[q] * v[q] * kDensityNorm[q];
        fre += base[1] * A[0] + base[3] * A[2] + base[5] * A[4];  // signed radial terms r_l = base[1 + l]
        fim += base[2] * A[1] + base[4] * A[3];
    }
    out[orig] = make_double2(fre, fim);
}

cudaError_t launch_form_factors(const DevStructure &S, const double *hc, const int *include, double2 *out,
                                cudaStream_t st)
{
    form_factor_kernel<<<(S.n_atoms + 127) / 128, 128, 0, st>>>(S, hc[0], hc[1], hc[2], include, out);
    return cudaGetLastError();
}

}  // namespace dsf
