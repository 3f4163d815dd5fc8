// Fused structure-factor + adjoint kernel for sm_103a.
//
// One block owns one tile of up to 128 atoms (one atom per thread, atoms
// sorted by type so a tile holds few types) and a contiguous chunk of
// reflections.  Reflections are staged in shared memory in sub-tiles: per
// (reflection, symmetry operation) the rotated index h' = R^T h (as integers
// for the phase and as reals for the derivative multipliers), the phase
// offset h.t and the 25 harmonics d_lm(h'/|h'|); per (reflection, type of the
// tile) the spherical form factor and the radial Fourier-Bessel terms of the
// deformation density.  Each thread then runs the sum over operations for
// its atom, reduces the per-reflection partial F across the block with warp
// shuffles and keeps its own derivative sums in registers.  Cross-block
// accumulation is in FP64 (atomics on F per reflection and on the per-atom
// derivative channels).
//
// Reference loop restated: HansenCoppens_SF_Engine3::calculateSF_Serial*
// (src/Scattering/HansenCoppens_SF_Engine3.cpp:1030-1509, 1511-1992,
// 2649-2894) and AnyScattererStructureFactorCalculator::calculateStructure
// FactorsAndDerivatives (src/Scattering/AnyScattererStructureFactor
// Calculator.cpp:614-829).
//
// R = double: the plain form, FP64 throughout.
// R = float : the FP32-bulk form.  Phases are reduced exactly in integer
// arithmetic (fractional coordinates as 2^32 fixed point, integer h', h.t
// from integer translations in 1/24) and turned into sin/cos by a
// polynomial on the exact remainder, so no FP64 is needed per term (FP64
// runs at 1/64 of the FP32 rate on GB300).  Derivative sums over a block's
// reflections are Kahan-compensated FP32; F and the sums over blocks are
// FP64.
#include "dsf_device.cuh"
#include "dsf_math.cuh"

namespace dsf {

template <typename R>
struct Vec2;
template <>
struct Vec2<float> { using T = float2; };
template <>
struct Vec2<double> { using T = double2; };

// sin and cos of 2 pi (P 2^-32 + lo) for a phase P in 2^32 fixed point (the
// exact integer reduction mod one turn) and a small FP32 remainder lo (in
// turns).  Quadrant from the two top bits, remainder angle in [-pi/4, pi/4]
// exact in FP32 up to rounding, Taylor polynomials to degree 9 (sin) and 8
// (cos): truncation below 3e-8, so the result is limited by FP32 rounding
// (~1e-7 absolute) instead of the ~1e-6 of the hardware approximation.
__device__ __forceinline__ void sincos_fixed(uint32_t P, float lo, float *sn, float *cs)
{
    const uint32_t q = (P + 0x20000000u) >> 30;
    const int32_t r = (int32_t)(P - (q << 30));
    const float th = fmaf((float)r, 1.4629180792671596e-09f, 6.283185307179586f * lo);
    const float t2 = th * th;
    float sp = fmaf(t2, 2.7557319e-06f, -1.9841270e-04f);
    sp = fmaf(t2, sp, 8.3333333e-03f);
    sp = fmaf(t2, sp, -1.6666667e-01f);
    const float sv = fmaf(th * t2, sp, th);
    float cp = fmaf(t2, 2.4801587e-05f, -1.3888889e-03f);
    cp = fmaf(t2, cp, 4.1666668e-02f);
    cp = fmaf(t2, cp, -0.5f);
    const float cv = fmaf(t2, cp, 1.0f);
    float ss = (q & 1u) ? cv : sv;
    float cc = (q & 1u) ? sv : cv;
    if (q & 2u) ss = -ss;
    if ((q + 1u) & 2u) cc = -cc;
    *sn = ss;
    *cs = cc;
}

// temperature factor from the exponent of the ADP quadratic form: FP64 exp;
// FP32 exp2 (the FP32 ADPs are stored multiplied by log2 e)
template <typename R>
__device__ __forceinline__ R texp(R x);
template <>
__device__ __forceinline__ float texp<float>(float x) { return exp2f(x); }
template <>
__device__ __forceinline__ double texp<double>(double x) { return exp(x); }

__device__ __forceinline__ float fexp(float x) { return expf(x); }
__device__ __forceinline__ double fexp(double x) { return exp(x); }

template <typename R>
__device__ __forceinline__ R shfl_xor(R v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

template <typename R>
struct Sel;
template <>
struct Sel<float> {
    static __device__ const TypeRadialT<float> *types(const DevStructure &S) { return S.types_f; }
    static __device__ const float *pre(const DevStructure &S) { return S.term_pre_f; }
    static __device__ const float *zexp(const DevStructure &S) { return S.term_exp_f; }
    static __device__ float B(const DevStructure &S, int i) { return S.Bf[i]; }
    static __device__ float h2(const DevStructure &S, int i) { return S.h2f[i]; }
    static __device__ float2 gw(const CallBuffers &C, int i) { return C.gw_f[i]; }
};
template <>
struct Sel<double> {
    static __device__ const TypeRadialT<double> *types(const DevStructure &S) { return S.types_d; }
    static __device__ const double *pre(const DevStructure &S) { return S.term_pre_d; }
    static __device__ const double *zexp(const DevStructure &S) { return S.term_exp_d; }
    static __device__ double B(const DevStructure &S, int i) { return S.B[i]; }
    static __device__ double h2(const DevStructure &S, int i) { return S.h2[i]; }
    static __device__ double2 gw(const CallBuffers &C, int i) { return C.gw_d[i]; }
};

// radial terms of one (reflection, type): out[0] = spherical f (core + Pv*val
// or the Gaussian f0), out[1..5] = signed 4 pi N_l g_l (signs of i^l folded:
// +,+,-,-,+ for real/imag bookkeeping), out[6] = f_val, out[7] = Pv df_val/dkappa,
// out[8..12] = signed 4 pi N_l dg_l/dkappa'
template <typename R>
__device__ void radial_terms(const DevStructure &S, const TypeRadialT<R> &t, int model, R h2, R *out, bool mp)
{
    const R hl = sqrt(h2);
    const R K = R(2.0 * DSF_PI) * hl;
    for (int q = 0; q < kRad; q++) out[q] = R(0);
    if (model == MODEL_IAM) {
        R s = t.iam_c;
        const R x2 = h2 * R(0.25);
        for (int q = 0; q < t.iam_n; q++) s += t.iam_a[q] * fexp(-t.iam_b[q] * x2);
        out[0] = s;
        return;
    }
    if (model != MODEL_HC) return;
    const R *pre = Sel<R>::pre(S);
    const R *zx = Sel<R>::zexp(S);
    R fc = R(0);
    for (int q = t.core_begin; q < t.core_end; q++) fc += pre[q] * gcore<R>(0, S.term_m[q], K, zx[q]);
    const R Kv = K * t.inv_kappa, Kd = K * t.inv_kappa_p;
    R fv = R(0), dfv = R(0);
    for (int q = t.val_begin; q < t.val_end; q++) {
        fv += pre[q] * gcore<R>(0, S.term_m[q], Kv, zx[q]);
        if (mp) dfv -= R(2) * pre[q] * gcore<R>(1, S.term_m[q], Kv, zx[q]);  // dG(n,0)/dK = -G(n+1,1)
    }
    out[0] = fc + t.pv * fv;
    out[6] = fv;
    out[7] = t.pv * dfv * (-Kv * t.inv_kappa);
    for (int l = 0; l < t.n_def; l++) {
        const R g = gcore<R>(l, t.def_m[l], Kd, t.zeta);
        out[1 + l] = t.def_pre[l] * g;
        if (mp && Kd > R(0)) {
            // dG/dK = (l/K) G(n,l) - G(n+1,l+1); prefactor ratio of the second term 2(l+1)
            const R dg = R(l) / Kd * g - R(2 * (l + 1)) * gcore<R>(l + 1, t.def_m[l], Kd, t.zeta);
            out[8 + l] = t.def_pre[l] * dg * (-Kd * t.inv_kappa_p);
        }
    }
}

// Kahan-compensated add of a partial sum into a running total
template <typename R>
__device__ __forceinline__ void kahan_add(R &sum, R &comp, R v)
{
    const R y = v - comp;
    const R t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

template <typename R, bool MP>
__global__ void __launch_bounds__(kTileAtoms)
sf_grad_kernel(DevStructure S, CallBuffers C, int hkl_chunk, int ht)
{
    using R2 = typename Vec2<R>::T;
    constexpr bool F32 = sizeof(R) == 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nS = S.n_sym;
    const int tile = blockIdx.x;
    const int chunk = blockIdx.y;
    const int h_begin = chunk * hkl_chunk;
    const int h_end = min(S.n_hkl, h_begin + hkl_chunk);
    if (h_begin >= h_end) return;
    const int a_begin = S.tile_begin[tile], a_end = S.tile_begin[tile + 1];
    const int nT = S.tile_ntypes[tile];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kWarps = kTileAtoms / 32;
    const bool table_model = S.model == MODEL_TABLE;
    const bool hc_model = S.model == MODEL_HC;

    // shared memory carve-up (16-byte aligned pieces first)
    int4 *sHi = reinterpret_cast<int4 *>(smem_raw);                       // [ht][nS] h'(int), phase offset
    R *sHf = reinterpret_cast<R *>(sHi + (size_t)ht * nS);                // [ht][nS][4] h' (real), offset (FP64)
    R *sY = sHf + (size_t)ht * nS * 4;                                      // [ht][nS][25]
    R *sRad = sY + (size_t)ht * nS * 25;                                    // [ht][kMaxTileTypes][kRad]
    R2 *sG = reinterpret_cast<R2 *>(sRad + (size_t)ht * kMaxTileTypes * kRad);  // [ht]
    R2 *sF = sG + ht;                                                       // [kWarps][ht]
    R *sH2 = reinterpret_cast<R *>(sF + kWarps * ht);                      // [ht]
    int *sRot = reinterpret_cast<int *>(sH2 + ht);                          // [nS][9]
    int *sT24 = sRot + nS * 9;                                              // [nS][3]
    int *sTypes = sT24 + nS * 3;                                            // [nT]

    for (int i = tid; i < nS * 9; i += blockDim.x) sRot[i] = S.sym_rot[i];
    for (int i = tid; i < nS * 3; i += blockDim.x) sT24[i] = S.sym_t24[i];
    for (int i = tid; i < nT; i += blockDim.x) sTypes[i] = S.tile_types[tile * kMaxTileTypes + i];

    // per-atom registers
    const int a = a_begin + tid;
    const bool have = a < a_end;
    bool active = false;
    int lt = 0, adpk = 0;
    R w = R(0), pg[25], adp[6];
    R anre = R(0), anim = R(0);
    uint32_t xq0 = 0, xq1 = 0, xq2 = 0;
    R x0 = R(0), x1 = R(0), x2 = R(0);  // FP32: low parts (turns); FP64: coordinates
#pragma unroll
    for (int q = 0; q < 25; q++) pg[q] = R(0);
#pragma unroll
    for (int q = 0; q < 6; q++) adp[q] = R(0);
    if (have) {
        active = S.atom_active[a] != 0;
        lt = S.atom_ltype[a];
        adpk = S.atom_adpk[a];
        if constexpr (F32) {
            w = S.atom_w_f[a];
            const float2 an = S.atom_anom_f[a];
            anre = an.x; anim = an.y;
            xq0 = S.atom_xq[3 * a]; xq1 = S.atom_xq[3 * a + 1]; xq2 = S.atom_xq[3 * a + 2];
            x0 = S.atom_xlo[3 * a]; x1 = S.atom_xlo[3 * a + 1]; x2 = S.atom_xlo[3 * a + 2];
#pragma unroll
            for (int q = 0; q < 6; q++) adp[q] = S.atom_adp_f[6 * a + q];
            if (hc_model)
#pragma unroll
                for (int q = 0; q < 25; q++) pg[q] = S.atom_pg_f[25 * a + q];
        } else {
            w = S.atom_w_d[a];
            const double2 an = S.atom_anom_d[a];
            anre = an.x; anim = an.y;
            x0 = S.atom_xd[3 * a]; x1 = S.atom_xd[3 * a + 1]; x2 = S.atom_xd[3 * a + 2];
#pragma unroll
            for (int q = 0; q < 6; q++) adp[q] = S.atom_adp_d[6 * a + q];
            if (hc_model)
#pragma unroll
                for (int q = 0; q < 25; q++) pg[q] = S.atom_pg_d[25 * a + q];
        }
    }
    const int a_orig = have ? S.atom_orig[a] : 0;

    // derivative totals of this block (running Kahan sums in R)
    constexpr int NT = MP ? 38 : 13;
    R tot[NT], cmp[NT];
#pragma unroll
    for (int q = 0; q < NT; q++) { tot[q] = R(0); cmp[q] = R(0); }

    for (int h0 = h_begin; h0 < h_end; h0 += ht) {
        const int nh = min(ht, h_end - h0);
        __syncthreads();
        // ---- stage reflections: h', phase offsets, harmonics
        for (int i = tid; i < nh * nS; i += blockDim.x) {
            const int hl = i / nS, s = i - hl * nS;
            const int4 hv = S.hkl[h0 + hl];
            const int *Rm = sRot + 9 * s;
            // h' = R^T h (row vector h times R)
            const int hp0 = hv.x * Rm[0] + hv.y * Rm[3] + hv.z * Rm[6];
            const int hp1 = hv.x * Rm[1] + hv.y * Rm[4] + hv.z * Rm[7];
            const int hp2 = hv.x * Rm[2] + hv.y * Rm[5] + hv.z * Rm[8];
            // h.t mod 1, exact: translations are multiples of 1/24
            int tr = (hv.x * sT24[3 * s] + hv.y * sT24[3 * s + 1] + hv.z * sT24[3 * s + 2]) % 24;
            if (tr < 0) tr += 24;
            const uint32_t tq = (uint32_t)((((uint64_t)tr << 32) + 12u) / 24u);
            sHi[i] = make_int4(hp0, hp1, hp2, (int)tq);
            R *hf = sHf + 4 * (size_t)i;
            hf[0] = R(hp0); hf[1] = R(hp1); hf[2] = R(hp2);
            hf[3] = F32 ? R(0) : R(tr) * (R(1) / R(24));
            R *y = sY + 25 * (size_t)i;
            if (hc_model) {
                const R cx = Sel<R>::B(S, 0) * R(hp0) + Sel<R>::B(S, 1) * R(hp1) + Sel<R>::B(S, 2) * R(hp2);
                const R cy = Sel<R>::B(S, 3) * R(hp0) + Sel<R>::B(S, 4) * R(hp1) + Sel<R>::B(S, 5) * R(hp2);
                const R cz = Sel<R>::B(S, 6) * R(hp0) + Sel<R>::B(S, 7) * R(hp1) + Sel<R>::B(S, 8) * R(hp2);
                const R n2 = cx * cx + cy * cy + cz * cz;
                if (n2 > R(1e-20)) {
                    const R inv = rsqrt_<R>(n2);
                    R v[25];
                    harmonic_polys<R>(cx * inv, cy * inv, cz * inv, v);
#pragma unroll
                    for (int q = 0; q < 25; q++) y[q] = v[q] * R(kDensityNorm[q]);
                } else {
#pragma unroll
                    for (int q = 0; q < 25; q++) y[q] = R(0);  // F(000): no deformation term
                }
            }
        }
        for (int i = tid; i < nh * nT; i += blockDim.x) {
            const int hl = i / nT, t = i - hl * nT;
            R rad[kRad];
            radial_terms<R>(S, Sel<R>::types(S)[sTypes[t]], S.model, Sel<R>::h2(S, h0 + hl), rad, MP);
            R *dst = sRad + ((size_t)hl * kMaxTileTypes + t) * kRad;
#pragma unroll
            for (int q = 0; q < kRad; q++) dst[q] = rad[q];
        }
        for (int i = tid; i < nh; i += blockDim.x) {
            sG[i] = Sel<R>::gw(C, h0 + i);
            sH2[i] = Sel<R>::h2(S, h0 + i);
        }
        __syncthreads();

        // ---- per-atom sums over the reflections of the sub-tile
        R part[NT];
#pragma unroll
        for (int q = 0; q < NT; q++) part[q] = R(0);

        for (int hl = 0; hl < nh; hl++) {
            R Fre = R(0), Fim = R(0);
            if (active) {
                const R2 g = sG[hl];
                const R *rad = sRad + ((size_t)hl * kMaxTileTypes + lt) * kRad;
                const R fsre = rad[0] + anre, fsim = anim;
                const R r0 = rad[1], r1 = rad[2], r2 = rad[3], r3 = rad[4], r4 = rad[5];
                R Tiso = R(1);
                if (adpk == 1) Tiso = texp<R>(-adp[0] * sH2[hl]);
                const R gre = g.x * Tiso, gim = g.y * Tiso;  // adjoint weight with the isotropic factor
                R Ure = 0, Uim = 0;
                R Xre[3] = {0, 0, 0}, Xim[3] = {0, 0, 0};
                R Are[6] = {0, 0, 0, 0, 0, 0}, Aim[6] = {0, 0, 0, 0, 0, 0};
                R Ere = 0, Eim = 0, Kre = 0, Kim = 0;
                const int4 *hib = sHi + (size_t)hl * nS;
                const R *hfb = sHf + (size_t)hl * nS * 4;
                const R *yb = sY + (size_t)hl * nS * 25;
                for (int s = 0; s < nS; s++) {
                    const R *hf = hfb + 4 * s;
                    const R h0f = hf[0], h1f = hf[1], h2f = hf[2];
                    R sn, cs;
                    if constexpr (F32) {
                        const int4 hi = hib[s];
                        const uint32_t P = (uint32_t)hi.x * xq0 + (uint32_t)hi.y * xq1 + (uint32_t)hi.z * xq2 +
                                           (uint32_t)hi.w;
                        sincos_fixed(P, h0f * x0 + h1f * x1 + h2f * x2, &sn, &cs);
                    } else {
                        double ph = h0f * x0 + h1f * x1 + h2f * x2 + hf[3];
                        ph -= rint(ph);
                        sincospi(2.0 * ph, &sn, &cs);
                    }
                    R zre = cs, zim = sn;  // e^{i theta} T_s
                    R m6[6];
                    if (adpk == 6) {
                        m6[0] = h0f * h0f; m6[1] = h1f * h1f; m6[2] = h2f * h2f;
                        m6[3] = R(2) * h0f * h1f; m6[4] = R(2) * h0f * h2f; m6[5] = R(2) * h1f * h2f;
                        const R q = adp[0] * m6[0] + adp[1] * m6[1] + adp[2] * m6[2] + adp[3] * m6[3] +
                                    adp[4] * m6[4] + adp[5] * m6[5];
                        const R T = texp<R>(-q);
                        zre *= T; zim *= T;
                    }
                    R fre, fim;
                    R A0 = 0, A1 = 0, A2 = 0, A3 = 0, A4 = 0;
                    const R *y = yb + 25 * s;
                    if (table_model) {
                        if constexpr (F32) {
                            const float2 tv = S.table_f[((size_t)(h0 + hl) * nS + s) * S.n_atoms + a_orig];
                            fre = tv.x + anre; fim = tv.y + anim;
                        } else {
                            const double2 tv = S.table_d[((size_t)(h0 + hl) * nS + s) * S.n_atoms + a_orig];
                            fre = tv.x + anre; fim = tv.y + anim;
                        }
                    } else if (hc_model) {
                        A0 = pg[0] * y[0];
                        A1 = pg[1] * y[1] + pg[2] * y[2] + pg[3] * y[3];
                        A2 = pg[4] * y[4] + pg[5] * y[5] + pg[6] * y[6] + pg[7] * y[7] + pg[8] * y[8];
                        A3 = pg[9] * y[9] + pg[10] * y[10] + pg[11] * y[11] + pg[12] * y[12] + pg[13] * y[13] +
                             pg[14] * y[14] + pg[15] * y[15];
                        A4 = pg[16] * y[16] + pg[17] * y[17] + pg[18] * y[18] + pg[19] * y[19] + pg[20] * y[20] +
                             pg[21] * y[21] + pg[22] * y[22] + pg[23] * y[23] + pg[24] * y[24];
                        fre = fsre + r0 * A0 + r2 * A2 + r4 * A4;
                        fim = fsim + r1 * A1 + r3 * A3;
                    } else {
                        fre = fsre;
                        fim = fsim;
                    }
                    const R ure = fre * zre - fim * zim;
                    const R uim = fre * zim + fim * zre;
                    Ure += ure; Uim += uim;
                    Xre[0] += h0f * ure; Xim[0] += h0f * uim;
                    Xre[1] += h1f * ure; Xim[1] += h1f * uim;
                    Xre[2] += h2f * ure; Xim[2] += h2f * uim;
                    if (adpk == 6) {
#pragma unroll
                        for (int k = 0; k < 6; k++) { Are[k] -= m6[k] * ure; Aim[k] -= m6[k] * uim; }
                    }
                    if constexpr (MP) {
                        if (hc_model) {
                            Ere += zre; Eim += zim;
                            // q_l = Re(g i^l rr_l z): even l rs_l Re(gz), odd l -rs_l Im(gz)
                            const R wre = gre * zre - gim * zim, wim = gre * zim + gim * zre;
                            const R q0 = r0 * wre, q1 = -r1 * wim, q2 = r2 * wre, q3 = -r3 * wim, q4 = r4 * wre;
                            part[CH_PLM] += q0 * y[0];
#pragma unroll
                            for (int q = 1; q < 4; q++) part[CH_PLM + q] += q1 * y[q];
#pragma unroll
                            for (int q = 4; q < 9; q++) part[CH_PLM + q] += q2 * y[q];
#pragma unroll
                            for (int q = 9; q < 16; q++) part[CH_PLM + q] += q3 * y[q];
#pragma unroll
                            for (int q = 16; q < 25; q++) part[CH_PLM + q] += q4 * y[q];
                            const R dre = rad[8] * A0 + rad[10] * A2 + rad[12] * A4;
                            const R dim = rad[9] * A1 + rad[11] * A3;
                            Kre += dre * zre - dim * zim;
                            Kim += dre * zim + dim * zre;
                        }
                    }
                }
                if (adpk == 1) {
                    Ure *= Tiso; Uim *= Tiso;
#pragma unroll
                    for (int j = 0; j < 3; j++) { Xre[j] *= Tiso; Xim[j] *= Tiso; }
                    Ere *= Tiso; Eim *= Tiso; Kre *= Tiso; Kim *= Tiso;
                }
                Fre = w * Ure;
                Fim = w * Uim;
                const R gU = g.x * Ure - g.y * Uim;  // Re(g U)
                part[CH_OCC] += gU;
                if (adpk == 1) part[CH_ADP] -= sH2[hl] * gU;
                if (adpk == 6) {
#pragma unroll
                    for (int k = 0; k < 6; k++) part[CH_ADP + k] += g.x * Are[k] - g.y * Aim[k];
                }
#pragma unroll
                for (int j = 0; j < 3; j++) part[CH_XYZ + j] -= g.x * Xim[j] + g.y * Xre[j];  // -Im(g X)
                if constexpr (MP) {
                    const R gE = g.x * Ere - g.y * Eim;
                    part[CH_PV] += rad[6] * gE;
                    part[CH_KAPPA] += rad[7] * gE;
                    part[CH_KAPPA_P] += g.x * Kre - g.y * Kim;
                }
            }
            // block reduction of the partial F of this reflection
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                Fre += shfl_xor<R>(Fre, o);
                Fim += shfl_xor<R>(Fim, o);
            }
            if (lane == 0) {
                R2 v;
                v.x = Fre; v.y = Fim;
                sF[warp * ht + hl] = v;
            }
        }
        // fold the sub-tile sums into the running totals
#pragma unroll
        for (int q = 0; q < NT; q++) kahan_add<R>(tot[q], cmp[q], part[q]);
        __syncthreads();
        for (int i = tid; i < nh; i += blockDim.x) {
            R sre = 0, sim = 0;
#pragma unroll
            for (int wp = 0; wp < kWarps; wp++) {
                const R2 v = sF[wp * ht + i];
                sre += v.x;
                sim += v.y;
            }
            atomicAdd(&C.f_acc[h0 + i].x, (double)sre);
            atomicAdd(&C.f_acc[h0 + i].y, (double)sim);
        }
    }
    if (active) {
        double *G = C.g_acc + (size_t)a * kNch;
#pragma unroll
        for (int j = 0; j < 3; j++) atomicAdd(G + CH_XYZ + j, (double)tot[CH_XYZ + j] - (double)cmp[CH_XYZ + j]);
        if (adpk == 1) atomicAdd(G + CH_ADP, (double)tot[CH_ADP] - (double)cmp[CH_ADP]);
        if (adpk == 6)
#pragma unroll
            for (int k = 0; k < 6; k++) atomicAdd(G + CH_ADP + k, (double)tot[CH_ADP + k] - (double)cmp[CH_ADP + k]);
        atomicAdd(G + CH_OCC, (double)tot[CH_OCC] - (double)cmp[CH_OCC]);
        if constexpr (MP) {
#pragma unroll
            for (int q = CH_PV; q < NT; q++) atomicAdd(G + q, (double)tot[q] - (double)cmp[q]);
        }
    }
}

// shared memory bytes of one block
template <typename R>
size_t sf_grad_smem(int ht, int n_sym)
{
    size_t b = 0;
    b += (size_t)ht * n_sym * sizeof(int4);
    b += (size_t)ht * n_sym * 4 * sizeof(R);
    b += (size_t)ht * n_sym * 25 * sizeof(R);
    b += (size_t)ht * kMaxTileTypes * kRad * sizeof(R);
    b += (size_t)ht * 2 * sizeof(R);                       // sG
    b += (size_t)(kTileAtoms / 32) * ht * 2 * sizeof(R);  // sF
    b += (size_t)ht * sizeof(R);                           // sH2
    b += (size_t)n_sym * 12 * sizeof(int);
    b += (size_t)kMaxTileTypes * sizeof(int);
    return b + 64;
}

template <typename R, bool MP>
cudaError_t launch_sf_grad_t(const DevStructure &S, const CallBuffers &C, int hkl_chunk, int ht, cudaStream_t st)
{
    const size_t smem = sf_grad_smem<R>(ht, S.n_sym);
    cudaError_t e = cudaFuncSetAttribute(sf_grad_kernel<R, MP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(S.n_tiles, (S.n_hkl + hkl_chunk - 1) / hkl_chunk);
    sf_grad_kernel<R, MP><<<grid, kTileAtoms, smem, st>>>(S, C, hkl_chunk, ht);
    return cudaGetLastError();
}

cudaError_t launch_sf_grad(const DevStructure &S, const CallBuffers &C, bool fp64, bool mp, int hkl_chunk, int ht,
                           cudaStream_t st)
{
    if (fp64) return mp ? launch_sf_grad_t<double, true>(S, C, hkl_chunk, ht, st)
                        : launch_sf_grad_t<double, false>(S, C, hkl_chunk, ht, st);
    return mp ? launch_sf_grad_t<float, true>(S, C, hkl_chunk, ht, st)
              : launch_sf_grad_t<float, false>(S, C, hkl_chunk, ht, st);
}

size_t sf_grad_smem_bytes(bool fp64, int ht, int n_sym)
{
    return fp64 ? sf_grad_smem<double>(ht, n_sym) : sf_grad_smem<float>(ht, n_sym);
}

}  // namespace dsf
