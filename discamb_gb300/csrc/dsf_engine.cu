// Host side of the dsf_gb300 C ABI: resident structures, host preparation
// (atom tiling by type, symmetry in integer form, convention matrices,
// global-frame multipole populations) and the per-call launch sequence
//   adjoint weights -> fused SF+adjoint kernel -> F / derivative epilogues.
//
// Host restatements of the reference's set-up steps:
//   HansenCoppensStructureFactorCalculator::setModel / prepareDataForEngine_part
//     (src/Scattering/HansenCoppensStructureFactorCalculator.cpp:157-290, 897-990)
//   HansenCoppens_SF_Engine3::pre_hkl_loop_sf_calc (src/Scattering/HansenCoppens_SF_Engine3.cpp:195-256)
//   HansenCoppens_SF_Engine3::calculateGlobalCoordinatesPlm (same file :594-654): here the rotation
//     of each P_l block into the global frame is obtained by sampling the local-frame angular
//     function at fixed directions and fitting global-frame harmonics (exact for degree-l
//     harmonic polynomials; no Wigner recursion)
//   scattering_utilities::centeringSfMultipliers (src/Scattering/scattering_utilities.cpp:103-170)
//   HansenCoppensStructureFactorCalculator::convertDerivatives (same file :634-664)
#include "../../include/dsf_gb300.h"
#include "dsf_device.cuh"
#include "dsf_math.cuh"
#include "dsf_launch_v3.cuh"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

namespace dsf {
cudaError_t launch_rs_prep(const DevStructure &S, int n_hkl_pad, void *rs_f, void *rs_d, cudaStream_t st);
cudaError_t launch_tr_prep(const DevStructure &S, int n_hkl_pad, void *tr_f, void *tr_d, void *trm_f, void *trm_d,
                           bool mp, cudaStream_t st);
size_t rs_record_bytes(bool fp64);
int tsc_expand(const char *path, int n_atoms, int n_hkl, const int *hkl, int ns, const int *rot,
               std::vector<float> &tab, std::string &err);
cudaError_t launch_global_plm(int n, int K, const int *perm, const int *atom_type, const double *lcs,
                              const double *type_plm, const int *type_lmax, const double *fit, double *dmat,
                              double *pg_d, float *pg_f, cudaStream_t st);
size_t sf3_smem_bytes(bool fp64, bool mp, int ht, int n_sym, int max_types, bool table);
cudaError_t launch_form_factors(const DevStructure &S, const double *hc, const int *include, double2 *out,
                                cudaStream_t st);
cudaError_t launch_sf3(const K3Args &A, int model, bool fp64, bool mp, bool aniso);
cudaError_t launch_sf_grad(const DevStructure &S, const CallBuffers &C, bool fp64, bool mp, int hkl_chunk, int ht,
                           cudaStream_t st);
size_t sf_grad_smem_bytes(bool fp64, int ht, int n_sym);
}  // namespace dsf

using namespace dsf;

namespace {
// host record of one atom type (HC or IAM)
struct TypeHost {
    double pv = 0, kappa = 1, kappa_p = 1, zeta = 1;
    double norm[5] = {0, 0, 0, 0, 0};  // density normalisation of the deformation radial functions
    int npow[5] = {0, 0, 0, 0, 0};
    int n_def = 0;
    int lmax_used = -1;
    int core_begin = 0, core_end = 0, val_begin = 0, val_end = 0;
    int iam_n = 0;
    double iam_a[5] = {0, 0, 0, 0, 0}, iam_b[5] = {0, 0, 0, 0, 0}, iam_c = 0;
    double e_z = 0, e_f000 = 0;  // electron scattering: atomic number and f_e(0) of the type's wavefunction
};
}  // namespace

// One engine serves calculations on `stream` (or a caller's stream) and
// structure set-up (uploads, table builds) on `setup`, so a thread may create
// structures while another runs calculations on the engine's other structures.
struct dsf_engine {
    int device = 0;
    std::atomic<int> live_structures{0};
    cudaStream_t stream = nullptr;
    cudaStream_t setup = nullptr;
    std::mutex setup_mtx;  // one-time device tables
    int n_sm = 0;
    size_t max_smem = 0;
    double *d_rotfit = nullptr;  // rotation-block fit (pinv blocks + sample directions) on this device
    // batched launches alternate between the call's stream and this one (under the batch launch lock)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // tile shapes chosen by the autotuner, per shape key (tune_key): blocks per SM the reflection chunks
    // aim at, and the sub-tile length (0: the longest the shared-memory budget allows)
    std::map<std::string, std::array<int, 3> > tuned;  // blocks per SM, sub-tile cap, register-capped form
    std::mutex tune_mtx;
};

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t alloc(size_t n)
    {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T *as() const { return reinterpret_cast<T *>(p); }
};

struct Status {
    int code = DSF_OK;
    std::string msg;
};

#define DSF_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t _e = (call);                                                                    \
        if (_e != cudaSuccess) {                                                                    \
            return fail(e, _e == cudaErrorMemoryAllocation ? DSF_ERR_MEMORY : DSF_ERR_CUDA,         \
                        std::string(#call) + ": " + cudaGetErrorString(_e));                        \
        }                                                                                           \
    } while (0)

// the last error message of the calling thread (each thread sees its own calls' errors)
thread_local std::string tl_err;

int fail(dsf_engine *e, int code, const std::string &msg)
{
    (void)e;
    tl_err = msg;
    return code;
}

bool mat_inverse(const double *a, double *inv, int n)
{
    std::vector<double> m(a, a + n * n), r(n * n, 0.0);
    for (int i = 0; i < n; i++) r[i * n + i] = 1.0;
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int i = c + 1; i < n; i++)
            if (std::fabs(m[i * n + c]) > std::fabs(m[p * n + c])) p = i;
        if (std::fabs(m[p * n + c]) < 1e-300) return false;
        if (p != c)
            for (int j = 0; j < n; j++) { std::swap(m[p * n + j], m[c * n + j]); std::swap(r[p * n + j], r[c * n + j]); }
        const double d = 1.0 / m[c * n + c];
        for (int j = 0; j < n; j++) { m[c * n + j] *= d; r[c * n + j] *= d; }
        for (int i = 0; i < n; i++) {
            if (i == c) continue;
            const double f = m[i * n + c];
            if (f == 0.0) continue;
            for (int j = 0; j < n; j++) { m[i * n + j] -= f * m[c * n + j]; r[i * n + j] -= f * r[c * n + j]; }
        }
    }
    std::copy(r.begin(), r.end(), inv);
    return true;
}

// UnitCell::calculateTransformationMatrices (src/CrystalStructure/UnitCell.cpp:183-212)
void cell_matrices(const double *cell, double *M, double *Minv, double *B)
{
    const double f = DSF_PI / 180.0;
    const double ca = std::cos(cell[3] * f), cb = std::cos(cell[4] * f), cg = std::cos(cell[5] * f),
                 sg = std::sin(cell[5] * f);
    const double phi = std::sqrt(1 - ca * ca - cb * cb - cg * cg + 2 * ca * cb * cg);
    const double a = cell[0], b = cell[1], c = cell[2];
    double m[9] = {a, b * cg, c * cb, 0, b * sg, (c / sg) * (ca - cb * cg), 0, 0, c * phi / sg};
    std::copy(m, m + 9, M);
    mat_inverse(M, Minv, 3);
    // B = M^{-T}: columns are a*, b*, c*
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[3 * i + j] = Minv[3 * j + i];
}

// U (symmetric 3x3) -> Voigt param vector helpers; A6 maps U_param -> U*_param for U* = A U A^T
void adp_param_map(const double *A, double *A6)
{
    static const int I[6] = {0, 1, 2, 0, 0, 1}, J[6] = {0, 1, 2, 1, 2, 2};
    for (int p = 0; p < 6; p++)       // output param (i,j)
        for (int q = 0; q < 6; q++) { // input param (k,l), symmetric
            const int i = I[p], j = J[p], k = I[q], l = J[q];
            double v = A[3 * i + k] * A[3 * j + l];
            if (k != l) v += A[3 * i + l] * A[3 * j + k];
            A6[6 * p + q] = v;
        }
}

}  // namespace

struct dsf_structure {
    dsf_engine *eng = nullptr;
    int model = MODEL_HC;
    int n_atoms = 0, n_hkl = 0, n_sym = 0, n_types = 0, n_wfn = 0, n_tiles = 0;
    int xyz_conv = 0, adp_conv = 0;
    double M[9], Minv[9], B[9];
    double A6[36];  // beta_param (without 2 pi^2) = A6 U_param
    int centro_mode = 0;  // 0 none, 1 inversion at origin, 2 shifted
    int t_inv24[3] = {0, 0, 0};
    char centering = 'P';
    int obverse = 1;
    int n_total = 1;
    std::vector<int> sym_rot, sym_t24;
    // HC: operations ordered in cosets of coset_size (0: no such order) within
    // which they differ by a sign-diagonal Cartesian map of the reciprocal
    // vector; sym_sign: that map's signs relative to the coset's first operation
    int electron = 0;            // HC: Mott-Bethe electron scattering
    int coset_size = 0;
    int inv_pairs = 0;  // generic models: operations n/2 .. n-1 are the images of 0 .. n/2-1 under -1 at the origin
    int debug_stall = 0;  // dsf_debug_stall_next_call: the next call's kernel waits run out (timeout test)
    int tune_bps = 0, tune_ht = 0, tune_occ3 = 0;  // the autotuner's candidate for the next calls (bps 0: none)
    int pending = 0;      // a dsf_submit call of this structure not yet completed by dsf_poll
    std::vector<int> sym_sign;   // [n_sym][3] Cartesian
    std::vector<int> sym_fsign;  // [n_sym][3] fractional h' components
    // tabulated model: column of sorted atom a = a + (a >= table_split ? table_shift : 0), table_stride
    // columns per row (even), so every tile's columns start on a 16-byte boundary
    int table_stride = 0, table_split = 0, table_shift = 0;
    std::vector<int> perm;  // sorted -> original
    std::vector<int> tile_begin, tile_ntypes, tile_types;
    // host model copies
    std::vector<int> atom_type, atom_wfn, adpk;
    std::vector<double> mult_w, anom, lcs;
    std::vector<int> type_nl, type_wfn;
    std::vector<double> type_plm, type_pval, type_kappa, type_kappa_p;
    std::vector<TypeHost> trad;
    std::vector<double> tcoeff, texp;
    std::vector<int> tpow;
    std::vector<double> dmat;  // [n_atoms][165] D_l blocks (sorted order)
    // device
    DevBuf d_sym_rot, d_sym_t24, d_tile_begin, d_tile_ntypes, d_tile_types, d_atom_ltype, d_atom_adpk,
        d_active, d_xq, d_xlo, d_xd, d_adp_f, d_adp_d, d_w_f, d_w_d, d_anom_f, d_anom_d, d_pg_f, d_pg_d, d_types,
        d_types_f, d_tcoeff, d_texp, d_tpow, d_texp_f, d_tpre_f, d_hkl, d_h2, d_h2f, d_hmult, d_cinv, d_table_f, d_table_d, d_perm, d_multw, d_dmat,
        d_raw, d_dtdf, d_gw_d, d_gw_f, d_facc, d_gacc, d_out, d_plm_lmax,
        d_rs_f, d_rs_d, d_tr_f, d_tr_d, d_trm_f, d_trm_d, d_err, d_hperm, d_cont, d_tile_lmax,
        d_lcs, d_type_plm, d_type_lmax, d_atom_type0, d_step_f, d_step_d;
    std::vector<int> hperm;  // line-ordered reflection -> caller's index
    int n_hkl_pad = 0;
    // resident tables per precision (0: FP32, 1: FP64), built when a call first needs them
    bool rs_ok[2] = {false, false}, tr_ok[2] = {false, false}, trm_ok[2] = {false, false};
    int n_tiles_plain = 0;   // tiles [0, n_tiles_plain) hold atoms without anisotropic ADPs
    int max_types_plain = 1, max_types_aniso = 1;
    std::vector<uint8_t> active_host;
    bool have_hkl = false, have_atoms = false;
    int last_launches = 0;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    void *pinned = nullptr;  // host staging of dsf_calculate / dsf_calculate_atoms
    size_t pinned_bytes = 0;
    DevStructure dev{};
};

namespace {

// ------------------------------------------------------------------------
// small kernels: per-call adjoint weights, epilogues, atom conversion
// ------------------------------------------------------------------------

// g = conj(dT/dF) * centering multiplier; effective weight of the
// centrosymmetric forms: 2 Re g (inversion at origin), g + conj(g c_inv) (shifted)
// adjoint weight of reflection i (engine line order): g = conj(dT/dF) x centering
// multiplier, folded with the inversion centre (2 Re g at the origin,
// g + conj(g c_inv) away from it)
__device__ __forceinline__ void gw_one(int i, const double2 *dtdf, const double *mult, const double2 *cinv,
                                       int centro, double2 *gw_d, float2 *gw_f, const int *perm)
{
    const double m = mult[i];
    const int o = perm ? perm[i] : i;
    double gre = dtdf[o].x * m, gim = -dtdf[o].y * m;
    if (centro == 1) {
        gre = 2.0 * gre;
        gim = 0.0;
    } else if (centro == 2) {
        const double2 c = cinv[i];
        const double pre = gre * c.x - gim * c.y, pim = gre * c.y + gim * c.x;
        gre = gre + pre;
        gim = gim - pim;
    }
    gw_d[i] = make_double2(gre, gim);
    gw_f[i] = make_float2((float)gre, (float)gim);
}

__global__ void gw_kernel(int n, const double2 *dtdf, const double *mult, const double2 *cinv, int centro,
                          double2 *gw_d, float2 *gw_f, const int *perm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) gw_one(i, dtdf, mult, cinv, centro, gw_d, gw_f, perm);
}

// F of reflection i: the accumulated U, the inversion centre and the centering multiplier
__device__ __forceinline__ void f_epilogue_one(int i, const double2 *facc, const double *mult, const double2 *cinv,
                                               int centro, double *f_out, const int *perm)
{
    double2 F = facc[i];
    if (centro == 1) {
        F.x = 2.0 * F.x;
        F.y = 0.0;
    } else if (centro == 2) {
        const double2 c = cinv[i];
        const double re = F.x + (c.x * F.x + c.y * F.y);
        const double im = F.y + (c.y * F.x - c.x * F.y);
        F.x = re;
        F.y = im;
    }
    const int o = perm ? perm[i] : i;
    f_out[2 * o] = F.x * mult[i];
    f_out[2 * o + 1] = F.y * mult[i];
}

__global__ void f_epilogue_kernel(int n, const double2 *facc, const double *mult, const double2 *cinv, int centro,
                                  double *f_out, const int *perm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f_epilogue_one(i, facc, mult, cinv, centro, f_out, perm);
}

struct GradParams {
    int n_atoms;
    int xyz_conv;   // 0 frac, 1 cart
    double Minv[9];
    double A6[36];  // beta = 2 pi^2 A6 U
    int want_xyz, want_adp, want_occ, want_mp;
};

// derivatives of atom a (engine order) in the crystal's conventions, original atom order
__device__ __forceinline__ void grad_epilogue_one(int a, const GradParams &P, const double *g_acc, const int *perm,
                                                  const int *adpk, const double *w, const double *mult_w,
                                                  const double *dmat, const int *plm_lmax, double *d_xyz,
                                                  double *d_adp, double *d_occ, double *d_pval, double *d_plm,
                                                  double *d_kappa, double *d_kappa_p)
{
    const int o = perm[a];
    const double *G = g_acc + (size_t)a * kNch;
    const double wa = w[a];
    const double two_pi = 2.0 * DSF_PI, two_pi2 = 2.0 * DSF_PI * DSF_PI;
    if (P.want_xyz && d_xyz) {
        double gf[3];
        for (int j = 0; j < 3; j++) gf[j] = two_pi * wa * G[CH_XYZ + j];
        if (P.xyz_conv == 1) {
            for (int j = 0; j < 3; j++)
                d_xyz[3 * o + j] = gf[0] * P.Minv[0 * 3 + j] + gf[1] * P.Minv[1 * 3 + j] + gf[2] * P.Minv[2 * 3 + j];
        } else {
            for (int j = 0; j < 3; j++) d_xyz[3 * o + j] = gf[j];
        }
    }
    if (P.want_adp && d_adp) {
        const int k = adpk[a];
        for (int j = 0; j < 6; j++) d_adp[6 * o + j] = 0.0;
        if (k == 1) d_adp[6 * o] = two_pi2 * wa * G[CH_ADP];
        if (k == 6)
            for (int q = 0; q < 6; q++) {
                double s = 0;
                for (int p = 0; p < 6; p++) s += P.A6[6 * p + q] * G[CH_ADP + p];
                d_adp[6 * o + q] = two_pi2 * wa * s;
            }
    }
    if (P.want_occ && d_occ) d_occ[o] = mult_w[a] * G[CH_OCC];
    if (P.want_mp) {
        if (d_pval) d_pval[o] = wa * G[CH_PV];
        if (d_kappa) d_kappa[o] = wa * G[CH_KAPPA];
        if (d_kappa_p) d_kappa_p[o] = wa * G[CH_KAPPA_P];
        if (d_plm) {
            const double *D = dmat + (size_t)a * 165;
            int off = 0;
            for (int l = 0; l <= 4; l++) {
                const int n = 2 * l + 1;
                for (int i = 0; i < n; i++) {
                    double s = 0;
                    for (int j = 0; j < n; j++) s += D[off + i * n + j] * G[CH_PLM + l * l + j];
                    d_plm[25 * o + l * l + i] = l <= plm_lmax[a] ? wa * s : 0.0;
                }
                off += n * n;
            }
        }
    }
}

__global__ void grad_epilogue_kernel(GradParams P, const double *g_acc, const int *perm, const int *adpk,
                                     const double *w, const double *mult_w, const double *dmat,
                                     const int *plm_lmax, double *d_xyz,
                                     double *d_adp, double *d_occ, double *d_pval, double *d_plm, double *d_kappa,
                                     double *d_kappa_p)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < P.n_atoms)
        grad_epilogue_one(a, P, g_acc, perm, adpk, w, mult_w, dmat, plm_lmax, d_xyz, d_adp, d_occ, d_pval, d_plm,
                          d_kappa, d_kappa_p);
}

// a single structure's call in two small launches around the structure-factor kernels: before them the adjoint
// weights and the zeroed F and derivative accumulators (in place of a weight kernel and two memsets), after them
// F and the derivatives in the caller's conventions and order (in place of two epilogue kernels)
__global__ void call_pre_kernel(int n_hkl, int n_g, const double2 *dtdf, const double *mult, const double2 *cinv,
                                int centro, double2 *gw_d, float2 *gw_f, const int *perm, double2 *facc, double *gacc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_hkl) {
        gw_one(i, dtdf, mult, cinv, centro, gw_d, gw_f, perm);
        facc[i] = make_double2(0.0, 0.0);
    }
    if (i < n_g) gacc[i] = 0.0;
}

__global__ void call_post_kernel(int n_hkl, const double2 *facc, const double *mult, const double2 *cinv, int centro,
                                 double *f_out, const int *hperm, int grad, GradParams P, const double *g_acc,
                                 const int *perm, const int *adpk, const double *w, const double *mult_w,
                                 const double *dmat, const int *plm_lmax, double *d_xyz, double *d_adp,
                                 double *d_occ, double *d_pval, double *d_plm, double *d_kappa, double *d_kappa_p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_hkl) f_epilogue_one(i, facc, mult, cinv, centro, f_out, hperm);
    if (grad && i < P.n_atoms)
        grad_epilogue_one(i, P, g_acc, perm, adpk, w, mult_w, dmat, plm_lmax, d_xyz, d_adp, d_occ, d_pval, d_plm,
                          d_kappa, d_kappa_p);
}

// multipole-parameter derivatives summed over the atoms of each type (atoms of
// one type share P_val, P_lm in their local frames, kappa, kappa'); inputs and
// outputs in the caller's (original) atom order
__global__ void type_reduce_kernel(int n_atoms, int n_types, const int *atom_type, const double *pv, const double *plm,
                                   const double *ka, const double *kp, double *tpv, double *tplm, double *tka,
                                   double *tkp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_atoms * 28) return;
    const int a = i / 28, q = i - a * 28, t = atom_type[a];
    if (t < 0 || t >= n_types) return;
    if (q < 25) {
        if (plm && tplm) atomicAdd(&tplm[25 * (size_t)t + q], plm[25 * (size_t)a + q]);
    } else if (q == 25) {
        if (pv && tpv) atomicAdd(&tpv[t], pv[a]);
    } else if (q == 26) {
        if (ka && tka) atomicAdd(&tka[t], ka[a]);
    } else {
        if (kp && tkp) atomicAdd(&tkp[t], kp[a]);
    }
}

// the per-structure work of a batched submission before and after the SF
// kernels, for up to kPrePostItems structures per launch (kernel-parameter
// space): block row blockIdx.y is one structure, grid-stride over its
// reflections and atoms
constexpr int kPrePostItems = 40;
struct PrePostItem {
    int n_hkl, n_atoms, centro;
    const double2 *dtdf;
    const double *mult;
    const double2 *cinv;
    const int *hperm;
    double2 *gw_d;
    float2 *gw_f;
    double2 *facc;
    double *gacc;
    double *f_out;
    GradParams P;
    int want_grad;
    const int *perm, *adpk, *plm_lmax;
    const double *w, *mult_w, *dmat;
    dsf_outputs out;
};
struct PrePostBatch {
    int n;
    PrePostItem item[kPrePostItems];
};
static_assert(sizeof(PrePostBatch) <= 32000, "kernel parameters hold at most 32764 bytes");
static_assert(sizeof(dsf::SfBatch) <= 32000, "kernel parameters hold at most 32764 bytes");

__global__ void batch_pre_kernel(const __grid_constant__ PrePostBatch B)
{
    const PrePostItem &it = B.item[blockIdx.y];
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < it.n_hkl; i += stride) {
        gw_one(i, it.dtdf, it.mult, it.cinv, it.centro, it.gw_d, it.gw_f, it.hperm);
        it.facc[i] = make_double2(0.0, 0.0);
    }
    const int ng = it.n_atoms * kNch;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ng; i += stride) it.gacc[i] = 0.0;
}

__global__ void batch_post_kernel(const __grid_constant__ PrePostBatch B)
{
    const PrePostItem &it = B.item[blockIdx.y];
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < it.n_hkl; i += stride)
        f_epilogue_one(i, it.facc, it.mult, it.cinv, it.centro, it.f_out, it.hperm);
    if (!it.want_grad) return;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < it.n_atoms; a += stride)
        grad_epilogue_one(a, it.P, it.gacc, it.perm, it.adpk, it.w, it.mult_w, it.dmat, it.plm_lmax, it.out.d_xyz,
                          it.out.d_adp, it.out.d_occ, it.out.d_pval, it.out.d_plm, it.out.d_kappa,
                          it.out.d_kappa_prime);
}

struct AtomParams {
    int n_atoms;
    int xyz_conv;
    double Minv[9];
    double A6[36];
};

// raw atoms (original order: xyz[3], adp[6], occ) -> kernel representation (sorted order)
__global__ void atom_convert_kernel(AtomParams P, const double *raw, const int *perm, const int *adpk,
                                    const double *mult_w, uint32_t *xq, float *xlo, double *xd, float *adp_f,
                                    double *adp_d, float *w_f, double *w_d, int n_sym, const int *sym_rot,
                                    const int *sym_t24, float2 *step_f, double2 *step_d)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= P.n_atoms) return;
    const int o = perm[a];
    const double *r = raw + (size_t)o * 10;
    double x[3] = {r[0], r[1], r[2]};
    if (P.xyz_conv == 1) {
        double f[3];
        for (int i = 0; i < 3; i++) f[i] = P.Minv[3 * i] * x[0] + P.Minv[3 * i + 1] * x[1] + P.Minv[3 * i + 2] * x[2];
        for (int i = 0; i < 3; i++) x[i] = f[i];
    }
    for (int i = 0; i < 3; i++) {
        xd[3 * a + i] = x[i];
        const double xr = x[i] - floor(x[i]);
        const double q = rint(xr * 4294967296.0);
        xlo[3 * a + i] = (float)(xr - q * (1.0 / 4294967296.0));
        xq[3 * a + i] = (uint32_t)(unsigned long long)q;  // 2^32 wraps to 0
    }
    // line steps of the reflection-line recurrence: h -> h + e_l changes h'.x + h.t by row 3 of R times x plus t_z
    for (int op = 0; op < n_sym; op++) {
        const int *Rm = sym_rot + 9 * op;
        double ph = Rm[6] * x[0] + Rm[7] * x[1] + Rm[8] * x[2] + sym_t24[3 * op + 2] / 24.0;
        ph -= rint(ph);
        double sn, cs;
        sincospi(2.0 * ph, &sn, &cs);
        step_d[(size_t)a * n_sym + op] = make_double2(cs, sn);
        step_f[(size_t)a * n_sym + op] = make_float2((float)cs, (float)sn);
    }
    const double two_pi2 = 2.0 * DSF_PI * DSF_PI;
    const int k = adpk[a];
    for (int i = 0; i < 6; i++) {
        adp_d[6 * a + i] = 0.0;
        adp_f[6 * a + i] = 0.0f;
    }
    // FP32 copies carry log2(e) so the kernel can use exp2
    const double log2e = 1.4426950408889634;
    if (k == 1) {
        adp_d[6 * a] = two_pi2 * r[3];
        adp_f[6 * a] = (float)(two_pi2 * r[3] * log2e);
    } else if (k == 6) {
        for (int p = 0; p < 6; p++) {
            double s = 0;
            for (int q = 0; q < 6; q++) s += P.A6[6 * p + q] * r[3 + q];
            adp_d[6 * a + p] = two_pi2 * s;
            adp_f[6 * a + p] = (float)(two_pi2 * s * log2e);
        }
    }
    const double wt = r[9] * mult_w[a];
    w_d[a] = wt;
    w_f[a] = (float)wt;
}

// ------------------------------------------------------------------------
// host helpers
// ------------------------------------------------------------------------

// Orders the operations of an HC structure in cosets within which they differ
// by a sign-diagonal Cartesian map: Q_t Q_u^T = diag(+-1, +-1, +-1) with
// Q = B R^T B^{-1} (B^{-1} = M^T) the Cartesian action of h -> R^T h.  The
// harmonics of the operations of one coset are then signed copies of each
// other (sf_grad_kernel3's class-sum form).  Leaves the order alone unless all
// cosets have one size >= 2.
bool fractional_signs(dsf_structure *s, int cs);

// Cosets of four whose relative sign maps form a known group (222 or 2/m with b unique): each coset reordered
// to [e, a, b, ab] of that group's generators (kPatD2, kPatC2hB), the same pattern for every coset, so the
// Walsh-Hadamard coset kernels apply.  Only the order within a coset changes (the first operation stays, so
// the relative signs stay); cosets that fit no pattern keep their order.
void order_cosets_as_sign_group(dsf_structure *s)
{
    const int n = s->n_sym;
    auto mask = [&](int op) {
        int m = 0;
        for (int i = 0; i < 3; i++)
            if (s->sym_sign[3 * op + i] < 0) m |= 1 << i;
        return m;
    };
    for (const int pat : {kPatD2, kPatC2hB}) {
        const int want[4] = {0, pat & 7, (pat >> 3) & 7, (pat & 7) ^ ((pat >> 3) & 7)};
        std::vector<int> perm(n);
        bool fits = true;
        for (int c0 = 0; c0 < n && fits; c0 += 4)
            for (int j = 0; j < 4 && fits; j++) {
                int found = -1;
                for (int t = 0; t < 4; t++)
                    if (mask(c0 + t) == want[j]) found = c0 + t;
                if (found < 0) fits = false;
                else perm[c0 + j] = found;
            }
        if (!fits) continue;
        std::vector<int> rot(9 * (size_t)n), t24(3 * (size_t)n), sign(3 * (size_t)n);
        for (int k = 0; k < n; k++) {
            std::copy(&s->sym_rot[9 * perm[k]], &s->sym_rot[9 * perm[k]] + 9, &rot[9 * k]);
            std::copy(&s->sym_t24[3 * perm[k]], &s->sym_t24[3 * perm[k]] + 3, &t24[3 * k]);
            std::copy(&s->sym_sign[3 * perm[k]], &s->sym_sign[3 * perm[k]] + 3, &sign[3 * k]);
        }
        s->sym_rot.swap(rot);
        s->sym_t24.swap(t24);
        s->sym_sign.swap(sign);
        return;
    }
}

// the sign-group pattern of a launch's sign table: cosets of four whose every operation gives every parity
// class (fractional, and for the HC model harmonic) the sign of the pattern's character at its position, else 0
int wht_pattern_of(const SignTable &G, int n_sym, int coset, bool harmonics)
{
    if (coset != 4 || n_sym % 4 != 0) return 0;
    for (const int pat : {kPatD2, kPatC2hB}) {
        bool ok = true;
        for (int op = 0; op < n_sym && ok; op++) {
            const int j = op & 3;
            for (int c = 0; c < 8 && ok; c++) {
                const int k = wht_char(pat, c);
                const float want = (((k & 1) & (j & 1)) ^ (((k >> 1) & 1) & (j >> 1))) ? -1.0f : 1.0f;
                ok = (!harmonics || G.f[op][c] == want) && G.xf[op][c] == want;
            }
        }
        if (ok) return pat;
    }
    return 0;
}

void order_sign_cosets(dsf_structure *s)
{
    const int n = s->n_sym;
    std::vector<double> Q(9 * (size_t)n);
    for (int op = 0; op < n; op++) {
        const int *R = &s->sym_rot[9 * op];
        double BRt[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double v = 0;
                for (int k = 0; k < 3; k++) v += s->B[3 * i + k] * R[3 * j + k];
                BRt[3 * i + j] = v;
            }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double v = 0;
                for (int k = 0; k < 3; k++) v += BRt[3 * i + k] * s->M[3 * j + k];
                Q[9 * op + 3 * i + j] = v;
            }
    }
    // signs of Q_t Q_u^T when it is sign-diagonal
    auto rel = [&](int t, int u, int *sg) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double v = 0;
                for (int k = 0; k < 3; k++) v += Q[9 * t + 3 * i + k] * Q[9 * u + 3 * j + k];
                const double want = (i == j) ? std::copysign(1.0, v) : 0.0;
                if (std::fabs(v - want) > 1e-9) return false;
                if (i == j) sg[i] = v < 0 ? -1 : 1;
            }
        return true;
    };
    std::vector<int> order, sign(3 * (size_t)n, 1), used(n, 0);
    int cs = -1;
    for (int u = 0; u < n; u++) {
        if (used[u]) continue;
        int size = 0;
        for (int t = u; t < n; t++) {
            int sg[3];
            if (used[t] || !rel(t, u, sg)) continue;
            used[t] = 1;
            for (int i = 0; i < 3; i++) sign[3 * order.size() + i] = sg[i];
            order.push_back(t);
            size++;
        }
        if (cs < 0) cs = size;
        if (size != cs) cs = 0;
    }
    s->coset_size = 0;
    s->sym_sign.assign(3 * (size_t)n, 1);
    if (cs < 2) return;
    std::vector<int> rot(9 * (size_t)n), t24(3 * (size_t)n);
    for (int k = 0; k < n; k++) {
        std::copy(&s->sym_rot[9 * order[k]], &s->sym_rot[9 * order[k]] + 9, &rot[9 * k]);
        std::copy(&s->sym_t24[3 * order[k]], &s->sym_t24[3 * order[k]] + 3, &t24[3 * k]);
    }
    s->sym_rot.swap(rot);
    s->sym_t24.swap(t24);
    s->sym_sign = sign;
    s->coset_size = cs;
    if (cs == 4) order_cosets_as_sign_group(s);
    // the same cosets must be sign-diagonal on the fractional h' as well (standard settings are)
    if (!fractional_signs(s, cs)) s->coset_size = 0;
}

// fractional signs of every operation relative to the first of its coset (cosets of
// cs consecutive operations): R_s^T = D R_r^T with D = diag(+-1, +-1, +-1), i.e. column
// i of R_s is +-column i of R_r; false if an operation is not of that form
bool fractional_signs(dsf_structure *s, int cs)
{
    const int n = s->n_sym;
    s->sym_fsign.assign(3 * (size_t)n, 1);
    if (cs < 1) return false;
    for (int op = 0; op < n; op++) {
        const int *R = &s->sym_rot[9 * op], *Rr = &s->sym_rot[9 * (op - op % cs)];
        for (int i = 0; i < 3; i++) {
            int d = 0;
            for (int j = 0; j < 3; j++) {
                const int a = R[3 * j + i], b = Rr[3 * j + i];
                if (a == 0 && b == 0) continue;
                const int sg = (a == b) ? 1 : (a == -b ? -1 : 0);
                if (sg == 0 || (d != 0 && d != sg)) return false;
                d = sg;
            }
            if (d == 0) return false;
            s->sym_fsign[3 * op + i] = d;
        }
    }
    return true;
}

int sym_from_desc(dsf_engine *e, dsf_structure *s, const dsf_symmetry *sym)
{
    if (!sym || sym->n_symops < 1 || sym->n_symops > kMaxSym)
        return fail(e, DSF_ERR_ARGUMENT, "n_symops must be in 1..48");
    for (int i = 0; i < 3; i++)
        if (!(sym->cell[i] > 0)) return fail(e, DSF_ERR_ARGUMENT, "cell lengths must be positive");
    cell_matrices(sym->cell, s->M, s->Minv, s->B);
    s->n_sym = sym->n_symops;
    s->sym_rot.assign(sym->symop_rotation, sym->symop_rotation + 9 * s->n_sym);
    s->sym_t24.resize(3 * s->n_sym);
    for (int i = 0; i < 3 * s->n_sym; i++) {
        const double t = sym->symop_translation[i] * 24.0;
        const double r = std::rint(t);
        if (std::fabs(t - r) > 1e-6) return fail(e, DSF_ERR_ARGUMENT, "symmetry translations must be multiples of 1/24");
        int v = (int)r % 24;
        if (v < 0) v += 24;
        s->sym_t24[i] = v;
    }
    if (s->model == MODEL_HC) {
        order_sign_cosets(s);
    } else {
        // generic engine: the operations keep the caller's order (the tabulated model's table follows it);
        // one coset when every operation is a sign-diagonal image of the first
        s->coset_size = (s->n_sym >= 2 && fractional_signs(s, s->n_sym)) ? s->n_sym : 0;
        s->sym_sign.assign(3 * (size_t)s->n_sym, 1);
        // the caller's order as n/2 operations and then their images under an inversion at the origin
        // (x -> -R x - t), as the standard operation lists of centrosymmetric groups come
        const int n = s->n_sym, h = n / 2;
        bool pairs = n >= 2 && n % 2 == 0;
        for (int k = 0; pairs && k < h; k++) {
            for (int j = 0; j < 9; j++) pairs = pairs && s->sym_rot[9 * (k + h) + j] == -s->sym_rot[9 * k + j];
            for (int j = 0; j < 3; j++) pairs = pairs && (s->sym_t24[3 * (k + h) + j] + s->sym_t24[3 * k + j]) % 24 == 0;
        }
        s->inv_pairs = pairs ? 1 : 0;
    }
    s->centro_mode = 0;
    if (sym->centrosymmetric) {
        bool origin = true;
        for (int i = 0; i < 3; i++) {
            const double t = sym->inversion_translation[i] * 24.0;
            const double r = std::rint(t);
            if (std::fabs(t - r) > 1e-6) return fail(e, DSF_ERR_ARGUMENT, "inversion translation must be a multiple of 1/24");
            int v = (int)r % 24;
            if (v < 0) v += 24;
            s->t_inv24[i] = v;
            if (v != 0) origin = false;
        }
        s->centro_mode = origin ? 1 : 2;
    }
    s->centering = sym->centering ? sym->centering : 'P';
    s->obverse = sym->obverse;
    s->n_total = sym->n_symops_total > 0 ? sym->n_symops_total : s->n_sym;
    const char c = (char)toupper(s->centering);
    if (!strchr("PABCIFR", c)) return fail(e, DSF_ERR_ARGUMENT, "unsupported lattice centering");
    s->centering = c;
    return DSF_OK;
}

double centering_multiplier(char c, int obverse, int h, int k, int l)
{
    switch (c) {
    case 'P': return 1.0;
    // obverse: -h + k + l = 3n; the reverse setting tests (h - k + l) mod 2, as the reference does
    // (scattering_utilities.cpp:117-134), so that results match it on the same input
    case 'R':
        if (obverse) return (std::abs(-h + k + l) % 3 == 0) ? 3.0 : 0.0;
        return (std::abs(h - k + l) % 2 == 0) ? 3.0 : 0.0;
    case 'F': {
        const int a = std::abs(h % 2), b = std::abs(k % 2), d = std::abs(l % 2);
        return (a == b && a == d) ? 4.0 : 0.0;
    }
    case 'I': return ((h + k + l) % 2 == 0) ? 2.0 : 0.0;
    case 'A': return ((k + l) % 2 == 0) ? 2.0 : 0.0;
    case 'B': return ((h + l) % 2 == 0) ? 2.0 : 0.0;
    case 'C': return ((h + k) % 2 == 0) ? 2.0 : 0.0;
    }
    return 1.0;
}

// fixed sampling directions and the least-squares fit matrices for the
// global-frame rotation of P_lm (per l: pinv (2l+1) x K)
struct RotationFit {
    static constexpr int K = 40;
    double u[K][3];
    std::vector<double> pinv[5];
    RotationFit()
    {
        const double ga = DSF_PI * (3.0 - std::sqrt(5.0));
        for (int k = 0; k < K; k++) {
            const double z = 1.0 - (2.0 * k + 1.0) / K;
            const double r = std::sqrt(1.0 - z * z);
            u[k][0] = r * std::cos(ga * k);
            u[k][1] = r * std::sin(ga * k);
            u[k][2] = z;
        }
        for (int l = 0; l <= 4; l++) {
            const int n = 2 * l + 1;
            std::vector<double> A(K * n), AtA(n * n, 0.0), inv(n * n);
            for (int k = 0; k < K; k++) {
                double v[25];
                harmonic_polys<double>(u[k][0], u[k][1], u[k][2], v);
                for (int m = 0; m < n; m++) A[k * n + m] = v[l * l + m] * kDensityNormHost[l * l + m];
            }
            for (int i = 0; i < n; i++)
                for (int j = 0; j < n; j++)
                    for (int k = 0; k < K; k++) AtA[i * n + j] += A[k * n + i] * A[k * n + j];
            mat_inverse(AtA.data(), inv.data(), n);
            pinv[l].assign(n * K, 0.0);
            for (int i = 0; i < n; i++)
                for (int k = 0; k < K; k++) {
                    double s = 0;
                    for (int j = 0; j < n; j++) s += inv[i * n + j] * A[k * n + j];
                    pinv[l][i * K + k] = s;
                }
        }
    }
};

const RotationFit &rotation_fit()
{
    static RotationFit f;
    return f;
}

// D_l with d_l(L^T u) = D_l d_l(u); stored row-major per l (165 doubles)
template <typename T>
int upload(dsf_engine *e, DevBuf &b, const T *src, size_t n)
{
    DSF_CUDA(b.alloc(sizeof(T) * std::max<size_t>(n, 1)));
    if (n) DSF_CUDA(cudaMemcpyAsync(b.p, src, sizeof(T) * n, cudaMemcpyHostToDevice, e->setup));
    return DSF_OK;
}

int compute_global_plm(dsf_structure *s)
{
    dsf_engine *e = s->eng;
    const int n = s->n_atoms;
    int rc;
    const int K = RotationFit::K;
    std::lock_guard<std::mutex> lock(e->setup_mtx);
    if (!e->d_rotfit) {
        const RotationFit &F = rotation_fit();
        std::vector<double> fit(25 * (size_t)K + 3 * (size_t)K);
        for (int l = 0; l <= 4; l++) std::copy(F.pinv[l].begin(), F.pinv[l].end(), fit.begin() + (size_t)K * l * l);
        for (int k = 0; k < K; k++)
            for (int j = 0; j < 3; j++) fit[25 * (size_t)K + 3 * k + j] = F.u[k][j];
        DSF_CUDA(cudaMalloc(&e->d_rotfit, sizeof(double) * fit.size()));
        DSF_CUDA(cudaMemcpy(e->d_rotfit, fit.data(), sizeof(double) * fit.size(), cudaMemcpyHostToDevice));
    }
    std::vector<int> tlmax(std::max(1, s->n_types));
    for (int t = 0; t < s->n_types; t++) tlmax[t] = s->trad[t].lmax_used;
    std::vector<int> atype(s->atom_type.begin(), s->atom_type.end());
    if ((rc = upload(e, s->d_lcs, s->lcs.data(), s->lcs.size()))) return rc;
    if ((rc = upload(e, s->d_type_plm, s->type_plm.data(), s->type_plm.size()))) return rc;
    if ((rc = upload(e, s->d_type_lmax, tlmax.data(), tlmax.size()))) return rc;
    if ((rc = upload(e, s->d_atom_type0, atype.data(), atype.size()))) return rc;
    DSF_CUDA(s->d_dmat.alloc(sizeof(double) * 165 * (size_t)n));
    DSF_CUDA(s->d_pg_d.alloc(sizeof(double) * 25 * (size_t)n));
    DSF_CUDA(s->d_pg_f.alloc(sizeof(float) * 25 * (size_t)n));
    DSF_CUDA(launch_global_plm(n, K, s->d_perm.as<int>(), s->d_atom_type0.as<int>(), s->d_lcs.as<double>(),
                               s->d_type_plm.as<double>(), s->d_type_lmax.as<int>(), e->d_rotfit,
                               s->d_dmat.as<double>(), s->d_pg_d.as<double>(), s->d_pg_f.as<float>(), e->setup));
    std::vector<int> lmx(n);
    for (int a = 0; a < n; a++) {
        const int t = s->atom_type[s->perm[a]];
        lmx[a] = std::min(std::min(s->type_nl[t] - 1, s->trad[t].n_def - 1), 4);
    }
    // per tile: highest l of the angular sums (tiles of hydrogen-like types skip l = 3, 4)
    std::vector<int> tl(s->n_tiles, -1);
    for (int t = 0; t < s->n_tiles; t++)
        for (int a = s->tile_begin[t]; a < s->tile_begin[t + 1]; a++)
            tl[t] = std::max(tl[t], s->trad[s->atom_type[s->perm[a]]].lmax_used);
    if ((rc = upload(e, s->d_tile_lmax, tl.data(), tl.size()))) return rc;
    if ((rc = upload(e, s->d_plm_lmax, lmx.data(), lmx.size()))) return rc;
    return DSF_OK;
}

// pre_hkl_loop_sf_calc: l used in the sum and the deformation normalisation
int build_type_radial(dsf_structure *s, const dsf_hc_model *m)
{
    dsf_engine *e = s->eng;
    const int nT = s->n_types;
    s->trad.assign(nT, TypeHost{});
    for (int t = 0; t < nT; t++) {
        TypeHost &r = s->trad[t];
        r.pv = s->type_pval[t];
        r.kappa = s->type_kappa[t];
        r.kappa_p = s->type_kappa_p[t];
        const int w = s->type_wfn[t];
        if (m) {
            r.zeta = m->def_val_exp[w];
            r.n_def = std::min(5, m->def_val_npow[w]);
            for (int l = 0; l < 5; l++) {
                r.npow[l] = l < r.n_def ? m->def_val_pow[5 * w + l] : 0;
                if (l < r.n_def) {
                    if (r.npow[l] < l || r.npow[l] > 8)
                        return fail(e, DSF_ERR_ARGUMENT, "deformation-valence r power n_l must satisfy l <= n_l <= 8");
                    double nrm = std::pow(r.zeta, r.npow[l] + 3);
                    for (int q = 2; q <= r.npow[l] + 2; q++) nrm /= q;
                    r.norm[l] = nrm;
                }
            }
            r.core_begin = m->core_offset[w];
            r.core_end = m->core_offset[w + 1];
            int lp = -1;
            for (int l = 0; l < s->type_nl[t] && l <= 4; l++)
                for (int q = 0; q < 2 * l + 1; q++)
                    if (s->type_plm[25 * (size_t)t + l * l + q] != 0.0) lp = l;
            r.lmax_used = std::min(lp, std::min(4, r.n_def - 1));
        } else {
            r.lmax_used = -1;
        }
    }
    return DSF_OK;
}

int build_tiles(dsf_structure *s, bool by_type)
{
    const int n = s->n_atoms;
    s->perm.resize(n);
    std::iota(s->perm.begin(), s->perm.end(), 0);
    // atoms without anisotropic ADPs first, then by type: a tile holds one ADP kind
    std::stable_sort(s->perm.begin(), s->perm.end(), [&](int x, int y) {
        const int kx = s->adpk[x] == 6, ky = s->adpk[y] == 6;
        if (kx != ky) return kx < ky;
        if (by_type && s->atom_type[x] != s->atom_type[y]) return s->atom_type[x] < s->atom_type[y];
        return false;
    });
    s->tile_begin.clear();
    s->tile_ntypes.clear();
    s->tile_types.clear();
    std::vector<int> ltype(n);
    int a = 0;
    while (a < n) {
        s->tile_begin.push_back(a);
        std::vector<int> types;
        int cnt = 0;
        const int kind = s->adpk[s->perm[a]] == 6;
        while (a < n && cnt < kTileAtoms && (s->adpk[s->perm[a]] == 6) == kind) {
            const int t = by_type ? s->atom_type[s->perm[a]] : 0;
            auto it = std::find(types.begin(), types.end(), t);
            int li;
            if (it == types.end()) {
                if ((int)types.size() == kMaxTileTypes) break;
                types.push_back(t);
                li = (int)types.size() - 1;
            } else {
                li = (int)(it - types.begin());
            }
            ltype[a] = li;
            a++;
            cnt++;
        }
        s->tile_ntypes.push_back((int)types.size());
        for (int i = 0; i < kMaxTileTypes; i++) s->tile_types.push_back(i < (int)types.size() ? types[i] : 0);
    }
    s->tile_begin.push_back(n);
    s->n_tiles = (int)s->tile_ntypes.size();
    s->n_tiles_plain = 0;
    s->max_types_plain = s->max_types_aniso = 1;
    for (int t = 0; t < s->n_tiles; t++) {
        const bool aniso = s->adpk[s->perm[s->tile_begin[t]]] == 6;
        if (!aniso) {
            s->n_tiles_plain = t + 1;
            s->max_types_plain = std::max(s->max_types_plain, s->tile_ntypes[t]);
        } else {
            s->max_types_aniso = std::max(s->max_types_aniso, s->tile_ntypes[t]);
        }
    }
    dsf_engine *e = s->eng;
    int rc;
    std::vector<int> adpk_sorted(n);
    std::vector<double> mw_sorted(n);
    std::vector<double> an_d(2 * (size_t)n);
    std::vector<float> an_f(2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        const int o = s->perm[i];
        adpk_sorted[i] = s->adpk[o];
        mw_sorted[i] = s->mult_w[o];
        an_d[2 * i] = s->anom[2 * o];
        an_d[2 * i + 1] = s->anom[2 * o + 1];
        an_f[2 * i] = (float)an_d[2 * i];
        an_f[2 * i + 1] = (float)an_d[2 * i + 1];
    }
    if ((rc = upload(e, s->d_tile_begin, s->tile_begin.data(), s->tile_begin.size()))) return rc;
    if ((rc = upload(e, s->d_tile_ntypes, s->tile_ntypes.data(), s->tile_ntypes.size()))) return rc;
    if ((rc = upload(e, s->d_tile_types, s->tile_types.data(), s->tile_types.size()))) return rc;
    if ((rc = upload(e, s->d_atom_ltype, ltype.data(), ltype.size()))) return rc;
    if ((rc = upload(e, s->d_atom_adpk, adpk_sorted.data(), adpk_sorted.size()))) return rc;
    if ((rc = upload(e, s->d_perm, s->perm.data(), s->perm.size()))) return rc;
    if ((rc = upload(e, s->d_multw, mw_sorted.data(), mw_sorted.size()))) return rc;
    if ((rc = upload(e, s->d_anom_d, an_d.data(), an_d.size()))) return rc;
    if ((rc = upload(e, s->d_anom_f, an_f.data(), an_f.size()))) return rc;
    s->active_host.assign(n, 1);
    if ((rc = upload(e, s->d_active, s->active_host.data(), s->active_host.size()))) return rc;
    // per-atom buffers
    DSF_CUDA(s->d_xq.alloc(12 * (size_t)n));
    DSF_CUDA(s->d_xlo.alloc(12 * (size_t)n));
    DSF_CUDA(s->d_xd.alloc(24 * (size_t)n));
    DSF_CUDA(s->d_adp_f.alloc(24 * (size_t)n));
    DSF_CUDA(s->d_adp_d.alloc(48 * (size_t)n));
    DSF_CUDA(s->d_w_f.alloc(4 * (size_t)n));
    DSF_CUDA(s->d_w_d.alloc(8 * (size_t)n));
    DSF_CUDA(s->d_raw.alloc(80 * (size_t)n));
    DSF_CUDA(s->d_gacc.alloc(sizeof(double) * kNch * (size_t)n));
    return DSF_OK;
}

void refresh_dev(dsf_structure *s);

// resident per-(type, reflection) radial tables; mp = the multipole-adjoint table
// builds the tables a call of one precision needs: reflection-operation records,
// radial terms, and (with the multipole adjoint) their kappa derivatives
int ensure_tables(dsf_structure *s, bool fp64, bool mp)
{
    dsf_engine *e = s->eng;
    if (!s->have_hkl || s->n_hkl == 0) return DSF_OK;  // an empty reflection set has no tables
    const int p = fp64 ? 1 : 0;
    const size_t esz = fp64 ? sizeof(double) : sizeof(float);
    const size_t row = 8 * (size_t)s->n_hkl_pad * std::max(1, s->n_types);
    const bool built = !s->rs_ok[p] || !s->tr_ok[p] || (mp && !s->trm_ok[p]);
    if (!s->rs_ok[p]) {
        DevBuf &rs = fp64 ? s->d_rs_d : s->d_rs_f;
        DSF_CUDA(rs.alloc(rs_record_bytes(fp64) * (size_t)s->n_hkl_pad * s->n_sym));
        DSF_CUDA(launch_rs_prep(s->dev, s->n_hkl_pad, fp64 ? nullptr : rs.p, fp64 ? rs.p : nullptr, e->setup));
        s->rs_ok[p] = true;
    }
    if (!s->tr_ok[p]) {
        DevBuf &tr = fp64 ? s->d_tr_d : s->d_tr_f;
        DSF_CUDA(tr.alloc(esz * row));
        DSF_CUDA(launch_tr_prep(s->dev, s->n_hkl_pad, fp64 ? nullptr : tr.p, fp64 ? tr.p : nullptr, nullptr,
                                nullptr, false, e->setup));
        s->tr_ok[p] = true;
    }
    if (mp && !s->trm_ok[p]) {
        DevBuf &trm = fp64 ? s->d_trm_d : s->d_trm_f;
        DSF_CUDA(trm.alloc(esz * row));
        DSF_CUDA(launch_tr_prep(s->dev, s->n_hkl_pad, nullptr, nullptr, fp64 ? nullptr : trm.p,
                                fp64 ? trm.p : nullptr, true, e->setup));
        s->trm_ok[p] = true;
    }
    // the calls that read the tables may run on another stream
    if (built) DSF_CUDA(cudaStreamSynchronize(e->setup));
    return DSF_OK;
}

// per-type constants of the kernels in both precisions (prefactors folded)
template <typename R>
TypeRadialT<R> type_constants(const TypeHost &h)
{
    TypeRadialT<R> t{};
    t.pv = R(h.pv);
    t.inv_kappa = R(1.0 / h.kappa);
    t.inv_kappa_p = R(1.0 / h.kappa_p);
    t.zeta = R(h.zeta);
    t.n_def = h.n_def;
    for (int l = 0; l < 5; l++) {
        t.def_m[l] = 0;
        t.def_pre[l] = R(0);
        if (l < h.n_def) {
            const int m = h.npow[l] + 1 - l;
            const double sgn = (l == 2 || l == 3) ? -1.0 : 1.0;
            t.def_m[l] = m;
            t.def_pre[l] = R(sgn * 4.0 * DSF_PI * h.norm[l] * g_prefactor(l, m));
        }
    }
    t.e_z = R(h.e_z);
    t.e_f000 = R(h.e_f000);
    t.core_begin = h.core_begin;
    t.core_end = h.core_end;
    t.val_begin = h.val_begin;
    t.val_end = h.val_end;
    t.iam_n = h.iam_n;
    for (int q = 0; q < 5; q++) {
        t.iam_a[q] = R(h.iam_a[q]);
        t.iam_b[q] = R(h.iam_b[q]);
    }
    t.iam_c = R(h.iam_c);
    return t;
}

int upload_types(dsf_structure *s)
{
    std::vector<TypeRadialT<double> > td;
    std::vector<TypeRadialT<float> > tf;
    for (const TypeHost &h : s->trad) {
        td.push_back(type_constants<double>(h));
        tf.push_back(type_constants<float>(h));
    }
    int rc;
    if ((rc = upload(s->eng, s->d_types, td.data(), td.size()))) return rc;
    if ((rc = upload(s->eng, s->d_types_f, tf.data(), tf.size()))) return rc;
    refresh_dev(s);
    return DSF_OK;
}

void refresh_dev(dsf_structure *s)
{
    DevStructure &d = s->dev;
    d.model = s->model;
    d.electron = s->electron;
    d.n_atoms = s->n_atoms;
    d.n_hkl = s->n_hkl;
    d.n_sym = s->n_sym;
    d.n_tiles = s->n_tiles;
    d.n_types = s->n_types;
    std::copy(s->B, s->B + 9, d.B);
    d.sym_rot = s->d_sym_rot.as<int>();
    d.sym_t24 = s->d_sym_t24.as<int>();
    d.tile_begin = s->d_tile_begin.as<int>();
    d.tile_ntypes = s->d_tile_ntypes.as<int>();
    d.tile_types = s->d_tile_types.as<int>();
    d.atom_ltype = s->d_atom_ltype.as<int>();
    d.atom_adpk = s->d_atom_adpk.as<int>();
    d.atom_active = s->d_active.as<uint8_t>();
    d.atom_xq = s->d_xq.as<uint32_t>();
    d.atom_xlo = s->d_xlo.as<float>();
    d.atom_xd = s->d_xd.as<double>();
    d.atom_adp_f = s->d_adp_f.as<float>();
    d.atom_adp_d = s->d_adp_d.as<double>();
    d.atom_w_f = s->d_w_f.as<float>();
    d.atom_w_d = s->d_w_d.as<double>();
    d.atom_anom_f = s->d_anom_f.as<float2>();
    d.atom_anom_d = s->d_anom_d.as<double2>();
    d.atom_pg_f = s->d_pg_f.as<float>();
    d.atom_pg_d = s->d_pg_d.as<double>();
    for (int i = 0; i < 9; i++) d.Bf[i] = (float)s->B[i];
    d.types_d = s->d_types.as<TypeRadialT<double> >();
    d.types_f = s->d_types_f.as<TypeRadialT<float> >();
    d.term_pre_d = s->d_tcoeff.as<double>();
    d.term_pre_f = s->d_tpre_f.as<float>();
    d.term_exp_d = s->d_texp.as<double>();
    d.term_exp_f = s->d_texp_f.as<float>();
    d.term_m = s->d_tpow.as<int>();
    d.hkl = s->d_hkl.as<int4>();
    d.h2 = s->d_h2.as<double>();
    d.h2f = s->d_h2f.as<float>();
    d.table_f = s->d_table_f.as<float2>();
    d.table_d = s->d_table_d.as<double2>();
    d.table_stride = s->table_stride;
    d.table_split = s->table_split;
    d.table_shift = s->table_shift;
    d.atom_orig = s->d_perm.as<int>();
    d.atom_step_f = s->d_step_f.as<float2>();
    d.atom_step_d = s->d_step_d.as<double2>();
    d.atom_plm_lmax = s->d_plm_lmax.as<int>();
}

int common_atoms(dsf_engine *e, dsf_structure *s, const dsf_atoms *at)
{
    if (!at || at->n_atoms < 1) return fail(e, DSF_ERR_ARGUMENT, "structure needs at least one atom");
    const int n = at->n_atoms;
    s->n_atoms = n;
    s->xyz_conv = at->xyz_convention;
    s->adp_conv = at->adp_convention;
    if (s->xyz_conv < 0 || s->xyz_conv > 1) return fail(e, DSF_ERR_ARGUMENT, "bad xyz convention");
    if (s->adp_conv < 0 || s->adp_conv > 2) return fail(e, DSF_ERR_ARGUMENT, "bad ADP convention");
    s->adpk.resize(n);
    s->mult_w.resize(n);
    s->anom.assign(2 * (size_t)n, 0.0);
    s->atom_type.assign(n, 0);
    s->atom_wfn.assign(n, 0);
    for (int i = 0; i < n; i++) {
        const int k = at->adp_components ? at->adp_components[i] : 1;
        if (k != 0 && k != 1 && k != 6) return fail(e, DSF_ERR_ARGUMENT, "adp_components must be 0, 1 or 6");
        s->adpk[i] = k;
        s->mult_w[i] = (at->multiplicity ? at->multiplicity[i] : (double)s->n_total) / (double)s->n_total;
        if (at->atom_type) s->atom_type[i] = at->atom_type[i];
        if (at->atom_wfn) s->atom_wfn[i] = at->atom_wfn[i];
        if (at->anomalous) {
            s->anom[2 * i] = at->anomalous[2 * i];
            s->anom[2 * i + 1] = at->anomalous[2 * i + 1];
        }
    }
    // U_param -> U*_param (the kernel's beta basis without 2 pi^2)
    double A[9];
    const double lam[3] = {std::sqrt(s->B[0] * s->B[0] + s->B[3] * s->B[3] + s->B[6] * s->B[6]),
                           std::sqrt(s->B[1] * s->B[1] + s->B[4] * s->B[4] + s->B[7] * s->B[7]),
                           std::sqrt(s->B[2] * s->B[2] + s->B[5] * s->B[5] + s->B[8] * s->B[8])};
    if (s->adp_conv == DSF_ADP_U_CIF) {
        for (int i = 0; i < 9; i++) A[i] = 0;
        for (int i = 0; i < 3; i++) A[4 * i] = lam[i];
    } else if (s->adp_conv == DSF_ADP_U_CART) {
        std::copy(s->Minv, s->Minv + 9, A);  // U* = M^-1 U_cart M^-T
    } else {
        for (int i = 0; i < 9; i++) A[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    adp_param_map(A, s->A6);
    return DSF_OK;
}

int finish_create(dsf_engine *e, dsf_structure *s)
{
    int rc;
    if ((rc = upload(e, s->d_sym_rot, s->sym_rot.data(), s->sym_rot.size()))) return rc;
    if ((rc = upload(e, s->d_sym_t24, s->sym_t24.data(), s->sym_t24.size()))) return rc;
    if ((rc = upload_types(s))) return rc;
    DSF_CUDA(s->d_step_f.alloc(sizeof(float2) * (size_t)s->n_atoms * s->n_sym));
    DSF_CUDA(s->d_step_d.alloc(sizeof(double2) * (size_t)s->n_atoms * s->n_sym));
    refresh_dev(s);
    DSF_CUDA(cudaStreamSynchronize(e->setup));
    return DSF_OK;
}

}  // namespace

// Launch helpers of the per-call kernels, for the allocation-free entry
// point (dsf_noalloc.cu), which runs them on caller-provided buffers.
namespace dsf {
void host_cell_matrices(const double *cell, double *M, double *Minv, double *B) { cell_matrices(cell, M, Minv, B); }
void host_adp_param_map(const double *A, double *A6) { adp_param_map(A, A6); }
double host_centering_multiplier(char c, int obverse, int h, int k, int l)
{
    return centering_multiplier(c, obverse, h, k, l);
}
cudaError_t launch_adjoint_weights(int n, const double2 *dtdf, const double *mult, const double2 *cinv, int centro,
                                   double2 *gw_d, float2 *gw_f, cudaStream_t st)
{
    gw_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, dtdf, mult, cinv, centro, gw_d, gw_f, nullptr);
    return cudaGetLastError();
}
cudaError_t launch_f_epilogue(int n, const double2 *facc, const double *mult, const double2 *cinv, int centro,
                              double *f_out, cudaStream_t st)
{
    f_epilogue_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, facc, mult, cinv, centro, f_out, nullptr);
    return cudaGetLastError();
}
cudaError_t launch_grad_epilogue(int n_atoms, int xyz_conv, const double *Minv, const double *A6, int flags,
                                 const double *g_acc, const int *perm, const int *adpk, const double *w,
                                 const double *mult_w, const dsf_outputs *out, cudaStream_t st)
{
    GradParams P;
    P.n_atoms = n_atoms;
    P.xyz_conv = xyz_conv;
    std::copy(Minv, Minv + 9, P.Minv);
    std::copy(A6, A6 + 36, P.A6);
    P.want_xyz = (flags & DSF_D_XYZ) != 0;
    P.want_adp = (flags & DSF_D_ADP) != 0;
    P.want_occ = (flags & DSF_D_OCC) != 0;
    P.want_mp = 0;
    grad_epilogue_kernel<<<(n_atoms + 127) / 128, 128, 0, st>>>(P, g_acc, perm, adpk, w, mult_w, nullptr, nullptr,
                                                                 out->d_xyz, out->d_adp, out->d_occ, nullptr, nullptr,
                                                                 nullptr, nullptr);
    return cudaGetLastError();
}
}  // namespace dsf

// ==========================================================================
// C ABI
// ==========================================================================
// host-buffer batches of at least kPipelineBytes of inputs and outputs run as up to
// kPipelineGroups groups, so the host copies of one group overlap the GPU work of another
constexpr size_t kPipelineBytes = 64u << 20;
constexpr int kPipelineGroups = 4;

// host-side work of many structures on several threads when the bytes are worth it (batches of large
// reflection sets: the staging and copy-out memcpys dominate the host time); f(i) must only touch structure i.
// At most half the host's cores, and only above 32 MB, so a serving loop's other threads (structure set-up)
// keep theirs.
template <class F>
static void host_parallel(int n, size_t bytes, F f)
{
    unsigned nt = bytes < (32u << 20) ? 1u : std::min(8u, std::max(1u, std::thread::hardware_concurrency() / 2));
    nt = std::min<unsigned>(nt, (unsigned)std::max(1, n));
    if (nt <= 1) {
        for (int i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int> next{0};
    auto work = [&] {
        for (int i; (i = next.fetch_add(1)) < n;) f(i);
    };
    std::vector<std::thread> th;
    for (unsigned k = 1; k < nt; k++) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
}

extern "C" {

int dsf_abi_version(void) { return DSF_ABI_VERSION; }

int dsf_engine_create(int device, dsf_engine **out)
{
    if (!out) return DSF_ERR_ARGUMENT;
    *out = nullptr;
    dsf_engine *e = new dsf_engine();
    e->device = device;
    cudaError_t ce = cudaSetDevice(device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    // structure set-up (uploads, table builds) on the greatest stream priority: its kernels take SMs ahead of the
    // pending blocks of calculations running on other streams, so a new structure's first call does not wait
    // behind them
    int prio_low = 0, prio_high = 0;
    if (ce == cudaSuccess) ce = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithPriority(&e->setup, cudaStreamNonBlocking, prio_high);
    if (ce != cudaSuccess) {
        delete e;
        return DSF_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, device);
    int smem = 0;
    cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    e->max_smem = (size_t)smem;
    *out = e;
    return DSF_OK;
}

int dsf_engine_destroy(dsf_engine *e)
{
    if (!e) return DSF_ERR_ARGUMENT;
    if (e->live_structures > 0) return fail(e, DSF_ERR_STATE, "engine still owns structures; destroy them first");
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->setup) cudaStreamDestroy(e->setup);
    if (e->side) cudaStreamDestroy(e->side);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    if (e->d_rotfit) cudaFree(e->d_rotfit);
    delete e;
    return DSF_OK;
}

const char *dsf_last_error(const dsf_engine *e) { return e ? tl_err.c_str() : "null engine"; }

static int create_common(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms, int model,
                         dsf_structure **out, dsf_structure **sp)
{
    if (!e || !out) return DSF_ERR_ARGUMENT;
    *out = nullptr;
    cudaSetDevice(e->device);
    dsf_structure *s = new dsf_structure();
    s->eng = e;
    s->model = model;
    int rc = sym_from_desc(e, s, sym);
    if (!rc) rc = common_atoms(e, s, atoms);
    if (rc) {
        delete s;
        return rc;
    }
    *sp = s;
    return DSF_OK;
}

int dsf_structure_create_hc(dsf_engine *e, const dsf_symmetry *sym, const dsf_hc_model *m, const dsf_atoms *atoms,
                            dsf_structure **out)
{
    dsf_structure *s = nullptr;
    int rc = create_common(e, sym, atoms, MODEL_HC, out, &s);
    if (rc) return rc;
    auto bail = [&](int code) { delete s; return code; };
    if (!m || m->n_wfn < 1 || m->n_types < 1) return bail(fail(e, DSF_ERR_ARGUMENT, "HC model needs wavefunctions and types"));
    if (!atoms->lcs) return bail(fail(e, DSF_ERR_ARGUMENT, "HC model needs local coordinate systems"));
    s->n_wfn = m->n_wfn;
    s->n_types = m->n_types;
    for (int i = 0; i < s->n_atoms; i++) {
        if (s->atom_type[i] < 0 || s->atom_type[i] >= m->n_types) return bail(fail(e, DSF_ERR_ARGUMENT, "atom type index out of range"));
        if (s->atom_wfn[i] < 0 || s->atom_wfn[i] >= m->n_wfn) return bail(fail(e, DSF_ERR_ARGUMENT, "atom wavefunction index out of range"));
        if (!atoms->anomalous) {
            s->anom[2 * i] = m->anomalous ? m->anomalous[2 * s->atom_wfn[i]] : 0.0;
            s->anom[2 * i + 1] = m->anomalous ? m->anomalous[2 * s->atom_wfn[i] + 1] : 0.0;
        }
    }
    s->lcs.assign(atoms->lcs, atoms->lcs + 9 * (size_t)s->n_atoms);
    s->type_nl.assign(m->type_nl, m->type_nl + m->n_types);
    s->type_plm.assign(m->type_plm, m->type_plm + 25 * (size_t)m->n_types);
    s->type_pval.assign(m->type_pval, m->type_pval + m->n_types);
    s->type_kappa.assign(m->type_kappa, m->type_kappa + m->n_types);
    s->type_kappa_p.assign(m->type_kappa_prime, m->type_kappa_prime + m->n_types);
    // type -> wavefunction: that of the atoms using the type (unused types keep wavefunction 0)
    s->type_wfn.assign(m->n_types, 0);
    for (int i = 0; i < s->n_atoms; i++) s->type_wfn[s->atom_type[i]] = s->atom_wfn[i];
    // concatenated density terms: core of all wfns then valence of all wfns
    const int ncore = m->core_offset[m->n_wfn], nval = m->val_offset[m->n_wfn];
    s->tcoeff.clear(); s->texp.clear(); s->tpow.clear();
    for (int q = 0; q < ncore; q++) { s->tcoeff.push_back(m->core_coeff[q]); s->texp.push_back(m->core_exp[q]); s->tpow.push_back(m->core_pow[q]); }
    for (int q = 0; q < nval; q++) { s->tcoeff.push_back(m->val_coeff[q]); s->texp.push_back(m->val_exp[q]); s->tpow.push_back(m->val_pow[q]); }
    for (size_t q = 0; q < s->tpow.size(); q++)
        if (s->tpow[q] < 0 || s->tpow[q] > 8) return bail(fail(e, DSF_ERR_ARGUMENT, "density term r powers must be in 0..8"));
    if ((rc = build_type_radial(s, m))) return bail(rc);
    // val ranges point behind the core terms
    for (int t = 0; t < s->n_types; t++) {
        const int w = s->type_wfn[t];
        s->trad[t].val_begin = ncore + m->val_offset[w];
        s->trad[t].val_end = ncore + m->val_offset[w + 1];
    }
    {
        // the kernels evaluate 4 pi c G(n,0) as pre * core with pre = 4 pi c m!, m = n - 1 = pow + 1
        const size_t nt = s->tcoeff.size();
        std::vector<double> pre(nt);
        std::vector<float> pref(nt), zf(nt);
        std::vector<int> mm(nt);
        for (size_t q = 0; q < nt; q++) {
            mm[q] = s->tpow[q] + 1;
            pre[q] = 4.0 * DSF_PI * s->tcoeff[q] * g_prefactor(0, mm[q]);
            pref[q] = (float)pre[q];
            zf[q] = (float)s->texp[q];
        }
        if ((rc = upload(e, s->d_tcoeff, pre.data(), nt))) return bail(rc);
        if ((rc = upload(e, s->d_tpre_f, pref.data(), nt))) return bail(rc);
        if ((rc = upload(e, s->d_texp, s->texp.data(), nt))) return bail(rc);
        if ((rc = upload(e, s->d_texp_f, zf.data(), nt))) return bail(rc);
        if ((rc = upload(e, s->d_tpow, mm.data(), nt))) return bail(rc);
    }
    if ((rc = build_tiles(s, true))) return bail(rc);
    if ((rc = compute_global_plm(s))) return bail(rc);
    if ((rc = finish_create(e, s))) return bail(rc);
    e->live_structures++;
    *out = s;
    return DSF_OK;
}

int dsf_structure_create_iam(dsf_engine *e, const dsf_symmetry *sym, const dsf_iam_model *m, const dsf_atoms *atoms,
                             dsf_structure **out)
{
    dsf_structure *s = nullptr;
    int rc = create_common(e, sym, atoms, MODEL_IAM, out, &s);
    if (rc) return rc;
    auto bail = [&](int code) { delete s; return code; };
    if (!m || m->n_types < 1) return bail(fail(e, DSF_ERR_ARGUMENT, "IAM model needs types"));
    s->n_types = m->n_types;
    s->trad.assign(m->n_types, TypeHost{});
    for (int t = 0; t < m->n_types; t++) {
        TypeHost &r = s->trad[t];
        r.lmax_used = -1;
        r.iam_n = m->n_gauss[t];
        if (r.iam_n < 0 || r.iam_n > 5) return bail(fail(e, DSF_ERR_ARGUMENT, "at most 5 Gaussians per IAM type"));
        for (int q = 0; q < r.iam_n; q++) { r.iam_a[q] = m->a[5 * t + q]; r.iam_b[q] = m->b[5 * t + q]; }
        r.iam_c = m->c[t];
    }
    for (int i = 0; i < s->n_atoms; i++)
        if (s->atom_type[i] < 0 || s->atom_type[i] >= m->n_types) return bail(fail(e, DSF_ERR_ARGUMENT, "atom type index out of range"));
    if ((rc = build_tiles(s, true))) return bail(rc);
    std::vector<double> z(25 * (size_t)s->n_atoms, 0.0);
    std::vector<float> zf(25 * (size_t)s->n_atoms, 0.0f);
    if ((rc = upload(e, s->d_pg_d, z.data(), z.size()))) return bail(rc);
    if ((rc = upload(e, s->d_pg_f, zf.data(), zf.size()))) return bail(rc);
    s->dmat.assign(165 * (size_t)s->n_atoms, 0.0);
    if ((rc = upload(e, s->d_dmat, s->dmat.data(), s->dmat.size()))) return bail(rc);
    {
        std::vector<int> lmx(s->n_atoms, -1), tl(s->n_tiles, -1);
        if ((rc = upload(e, s->d_plm_lmax, lmx.data(), lmx.size()))) return bail(rc);
        if ((rc = upload(e, s->d_tile_lmax, tl.data(), tl.size()))) return bail(rc);
    }
    if ((rc = finish_create(e, s))) return bail(rc);
    e->live_structures++;
    *out = s;
    return DSF_OK;
}

int dsf_structure_set_hkl(dsf_structure *s, int n_hkl, const int *hkl);

// column layout of the tabulated model (see dsf_structure::table_stride)
static void table_columns(dsf_structure *s)
{
    int n_plain = 0;
    while (n_plain < s->n_atoms && s->adpk[s->perm[n_plain]] != 6) n_plain++;
    s->table_split = n_plain;
    s->table_shift = n_plain % 2;
    s->table_stride = (s->n_atoms + s->table_shift + 1) / 2 * 2;
}

// column c -> sorted atom index, or -1 for a padding column
__host__ __device__ inline int table_column_atom(int c, int split, int shift, int n_atoms)
{
    if (c < split) return c;
    const int a = c - shift;
    return (a >= split && a < n_atoms) ? a : -1;
}

int dsf_structure_create_tabulated(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms, int n_hkl,
                                   const int *hkl, const double *table, int table_fp32, dsf_structure **out)
{
    dsf_structure *s = nullptr;
    int rc = create_common(e, sym, atoms, MODEL_TABLE, out, &s);
    if (rc) return rc;
    auto bail = [&](int code) { delete s; return code; };
    if (!table || n_hkl < 1) return bail(fail(e, DSF_ERR_ARGUMENT, "tabulated model needs a table and reflections"));
    s->n_types = 1;
    s->trad.assign(1, TypeHost{});
    s->trad[0].lmax_used = -1;
    if ((rc = build_tiles(s, false))) return bail(rc);
    std::vector<double> z(25 * (size_t)s->n_atoms, 0.0);
    std::vector<float> zf(25 * (size_t)s->n_atoms, 0.0f);
    if ((rc = upload(e, s->d_pg_d, z.data(), z.size()))) return bail(rc);
    if ((rc = upload(e, s->d_pg_f, zf.data(), zf.size()))) return bail(rc);
    s->dmat.assign(165 * (size_t)s->n_atoms, 0.0);
    if ((rc = upload(e, s->d_dmat, s->dmat.data(), s->dmat.size()))) return bail(rc);
    {
        std::vector<int> lmx(s->n_atoms, -1), tl(s->n_tiles, -1);
        if ((rc = upload(e, s->d_plm_lmax, lmx.data(), lmx.size()))) return bail(rc);
        if ((rc = upload(e, s->d_tile_lmax, tl.data(), tl.size()))) return bail(rc);
    }
    // rows in the engine's line order (the order dsf_structure_set_hkl gives the reflections), padded with
    // zero rows to a multiple of kMaxHT reflections: the kernel reads whole sub-tiles
    const int n_pad = (n_hkl + kMaxHT - 1) / kMaxHT * kMaxHT;
    std::vector<int> order(n_hkl);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        for (int j = 0; j < 3; j++)
            if (hkl[3 * x + j] != hkl[3 * y + j]) return hkl[3 * x + j] < hkl[3 * y + j];
        return false;
    });
    // columns in the engine's (sorted) atom order, padded so every tile starts on a 16-byte boundary
    table_columns(s);
    const int nA = s->n_atoms, nS = s->n_sym, stride = s->table_stride;
    const size_t row = (size_t)nS * stride;  // complex values per reflection
    // [n_pad][stride][nS] plus 16 bytes of slack (the staged kernels read whole 16-byte units)
    std::vector<float> tf(2 * row * n_pad + 4, 0.0f);
    std::vector<double> td(table_fp32 ? 0 : 2 * row * n_pad, 0.0);
    for (int i = 0; i < n_hkl; i++)
        for (int op = 0; op < nS; op++)
            for (int c = 0; c < stride; c++) {
                const int a = table_column_atom(c, s->table_split, s->table_shift, nA);
                if (a < 0) continue;
                const size_t j = 2 * (((size_t)order[i] * nS + op) * nA + s->perm[a]);
                const size_t k = 2 * (row * i + (size_t)c * nS + op);
                tf[k] = (float)table[j];
                tf[k + 1] = (float)table[j + 1];
                if (!table_fp32) {
                    td[k] = table[j];
                    td[k + 1] = table[j + 1];
                }
            }
    if ((rc = upload(e, s->d_table_f, tf.data(), tf.size()))) return bail(rc);
    // an FP32 table is read widened by the plain form (no FP64 copy)
    if (!table_fp32 && (rc = upload(e, s->d_table_d, td.data(), td.size()))) return bail(rc);
    if ((rc = finish_create(e, s))) return bail(rc);
    s->eng->live_structures++;
    if ((rc = dsf_structure_set_hkl(s, n_hkl, hkl))) { s->eng->live_structures--; return bail(rc); }
    *out = s;
    return DSF_OK;
}

// gathers a caller's [n_hkl][n_sym][n_atoms] complex table (complex64 or
// complex128, the caller's reflection and atom order) into the engine's
// line-ordered, padded complex64 table [n_pad][stride][n_sym] with columns in
// the engine's atom order; rows past n_hkl are zero
__global__ void table_gather_kernel(int n_pad, int n_hkl, int n_sym, int n_atoms, int stride, int split, int shift,
                                    const int *order, const int *perm, const void *src, int src_fp64, float2 *dst)
{
    const size_t row = (size_t)n_sym * stride, total = (size_t)n_pad * row;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / row, q = i - r * row;
        const int c = (int)(q / n_sym), op = (int)(q - (size_t)c * n_sym);
        const int a = table_column_atom(c, split, shift, n_atoms);
        float2 v = make_float2(0.f, 0.f);
        if (r < (size_t)n_hkl && a >= 0) {
            const size_t j = ((size_t)order[r] * n_sym + op) * n_atoms + perm[a];
            if (src_fp64) {
                const double2 d = reinterpret_cast<const double2 *>(src)[j];
                v = make_float2((float)d.x, (float)d.y);
            } else {
                v = reinterpret_cast<const float2 *>(src)[j];
            }
        }
        dst[i] = v;
    }
}

int dsf_structure_create_tabulated_device(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms, int n_hkl,
                                          const int *hkl, const void *table_device, int table_fp64,
                                          dsf_structure **out)
{
    dsf_structure *s = nullptr;
    int rc = create_common(e, sym, atoms, MODEL_TABLE, out, &s);
    if (rc) return rc;
    auto bail = [&](int code) { delete s; return code; };
    if (!table_device || n_hkl < 1 || !hkl)
        return bail(fail(e, DSF_ERR_ARGUMENT, "tabulated model needs a table and reflections"));
    s->n_types = 1;
    s->trad.assign(1, TypeHost{});
    s->trad[0].lmax_used = -1;
    if ((rc = build_tiles(s, false))) return bail(rc);
    std::vector<double> z(25 * (size_t)s->n_atoms, 0.0);
    std::vector<float> zf(25 * (size_t)s->n_atoms, 0.0f);
    if ((rc = upload(e, s->d_pg_d, z.data(), z.size()))) return bail(rc);
    if ((rc = upload(e, s->d_pg_f, zf.data(), zf.size()))) return bail(rc);
    s->dmat.assign(165 * (size_t)s->n_atoms, 0.0);
    if ((rc = upload(e, s->d_dmat, s->dmat.data(), s->dmat.size()))) return bail(rc);
    {
        std::vector<int> lmx(s->n_atoms, -1), tl(s->n_tiles, -1);
        if ((rc = upload(e, s->d_plm_lmax, lmx.data(), lmx.size()))) return bail(rc);
        if ((rc = upload(e, s->d_tile_lmax, tl.data(), tl.size()))) return bail(rc);
    }
    // the engine's line order, as dsf_structure_set_hkl orders the reflections
    const int n_pad = (n_hkl + kMaxHT - 1) / kMaxHT * kMaxHT;
    std::vector<int> order(n_hkl);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        for (int j = 0; j < 3; j++)
            if (hkl[3 * x + j] != hkl[3 * y + j]) return hkl[3 * x + j] < hkl[3 * y + j];
        return false;
    });
    DevBuf d_order;
    if ((rc = upload(e, d_order, order.data(), order.size()))) return bail(rc);
    table_columns(s);
    const size_t row = (size_t)s->n_sym * s->table_stride;
    cudaError_t ce = s->d_table_f.alloc(sizeof(float2) * (row * n_pad + 2));  // 16 bytes of slack
    if (ce != cudaSuccess) {
        d_order.release();
        return bail(fail(e, DSF_ERR_MEMORY, "table allocation failed"));
    }
    cudaMemsetAsync(s->d_table_f.as<float2>() + row * n_pad, 0, 2 * sizeof(float2), e->setup);
    table_gather_kernel<<<std::max(1, e->n_sm) * 8, 256, 0, e->setup>>>(
        n_pad, n_hkl, s->n_sym, s->n_atoms, s->table_stride, s->table_split, s->table_shift, d_order.as<int>(),
        s->d_perm.as<int>(), table_device, table_fp64, s->d_table_f.as<float2>());
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->setup);
    d_order.release();
    if (ce != cudaSuccess) return bail(fail(e, DSF_ERR_CUDA, cudaGetErrorString(ce)));
    if ((rc = finish_create(e, s))) return bail(rc);
    s->eng->live_structures++;
    if ((rc = dsf_structure_set_hkl(s, n_hkl, hkl))) { s->eng->live_structures--; return bail(rc); }
    *out = s;
    return DSF_OK;
}

int dsf_structure_create_tsc(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms, int n_hkl,
                             const int *hkl, const char *path, dsf_structure **out)
{
    if (!e || !sym || !atoms || !hkl || !path || !out || n_hkl < 1 || sym->n_symops < 1)
        return fail(e, DSF_ERR_ARGUMENT, "tsc structure needs symmetry, atoms, reflections and a file");
    std::vector<float> tab;
    std::string err;
    int rc = tsc_expand(path, atoms->n_atoms, n_hkl, hkl, sym->n_symops, sym->symop_rotation, tab, err);
    if (rc) return fail(e, rc, err);
    cudaSetDevice(e->device);
    DevBuf d;
    DSF_CUDA(d.alloc(sizeof(float) * tab.size()));
    cudaError_t ce = cudaMemcpy(d.p, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        d.release();
        return fail(e, DSF_ERR_CUDA, cudaGetErrorString(ce));
    }
    rc = dsf_structure_create_tabulated_device(e, sym, atoms, n_hkl, hkl, d.p, 0, out);
    d.release();
    return rc;
}

int dsf_structure_destroy(dsf_structure *s)
{
    if (!s) return DSF_ERR_ARGUMENT;
    if (s->pending) return fail(s->eng, DSF_ERR_STATE, "a submitted call of this structure is still pending (dsf_poll)");
    cudaSetDevice(s->eng->device);
    cudaStreamSynchronize(s->eng->stream);
    cudaStreamSynchronize(s->eng->setup);
    DevBuf *bufs[] = {&s->d_sym_rot, &s->d_sym_t24, &s->d_tile_begin, &s->d_tile_ntypes, &s->d_tile_types,
                      &s->d_atom_ltype, &s->d_atom_adpk, &s->d_active, &s->d_xq, &s->d_xlo, &s->d_xd, &s->d_adp_f,
                      &s->d_adp_d, &s->d_w_f, &s->d_w_d, &s->d_anom_f, &s->d_anom_d, &s->d_pg_f, &s->d_pg_d,
                      &s->d_types, &s->d_types_f, &s->d_tcoeff, &s->d_texp, &s->d_tpow, &s->d_texp_f, &s->d_tpre_f, &s->d_hkl, &s->d_h2, &s->d_h2f, &s->d_hmult,
                      &s->d_cinv, &s->d_table_f, &s->d_table_d, &s->d_perm, &s->d_multw, &s->d_dmat, &s->d_raw,
                      &s->d_dtdf, &s->d_gw_d, &s->d_gw_f, &s->d_facc, &s->d_gacc, &s->d_out, &s->d_plm_lmax,
                      &s->d_rs_f, &s->d_rs_d, &s->d_tr_f, &s->d_tr_d, &s->d_trm_f, &s->d_trm_d, &s->d_err,
                      &s->d_hperm, &s->d_cont, &s->d_tile_lmax, &s->d_lcs, &s->d_type_plm, &s->d_type_lmax,
                      &s->d_atom_type0, &s->d_step_f, &s->d_step_d};
    for (DevBuf *b : bufs) b->release();
    if (s->ev_begin) cudaEventDestroy(s->ev_begin);
    if (s->ev_end) cudaEventDestroy(s->ev_end);
    if (s->pinned) cudaFreeHost(s->pinned);
    s->eng->live_structures--;
    delete s;
    return DSF_OK;
}

int dsf_structure_set_hkl(dsf_structure *s, int n_hkl, const int *hkl)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (n_hkl < 0 || (n_hkl > 0 && !hkl)) return fail(e, DSF_ERR_ARGUMENT, "bad reflection list");
    if (s->model == MODEL_TABLE && s->have_hkl && n_hkl != s->n_hkl)
        return fail(e, DSF_ERR_ARGUMENT, "tabulated structures keep the reflection set of their table");
    cudaSetDevice(e->device);
    if (n_hkl == 0) {
        // an empty set, as the reference accepts it: calls return no F and zero derivatives
        s->hperm.clear();
        s->n_hkl = 0;
        s->n_hkl_pad = 0;
        s->have_hkl = true;
        for (int p = 0; p < 2; p++) s->rs_ok[p] = s->tr_ok[p] = s->trm_ok[p] = false;
        refresh_dev(s);
        return DSF_OK;
    }
    // tables and per-reflection arrays padded with zero rows to whole sub-tiles (ht divides kMaxHT)
    const int n_pad = (n_hkl + kMaxHT - 1) / kMaxHT * kMaxHT;
    // line order: sorted by (h, k, l) so runs of l + 1 share a lattice line
    // (keys pack h, k, l in 21 bits each, offset to non-negative; the index breaks ties, so the order is
    // that of a stable sort)
    for (int i = 0; i < 3 * n_hkl; i++)
        if (hkl[i] <= -(1 << 20) || hkl[i] >= (1 << 20)) return fail(e, DSF_ERR_ARGUMENT, "Miller index out of range");
    {
        std::vector<std::pair<uint64_t, int>> key(n_hkl);
        for (int i = 0; i < n_hkl; i++) {
            const uint64_t h = (uint64_t)(hkl[3 * i] + (1 << 20)), k = (uint64_t)(hkl[3 * i + 1] + (1 << 20)),
                           l = (uint64_t)(hkl[3 * i + 2] + (1 << 20));
            key[i] = {(h << 42) | (k << 21) | l, i};
        }
        std::sort(key.begin(), key.end());
        s->hperm.resize(n_hkl);
        for (int i = 0; i < n_hkl; i++) s->hperm[i] = key[i].second;
    }
    std::vector<int> cont(n_pad, 0);
    for (int i = 1; i < n_hkl; i++) {
        const int *p = hkl + 3 * s->hperm[i - 1], *q = hkl + 3 * s->hperm[i];
        cont[i] = (p[0] == q[0] && p[1] == q[1] && q[2] == p[2] + 1) ? 1 : 0;
    }
    std::vector<int4> h4(n_pad, make_int4(0, 0, 0, 0));
    std::vector<double> h2(n_pad, 0.0), mult(n_pad, 0.0), cinv(2 * (size_t)n_pad, 0.0);
    // e^{2 pi i r / 24}, exact at quarter turns
    double turn24[24][2];
    for (int r = 0; r < 24; r++) {
        turn24[r][0] = std::cos(2.0 * DSF_PI * r / 24.0);
        turn24[r][1] = std::sin(2.0 * DSF_PI * r / 24.0);
        if (r % 6 == 0) {
            const int q = r / 6;
            turn24[r][0] = q == 0 ? 1.0 : q == 2 ? -1.0 : 0.0;
            turn24[r][1] = q == 1 ? 1.0 : q == 3 ? -1.0 : 0.0;
        }
    }
    for (int i = 0; i < n_hkl; i++) {
        const int *hp = hkl + 3 * s->hperm[i];
        const int h = hp[0], k = hp[1], l = hp[2];
        h4[i] = make_int4(h, k, l, 0);
        double c[3];
        for (int j = 0; j < 3; j++) c[j] = s->B[3 * j] * h + s->B[3 * j + 1] * k + s->B[3 * j + 2] * l;
        h2[i] = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        mult[i] = centering_multiplier(s->centering, s->obverse, h, k, l);
        int r = (h * s->t_inv24[0] + k * s->t_inv24[1] + l * s->t_inv24[2]) % 24;
        if (r < 0) r += 24;
        cinv[2 * i] = turn24[r][0];
        cinv[2 * i + 1] = turn24[r][1];
    }
    int rc;
    if ((rc = upload(e, s->d_hperm, s->hperm.data(), s->hperm.size()))) return rc;
    if ((rc = upload(e, s->d_cont, cont.data(), cont.size()))) return rc;
    if ((rc = upload(e, s->d_hkl, h4.data(), h4.size()))) return rc;
    if ((rc = upload(e, s->d_h2, h2.data(), h2.size()))) return rc;
    {
        std::vector<float> h2f(h2.begin(), h2.end());
        if ((rc = upload(e, s->d_h2f, h2f.data(), h2f.size()))) return rc;
    }
    if ((rc = upload(e, s->d_hmult, mult.data(), mult.size()))) return rc;
    if ((rc = upload(e, s->d_cinv, cinv.data(), cinv.size()))) return rc;
    DSF_CUDA(s->d_dtdf.alloc(16 * (size_t)n_pad));
    DSF_CUDA(s->d_gw_d.alloc(16 * (size_t)n_pad));
    DSF_CUDA(s->d_gw_f.alloc(8 * (size_t)n_pad));
    DSF_CUDA(s->d_facc.alloc(16 * (size_t)n_pad));
    DSF_CUDA(cudaMemsetAsync(s->d_gw_d.p, 0, 16 * (size_t)n_pad, e->setup));
    DSF_CUDA(cudaMemsetAsync(s->d_gw_f.p, 0, 8 * (size_t)n_pad, e->setup));
    DSF_CUDA(s->d_err.alloc(sizeof(int)));
    DSF_CUDA(cudaMemsetAsync(s->d_err.p, 0, sizeof(int), e->setup));
    s->n_hkl = n_hkl;
    s->n_hkl_pad = n_pad;
    s->have_hkl = true;
    refresh_dev(s);
    // resident per-(reflection, operation) and radial tables: FP32 now, FP64 on the first FP64 call
    for (int p = 0; p < 2; p++) s->rs_ok[p] = s->tr_ok[p] = s->trm_ok[p] = false;
    int rc2 = ensure_tables(s, false, false);
    if (rc2) return rc2;
    DSF_CUDA(cudaStreamSynchronize(e->setup));
    return DSF_OK;
}

int dsf_structure_update_atoms(dsf_structure *s, const double *xyz, const double *adp, const double *occ)
{
    if (!s || !xyz || !occ) return s ? fail(s->eng, DSF_ERR_ARGUMENT, "xyz and occupancy are required") : DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    cudaSetDevice(e->device);
    const int n = s->n_atoms;
    std::vector<double> raw(10 * (size_t)n, 0.0);
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < 3; j++) {
            raw[10 * i + j] = xyz[3 * i + j];
            if (!std::isfinite(xyz[3 * i + j])) return fail(e, DSF_ERR_ARGUMENT, "non-finite coordinate");
        }
        if (adp)
            for (int j = 0; j < s->adpk[i]; j++) raw[10 * i + 3 + j] = adp[6 * i + j];
        raw[10 * i + 9] = occ[i];
    }
    DSF_CUDA(cudaMemcpyAsync(s->d_raw.p, raw.data(), raw.size() * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    AtomParams P;
    P.n_atoms = n;
    P.xyz_conv = s->xyz_conv;
    std::copy(s->Minv, s->Minv + 9, P.Minv);
    std::copy(s->A6, s->A6 + 36, P.A6);
    atom_convert_kernel<<<(n + 127) / 128, 128, 0, e->stream>>>(
        P, s->d_raw.as<double>(), s->d_perm.as<int>(), s->d_atom_adpk.as<int>(), s->d_multw.as<double>(),
        s->d_xq.as<uint32_t>(), s->d_xlo.as<float>(), s->d_xd.as<double>(), s->d_adp_f.as<float>(),
        s->d_adp_d.as<double>(), s->d_w_f.as<float>(), s->d_w_d.as<double>(), s->n_sym, s->d_sym_rot.as<int>(),
        s->d_sym_t24.as<int>(), s->d_step_f.as<float2>(), s->d_step_d.as<double2>());
    DSF_CUDA(cudaGetLastError());
    DSF_CUDA(cudaStreamSynchronize(e->stream));
    s->have_atoms = true;
    return DSF_OK;
}

int dsf_structure_update_types(dsf_structure *s, const double *plm, const double *pval, const double *kappa,
                               const double *kappa_p)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (s->model != MODEL_HC) return fail(e, DSF_ERR_STATE, "multipole parameters exist only for HC structures");
    cudaSetDevice(e->device);
    const int nT = s->n_types;
    if (plm) s->type_plm.assign(plm, plm + 25 * (size_t)nT);
    if (pval) s->type_pval.assign(pval, pval + nT);
    if (kappa) s->type_kappa.assign(kappa, kappa + nT);
    if (kappa_p) s->type_kappa_p.assign(kappa_p, kappa_p + nT);
    for (int t = 0; t < nT; t++) {
        TypeHost &r = s->trad[t];
        r.pv = s->type_pval[t];
        r.kappa = s->type_kappa[t];
        r.kappa_p = s->type_kappa_p[t];
        int lp = -1;
        for (int l = 0; l < s->type_nl[t] && l <= 4; l++)
            for (int q = 0; q < 2 * l + 1; q++)
                if (s->type_plm[25 * (size_t)t + l * l + q] != 0.0) lp = l;
        r.lmax_used = std::min(lp, std::min(4, r.n_def - 1));
    }
    int rc;
    if ((rc = upload_types(s))) return rc;
    if (plm && (rc = compute_global_plm(s))) return rc;
    for (int p = 0; p < 2; p++) s->tr_ok[p] = s->trm_ok[p] = false;
    if ((rc = ensure_tables(s, false, false))) return rc;
    refresh_dev(s);
    DSF_CUDA(cudaStreamSynchronize(e->setup));
    return DSF_OK;
}

int dsf_structure_set_electron(dsf_structure *s, int on, const int *wfn_z, const double *wfn_f000)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (s->model != MODEL_HC) return fail(e, DSF_ERR_STATE, "electron conversion applies to HC structures");
    if (on && (!wfn_z || !wfn_f000)) return fail(e, DSF_ERR_ARGUMENT, "atomic numbers and f_e(0) are required");
    cudaSetDevice(e->device);
    for (int t = 0; t < s->n_types; t++) {
        const int w = s->type_wfn[t];
        s->trad[t].e_z = on ? (double)wfn_z[w] : 0.0;
        s->trad[t].e_f000 = on ? wfn_f000[w] : 0.0;
    }
    s->electron = on ? 1 : 0;
    int rc;
    if ((rc = upload_types(s))) return rc;
    refresh_dev(s);
    for (int p = 0; p < 2; p++) s->tr_ok[p] = s->trm_ok[p] = false;
    if ((rc = ensure_tables(s, false, false))) return rc;
    return DSF_OK;
}

int dsf_structure_set_lcs(dsf_structure *s, const double *lcs)
{
    if (!s || !lcs) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (s->model != MODEL_HC) return fail(e, DSF_ERR_STATE, "local coordinate systems exist only for HC structures");
    cudaSetDevice(e->device);
    s->lcs.assign(lcs, lcs + 9 * (size_t)s->n_atoms);
    int rc = compute_global_plm(s);
    if (rc) return rc;
    refresh_dev(s);
    DSF_CUDA(cudaStreamSynchronize(e->setup));
    return DSF_OK;
}

int64_t dsf_structure_device_bytes(const dsf_structure *s)
{
    if (!s) return 0;
    const DevBuf *bufs[] = {&s->d_sym_rot, &s->d_sym_t24, &s->d_tile_begin, &s->d_tile_ntypes, &s->d_tile_types,
                            &s->d_atom_ltype, &s->d_atom_adpk, &s->d_active, &s->d_xq, &s->d_xlo, &s->d_xd,
                            &s->d_adp_f, &s->d_adp_d, &s->d_w_f, &s->d_w_d, &s->d_anom_f, &s->d_anom_d, &s->d_pg_f,
                            &s->d_pg_d, &s->d_types, &s->d_types_f, &s->d_tcoeff, &s->d_texp, &s->d_tpow, &s->d_texp_f, &s->d_tpre_f, &s->d_hkl, &s->d_h2, &s->d_h2f,
                            &s->d_hmult, &s->d_cinv, &s->d_table_f, &s->d_table_d, &s->d_perm, &s->d_multw,
                            &s->d_dmat, &s->d_raw, &s->d_dtdf, &s->d_gw_d, &s->d_gw_f, &s->d_facc, &s->d_gacc,
                            &s->d_out, &s->d_plm_lmax, &s->d_rs_f, &s->d_rs_d, &s->d_tr_f, &s->d_tr_d,
                            &s->d_trm_f, &s->d_trm_d, &s->d_err, &s->d_hperm, &s->d_cont, &s->d_tile_lmax,
                            &s->d_lcs, &s->d_type_plm, &s->d_type_lmax, &s->d_atom_type0, &s->d_step_f, &s->d_step_d};
    int64_t b = 0;
    for (const DevBuf *p : bufs) b += (int64_t)p->bytes;
    return b;
}

int dsf_last_launch_count(const dsf_structure *s) { return s ? s->last_launches : 0; }

double dsf_last_kernel_ms(dsf_structure *s)
{
    if (!s || !s->ev_begin) return -1.0;
    cudaSetDevice(s->eng->device);
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, s->ev_begin, s->ev_end) != cudaSuccess) {
        cudaGetLastError();
        return -1.0;
    }
    return (double)ms;
}

// ---------------------------------------------------------------------------
// one call, in phases: checks, adjoint weights + zeroed accumulators, the SF
// kernel launches (one per ADP kind), the F and derivative epilogues
// ---------------------------------------------------------------------------
static int call_check(dsf_structure *s, int precision, int flags, const double *dtdf_device, const dsf_outputs *out)
{
    dsf_engine *e = s->eng;
    if (!s->have_hkl) return fail(e, DSF_ERR_STATE, "no reflections set");
    if (!s->have_atoms) return fail(e, DSF_ERR_STATE, "atomic parameters not uploaded");
    if (!out || (s->n_hkl > 0 && (!out->f || !dtdf_device)))
        return fail(e, DSF_ERR_ARGUMENT, "dtdf and f are required");
    if (precision != DSF_FP64 && precision != DSF_FP32_BULK) return fail(e, DSF_ERR_ARGUMENT, "unknown precision");
    const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
    return ensure_tables(s, precision == DSF_FP64, mp);
}

static int call_pre(dsf_structure *s, const double *dtdf_device, cudaStream_t st)
{
    dsf_engine *e = s->eng;
    const int n_hkl = s->n_hkl, n_g = kNch * s->n_atoms, n = std::max(n_hkl, n_g);
    call_pre_kernel<<<(n + 255) / 256, 256, 0, st>>>(n_hkl, n_g, reinterpret_cast<const double2 *>(dtdf_device),
                                                     s->d_hmult.as<double>(), s->d_cinv.as<double2>(),
                                                     s->centro_mode, s->d_gw_d.as<double2>(),
                                                     s->d_gw_f.as<float2>(), s->d_hperm.as<int>(),
                                                     s->d_facc.as<double2>(), s->d_gacc.as<double>());
    DSF_CUDA(cudaGetLastError());
    return DSF_OK;
}

static void call_buffers(dsf_structure *s, bool fp64, CallBuffers &C, SfLaunch &L, SignTable &G)
{
    C.gw_d = s->d_gw_d.as<double2>();
    C.gw_f = s->d_gw_f.as<float2>();
    C.f_acc = s->d_facc.as<double2>();
    C.g_acc = s->d_gacc.as<double>();
    L = SfLaunch{};
    L.n_hkl_pad = s->n_hkl_pad;
    L.rs = fp64 ? s->d_rs_d.p : s->d_rs_f.p;
    L.tr = fp64 ? s->d_tr_d.p : s->d_tr_f.p;
    L.trm = fp64 ? s->d_trm_d.p : s->d_trm_f.p;
    L.error = s->d_err.as<int>();
    L.stall_first = s->debug_stall;
    s->debug_stall = 0;
    L.cont = s->d_cont.as<int>();
    L.tile_lmax = s->d_tile_lmax.as<int>();
    // coset kernels: operations in sign-diagonal cosets (HC: harmonics and ADPs; other models: ADPs)
    L.coset = 0;
    std::memset(&G, 0, sizeof(G));
    if (s->coset_size && coset_form_compiled(fp64, s->model, s->n_sym, s->coset_size)) {
        L.coset = s->coset_size;
        for (int op = 0; op < s->n_sym; op++)
            for (int c = 0; c < 8; c++) {
                int sg = 1, fs = 1;
                for (int i = 0; i < 3; i++)
                    if ((c >> i) & 1) {
                        sg *= s->sym_sign[3 * op + i];
                        fs *= s->sym_fsign[3 * op + i];
                    }
                G.f[op][c] = (float)sg;
                G.d[op][c] = (double)sg;
                G.xf[op][c] = (float)fs;
                G.xd[op][c] = (double)fs;
            }
    }
}

// launch shape of the tiles of one ADP kind: reflections per sub-tile from the
// shared-memory budget (several blocks per SM), reflection chunks of about
// `block_terms` atom x reflection pairs per block (at least four sub-tiles)
static int kind_shape(dsf_structure *s, int kind, bool fp64, bool mp, double block_terms, SfLaunch &L, int &nt,
                      int &n_chunks, size_t &smem, int ht_cap = 0, bool short_chunks = false)
{
    dsf_engine *e = s->eng;
    const int t0 = kind ? s->n_tiles_plain : 0, t1 = kind ? s->n_tiles : s->n_tiles_plain;
    nt = t1 - t0;
    n_chunks = 0;
    if (nt <= 0) return DSF_OK;
    L.tile_offset = t0;
    L.max_types = kind ? s->max_types_aniso : s->max_types_plain;
    int ht = kMaxHT;
    size_t budget = std::min<size_t>(e->max_smem, fp64 ? 200 * 1024 : 100 * 1024);
    const bool table = s->model == MODEL_TABLE;
    // the staged FP32 table dominates the stage: a smaller budget keeps four blocks per SM
    if (table && !fp64) budget = std::min<size_t>(budget, 64 * 1024);
    while (ht > 4 && sf3_smem_bytes(fp64, mp, ht, s->n_sym, L.max_types, table) > budget) ht /= 2;
    while (ht_cap >= 4 && ht > ht_cap) ht /= 2;
    smem = sf3_smem_bytes(fp64, mp, ht, s->n_sym, L.max_types, table);
    if (smem > e->max_smem) return fail(e, DSF_ERR_UNSUPPORTED, "shared-memory tile does not fit this device");
    int chunk = (int)std::min<double>(s->n_hkl, std::max(1.0, block_terms / kTileAtoms));
    // short_chunks (a single structure's launch): a small problem whose reflection chunks would be shorter than
    // four sub-tiles takes shorter sub-tiles instead (down to 4 reflections), so its grid still spreads over the
    // SMs; larger problems are unchanged
    if (short_chunks)
        while (ht > 4 && chunk < 4 * ht) ht /= 2;
    smem = sf3_smem_bytes(fp64, mp, ht, s->n_sym, L.max_types, table);
    L.ht = ht;
    chunk = std::max(chunk, 4 * ht);
    chunk = (chunk + ht - 1) / ht * ht;
    L.hkl_chunk = chunk;
    n_chunks = (s->n_hkl + chunk - 1) / chunk;
    return DSF_OK;
}

static int call_post(dsf_structure *s, int flags, const dsf_outputs *out, cudaStream_t st, int &launches)
{
    dsf_engine *e = s->eng;
    const int n_hkl = s->n_hkl, n = s->n_atoms;
    const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
    const bool grad = (flags & (DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC | DSF_D_MULTIPOLE)) != 0;
    GradParams P;
    P.n_atoms = n;
    P.xyz_conv = s->xyz_conv;
    std::copy(s->Minv, s->Minv + 9, P.Minv);
    std::copy(s->A6, s->A6 + 36, P.A6);
    P.want_xyz = (flags & DSF_D_XYZ) != 0;
    P.want_adp = (flags & DSF_D_ADP) != 0;
    P.want_occ = (flags & DSF_D_OCC) != 0;
    P.want_mp = mp;
    const int m = grad ? std::max(n_hkl, n) : n_hkl;
    call_post_kernel<<<(m + 127) / 128, 128, 0, st>>>(
        n_hkl, s->d_facc.as<double2>(), s->d_hmult.as<double>(), s->d_cinv.as<double2>(), s->centro_mode, out->f,
        s->d_hperm.as<int>(), grad ? 1 : 0, P, s->d_gacc.as<double>(), s->d_perm.as<int>(),
        s->d_atom_adpk.as<int>(), s->d_w_d.as<double>(), s->d_multw.as<double>(), s->d_dmat.as<double>(),
        s->d_plm_lmax.as<int>(), out->d_xyz, out->d_adp, out->d_occ, out->d_pval, out->d_plm, out->d_kappa,
        out->d_kappa_prime);
    launches++;
    DSF_CUDA(cudaGetLastError());
    return DSF_OK;
}

// reflection chunks of one structure's launch over ntk tiles: many blocks (about 75 per SM over the grid) so the
// blocks of unequal tiles even out across the SMs, but at least 256 reflections (16 sub-tiles) per block so the
// per-block set-up (atom loads, the final derivative commits) stays small -- unless that leaves fewer than four
// blocks per SM (small structures)
static int chunk_count(const dsf_engine *e, int ntk, int n_hkl, int blocks_per_sm = 75)
{
    const int sm = std::max(1, e->n_sm), t = std::max(1, ntk);
    return std::max(1, std::max(std::min(sm * blocks_per_sm / t, n_hkl / 256), sm * 4 / t));
}

// ---------------------------------------------------------------------------
// tile-shape autotuner: per shape key, the blocks per SM the reflection chunks
// aim at and the sub-tile length, chosen by timing a few candidates
// ---------------------------------------------------------------------------
static int log2_bucket(double x) { return x > 1 ? (int)std::lround(2.0 * std::log2(x)) : 0; }

// the shape a structure's call depends on: model, precision, multipole adjoint, derivative pass, operation
// count, coset form, atoms and reflections in half-octaves, the device's SM count
static std::string tune_key(const dsf_structure *s, bool fp64, bool mp, bool grad)
{
    char k[160];
    std::snprintf(k, sizeof k, "m%d-p%d-mp%d-g%d-ns%d-cs%d-iv%d-a%d-h%d-sm%d", s->model, fp64 ? 64 : 32, mp ? 1 : 0,
                  grad ? 1 : 0, s->n_sym, s->coset_size, s->inv_pairs, log2_bucket(s->n_atoms),
                  log2_bucket(s->n_hkl), s->eng->n_sm);
    return k;
}

// blocks per SM, sub-tile cap and register-capped form of a call: the autotuner's candidate under trial, else the
// tuned shape of the key, else the rule (75 blocks per SM, the longest sub-tile, the compiler's registers)
static void call_shape(dsf_structure *s, bool fp64, bool mp, bool grad, int &bps, int &ht, int &occ3)
{
    bps = 75;
    ht = 0;
    occ3 = 0;
    if (s->tune_bps > 0) {
        bps = s->tune_bps;
        ht = s->tune_ht;
        occ3 = s->tune_occ3;
        return;
    }
    dsf_engine *e = s->eng;
    std::lock_guard<std::mutex> lock(e->tune_mtx);
    auto it = e->tuned.find(tune_key(s, fp64, mp, grad));
    if (it != e->tuned.end()) {
        bps = it->second[0];
        ht = it->second[1];
        occ3 = it->second[2];
    }
}

// the inversion-pair kernels: FP32 generic models (tabulated, IAM) with a compiled operation count
static bool inv_kernel(const dsf_structure *s, bool fp64)
{
    return s->inv_pairs && !fp64 && s->model != MODEL_HC && table_count_compiled(s->n_sym);
}

// a call on an empty reflection set: no F, the requested derivatives zero (the reference's engines sum over no
// reflections); no kernels
static int empty_call(dsf_structure *s, int flags, const dsf_outputs *out, cudaStream_t st)
{
    dsf_engine *e = s->eng;
    const size_t n = (size_t)s->n_atoms;
    const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
    struct { double *p; size_t len; bool want; } z[] = {
        {out->d_xyz, 3 * n, (flags & DSF_D_XYZ) != 0}, {out->d_adp, 6 * n, (flags & DSF_D_ADP) != 0},
        {out->d_occ, n, (flags & DSF_D_OCC) != 0},     {out->d_pval, n, mp},
        {out->d_plm, 25 * n, mp},                       {out->d_kappa, n, mp},
        {out->d_kappa_prime, n, mp}};
    for (auto &q : z)
        if (q.want && q.p) DSF_CUDA(cudaMemsetAsync(q.p, 0, sizeof(double) * q.len, st));
    s->last_launches = 0;
    return DSF_OK;
}

int dsf_calculate_device(dsf_structure *s, int precision, int flags, const double *dtdf_device,
                         const dsf_outputs *out, void *stream)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    int rc = call_check(s, precision, flags, dtdf_device, out);
    if (rc) return rc;
    cudaSetDevice(e->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    if (s->n_hkl == 0) return empty_call(s, flags, out, st);
    const bool fp64 = precision == DSF_FP64;
    const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
    if ((rc = call_pre(s, dtdf_device, st))) return rc;
    int launches = 1;
    CallBuffers C;
    SfLaunch L;
    SignTable G;
    call_buffers(s, fp64, C, L, G);
    if (!s->ev_begin) {
        DSF_CUDA(cudaEventCreate(&s->ev_begin));
        DSF_CUDA(cudaEventCreate(&s->ev_end));
    }
    const bool grad = (flags & (DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC | DSF_D_MULTIPOLE)) != 0;
    int bps, ht_cap, occ3;
    call_shape(s, fp64, mp, grad, bps, ht_cap, occ3);
    DSF_CUDA(cudaEventRecord(s->ev_begin, st));
    // one launch per ADP kind (tiles [0, n_tiles_plain) without anisotropic ADPs), reflection chunks of
    // chunk_count
    for (int kind = 0; kind < 2; kind++) {
        int nt, n_chunks;
        size_t smem;
        const int ntk = kind ? s->n_tiles - s->n_tiles_plain : s->n_tiles_plain;
        const int n_chunks0 = chunk_count(e, ntk, s->n_hkl, bps);
        const double block_terms = (double)kTileAtoms * ((s->n_hkl + n_chunks0 - 1) / n_chunks0);
        if ((rc = kind_shape(s, kind, fp64, mp, block_terms, L, nt, n_chunks, smem, ht_cap, true))) return rc;
        if (nt <= 0) continue;
        K3Args A;
        A.S = &s->dev;
        A.C = &C;
        A.L = &L;
        A.G = &G;
        A.n_sym = s->n_sym;
        A.coset = L.coset;
        A.pattern = wht_pattern_of(G, s->n_sym, L.coset, s->model == MODEL_HC);
        A.n_tiles = nt;
        A.n_chunks = n_chunks;
        A.smem = smem;
        A.st = st;
        A.grad = grad;
        A.inv = inv_kernel(s, fp64);
        A.occ3 = occ3 != 0;
        DSF_CUDA(launch_sf3(A, s->model, fp64, mp, kind == 1));
        launches++;
    }
    DSF_CUDA(cudaEventRecord(s->ev_end, st));
    if ((rc = call_post(s, flags, out, st, launches))) return rc;
    s->last_launches = launches;
    return DSF_OK;
}

// Times the structure's call over a few tile shapes (reflection chunks aiming at 24, 48, 75 or 150 blocks per
// SM; the longest sub-tile the shared-memory budget allows, or at most 8 reflections) with a zero dT/dF on scratch
// buffers, and keeps the fastest for every later call of structures with the same shape key.  Any shape gives
// the same sums (the cross-block sums in another order).
int dsf_autotune(dsf_structure *s, int precision, int flags, int *blocks_per_sm, int *ht, int *occupancy,
                 double *best_ms)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (precision != DSF_FP64 && precision != DSF_FP32_BULK) return fail(e, DSF_ERR_ARGUMENT, "unknown precision");
    if (s->n_hkl == 0) return fail(e, DSF_ERR_STATE, "no reflections to tune on");
    cudaSetDevice(e->device);
    const bool fp64 = precision == DSF_FP64;
    const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
    const bool grad = (flags & (DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC | DSF_D_MULTIPOLE)) != 0;
    const size_t n = (size_t)s->n_atoms, m = (size_t)s->n_hkl;
    const size_t doubles = 2 * m + 2 * m + n * (3 + 6 + 1) + (mp ? n * 28 : 0);
    double *buf = nullptr;
    DSF_CUDA(cudaMalloc(&buf, sizeof(double) * doubles));
    DSF_CUDA(cudaMemsetAsync(buf, 0, sizeof(double) * doubles, e->stream));
    dsf_outputs out{};
    double *p = buf + 2 * m;  // buf[0, 2m): dT/dF = 0
    out.f = p; p += 2 * m;
    out.d_xyz = p; p += 3 * n;
    out.d_adp = p; p += 6 * n;
    out.d_occ = p; p += n;
    if (mp) {
        out.d_pval = p; p += n;
        out.d_plm = p; p += 25 * n;
        out.d_kappa = p; p += n;
        out.d_kappa_prime = p;
    }
    int rc = DSF_OK;
    auto timed = [&](int bps, int cap, int occ3, double &ms) {
        s->tune_bps = bps;
        s->tune_ht = cap;
        s->tune_occ3 = occ3;
        rc = dsf_calculate_device(s, precision, flags, buf, &out, e->stream);
        s->tune_bps = s->tune_ht = s->tune_occ3 = 0;
        if (rc) return false;
        if (cudaStreamSynchronize(e->stream) != cudaSuccess) {
            rc = fail(e, DSF_ERR_CUDA, "autotune call failed");
            return false;
        }
        ms = dsf_last_kernel_ms(s);
        return ms >= 0;
    };
    double warm = 0, best = 1e300;
    int best_bps = 75, best_cap = 0, best_occ3 = 0;
    // the register-capped form exists for the FP32 multipole-adjoint kernels
    const int n_occ = (s->model == MODEL_HC && mp && !fp64) ? 2 : 1;
    if (timed(75, 0, 0, warm)) {
        const int reps = warm < 20.0 ? 3 : 1;
        for (int occ3 = 0; occ3 < n_occ && !rc; occ3++)
            for (const int bps : {24, 48, 75, 150})
                for (const int cap : {0, 8}) {
                    double t = 1e300;
                    for (int r = 0; r < reps; r++) {
                        double ms;
                        if (!timed(bps, cap, occ3, ms)) break;
                        t = std::min(t, ms);
                    }
                    if (rc) break;
                    if (t < best) {
                        best = t;
                        best_bps = bps;
                        best_cap = cap;
                        best_occ3 = occ3;
                    }
                }
    }
    cudaFree(buf);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lock(e->tune_mtx);
        e->tuned[tune_key(s, fp64, mp, grad)] = {best_bps, best_cap, best_occ3};
    }
    if (blocks_per_sm) *blocks_per_sm = best_bps;
    if (ht) *ht = best_cap;
    if (occupancy) *occupancy = best_occ3 ? 3 : 0;
    if (best_ms) *best_ms = best;
    return DSF_OK;
}

// the tile shape the next call of s with these settings takes (tuned, or the rule's 75 blocks per SM and the
// longest sub-tile, ht = 0); *tuned = 1 when it comes from the autotuner
int dsf_tuning_lookup(dsf_structure *s, int precision, int flags, int *blocks_per_sm, int *ht, int *occupancy,
                      int *tuned)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    const bool fp64 = precision == DSF_FP64;
    const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
    const bool grad = (flags & (DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC | DSF_D_MULTIPOLE)) != 0;
    std::lock_guard<std::mutex> lock(e->tune_mtx);
    auto it = e->tuned.find(tune_key(s, fp64, mp, grad));
    const bool hit = it != e->tuned.end();
    if (blocks_per_sm) *blocks_per_sm = hit ? it->second[0] : 75;
    if (ht) *ht = hit ? it->second[1] : 0;
    if (occupancy) *occupancy = (hit && it->second[2]) ? 3 : 0;
    if (tuned) *tuned = hit ? 1 : 0;
    return DSF_OK;
}

// the tuned shapes as text, one "key blocks_per_sm ht" line each
int dsf_tuning_save(dsf_engine *e, const char *path)
{
    if (!e || !path) return DSF_ERR_ARGUMENT;
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(e, DSF_ERR_ARGUMENT, "cannot write the tuning file");
    std::lock_guard<std::mutex> lock(e->tune_mtx);
    for (const auto &kv : e->tuned)
        std::fprintf(f, "%s %d %d %d\n", kv.first.c_str(), kv.second[0], kv.second[1], kv.second[2]);
    std::fclose(f);
    return DSF_OK;
}

// adds the shapes of a file written by dsf_tuning_save (keys name the device's SM count, so shapes tuned on
// another kind of device are never matched)
int dsf_tuning_load(dsf_engine *e, const char *path)
{
    if (!e || !path) return DSF_ERR_ARGUMENT;
    FILE *f = std::fopen(path, "r");
    if (!f) return fail(e, DSF_ERR_ARGUMENT, "cannot read the tuning file");
    char key[160];
    int bps, ht, occ3;
    std::lock_guard<std::mutex> lock(e->tune_mtx);
    while (std::fscanf(f, "%159s %d %d %d", key, &bps, &ht, &occ3) == 4)
        if (bps > 0 && bps <= 4096 && ht >= 0 && ht <= kMaxHT && (occ3 == 0 || occ3 == 1)) e->tuned[key] = {bps, ht, occ3};
    std::fclose(f);
    return DSF_OK;
}

// Many structures of one engine in one submission: the FP32 SF kernels of all
// structures without the multipole adjoint run as batched launches (one per
// kernel shape and sign table, up to kBatchItems structures each); the rest
// (FP64, multipole adjoint) launch per structure.  Adjoint weights and
// epilogues launch per structure.
int dsf_calculate_batch_device(dsf_structure *const *structures, int n, int precision, int flags,
                               const double *const *dtdf_device, const dsf_outputs *out_device, void *stream)
{
    if (!structures || n < 1 || !dtdf_device || !out_device) return DSF_ERR_ARGUMENT;
    dsf_engine *e = structures[0] ? structures[0]->eng : nullptr;
    if (!e) return DSF_ERR_ARGUMENT;
    int n_empty = 0;
    for (int i = 0; i < n; i++) {
        if (!structures[i] || structures[i]->eng != e)
            return fail(e, DSF_ERR_ARGUMENT, "batch structures must belong to one engine");
        int rc = call_check(structures[i], precision, flags, dtdf_device[i], &out_device[i]);
        if (rc) return rc;
        n_empty += structures[i]->n_hkl == 0;
    }
    cudaSetDevice(e->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    if (n_empty) {  // structures with an empty reflection set: zero derivatives; the rest as a batch
        std::vector<dsf_structure *> sv;
        std::vector<const double *> dv;
        std::vector<dsf_outputs> ov;
        for (int i = 0; i < n; i++) {
            if (structures[i]->n_hkl == 0) {
                int rc = empty_call(structures[i], flags, &out_device[i], st);
                if (rc) return rc;
            } else {
                sv.push_back(structures[i]);
                dv.push_back(dtdf_device[i]);
                ov.push_back(out_device[i]);
            }
        }
        if (sv.empty()) return DSF_OK;
        return dsf_calculate_batch_device(sv.data(), (int)sv.size(), precision, flags, dv.data(), ov.data(), st);
    }
    const bool fp64 = precision == DSF_FP64;
    int launches = 0, rc;
    // adjoint weights and zeroed accumulators of all structures, kPrePostItems per launch
    std::vector<PrePostItem> pp(n);
    for (int i = 0; i < n; i++) {
        dsf_structure *s = structures[i];
        PrePostItem &it = pp[i];
        it.n_hkl = s->n_hkl;
        it.n_atoms = s->n_atoms;
        it.centro = s->centro_mode;
        it.dtdf = reinterpret_cast<const double2 *>(dtdf_device[i]);
        it.mult = s->d_hmult.as<double>();
        it.cinv = s->d_cinv.as<double2>();
        it.hperm = s->d_hperm.as<int>();
        it.gw_d = s->d_gw_d.as<double2>();
        it.gw_f = s->d_gw_f.as<float2>();
        it.facc = s->d_facc.as<double2>();
        it.gacc = s->d_gacc.as<double>();
        it.f_out = out_device[i].f;
        it.P.n_atoms = s->n_atoms;
        it.P.xyz_conv = s->xyz_conv;
        std::copy(s->Minv, s->Minv + 9, it.P.Minv);
        std::copy(s->A6, s->A6 + 36, it.P.A6);
        it.P.want_xyz = (flags & DSF_D_XYZ) != 0;
        it.P.want_adp = (flags & DSF_D_ADP) != 0;
        it.P.want_occ = (flags & DSF_D_OCC) != 0;
        it.P.want_mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
        it.want_grad = (flags & (DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC | DSF_D_MULTIPOLE)) != 0;
        it.perm = s->d_perm.as<int>();
        it.adpk = s->d_atom_adpk.as<int>();
        it.plm_lmax = s->d_plm_lmax.as<int>();
        it.w = s->d_w_d.as<double>();
        it.mult_w = s->d_multw.as<double>();
        it.dmat = s->d_dmat.as<double>();
        it.out = out_device[i];
    }
    static PrePostBatch PB;  // host staging of the launch parameters (copied at launch)
    static std::mutex pp_mtx;
    auto launch_prepost = [&](bool post) -> int {
        std::lock_guard<std::mutex> lock(pp_mtx);
        for (int b0 = 0; b0 < n; b0 += kPrePostItems) {
            const int m = std::min(kPrePostItems, n - b0);
            PB.n = m;
            int longest = 1;
            for (int k = 0; k < m; k++) {
                PB.item[k] = pp[b0 + k];
                longest = std::max(longest, std::max(pp[b0 + k].n_hkl, pp[b0 + k].n_atoms * (post ? 1 : kNch)));
            }
            const dim3 grid(std::min((longest + 255) / 256, 512), m);
            if (post) batch_post_kernel<<<grid, 256, 0, st>>>(PB);
            else batch_pre_kernel<<<grid, 256, 0, st>>>(PB);
            DSF_CUDA(cudaGetLastError());
            launches++;
        }
        return DSF_OK;
    };
    if ((rc = launch_prepost(false))) return rc;
    // group the batched items by kernel shape and sign table; the reflection
    // chunks are chosen per launch (below) so that each launch covers the SMs
    // about eight times
    struct Group {
        int model, aniso, n_sym, coset;
        bool inv;
        SignTable G;
        size_t smem = 0;
        std::vector<SfBatchItem> items;
    };
    std::vector<Group> groups;
    for (int i = 0; i < n; i++) {
        dsf_structure *s = structures[i];
        const bool mp = (flags & DSF_D_MULTIPOLE) && s->model == MODEL_HC;
        CallBuffers C;
        SfLaunch L;
        SignTable G;
        call_buffers(s, fp64, C, L, G);
        for (int kind = 0; kind < 2; kind++) {
            int nt, n_chunks;
            size_t smem;
            // per-structure launches size their chunks as dsf_calculate_device does
            const int ntk = kind ? s->n_tiles - s->n_tiles_plain : s->n_tiles_plain;
            const int n_chunks0 = chunk_count(e, ntk, s->n_hkl);
            const double own_terms = (double)kTileAtoms * ((s->n_hkl + n_chunks0 - 1) / n_chunks0);
            if ((rc = kind_shape(s, kind, fp64, mp, own_terms, L, nt, n_chunks, smem))) return rc;
            if (nt <= 0) continue;
            if (fp64 || mp) {  // per-structure launch
                K3Args A;
                A.S = &s->dev;
                A.C = &C;
                A.L = &L;
                A.G = &G;
                A.n_sym = s->n_sym;
                A.coset = L.coset;
                A.pattern = wht_pattern_of(G, s->n_sym, L.coset, s->model == MODEL_HC);
                A.n_tiles = nt;
                A.n_chunks = n_chunks;
                A.smem = smem;
                A.st = st;
                DSF_CUDA(launch_sf3(A, s->model, fp64, mp, kind == 1));
                launches++;
                continue;
            }
            Group *g = nullptr;
            for (auto &x : groups)
                if (x.model == s->model && x.aniso == kind && x.n_sym == s->n_sym && x.coset == L.coset &&
                    x.inv == inv_kernel(s, fp64) && (L.coset == 0 || std::memcmp(&x.G, &G, sizeof(G)) == 0)) {
                    g = &x;
                    break;
                }
            if (!g) {
                groups.emplace_back();
                g = &groups.back();
                g->model = s->model;
                g->aniso = kind;
                g->n_sym = s->n_sym;
                g->coset = L.coset;
                g->inv = inv_kernel(s, fp64);
                g->G = G;
            }
            SfBatchItem it;
            it.S = s->dev;
            it.C = C;
            it.L = L;
            it.n_tiles = nt;
            g->items.push_back(it);
            g->smem = std::max(g->smem, smem);
        }
    }
    static SfBatch B;  // host staging of the launch parameters (copied at launch)
    static std::mutex mtx;
    std::lock_guard<std::mutex> lock(mtx);
    // consecutive batched launches alternate between the call's stream and the engine's side stream, so the
    // last wave of one launch overlaps the start of the next; the side stream forks from and joins the call's
    if (!e->side) {
        DSF_CUDA(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
        DSF_CUDA(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
        DSF_CUDA(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
    }
    DSF_CUDA(cudaEventRecord(e->ev_fork, st));
    DSF_CUDA(cudaStreamWaitEvent(e->side, e->ev_fork, 0));
    int lane = 0;
    for (auto &g : groups)
        for (size_t b0 = 0; b0 < g.items.size(); b0 += kBatchItems) {
            const int m = (int)std::min<size_t>(kBatchItems, g.items.size() - b0);
            B.n = m;
            // atom x reflection pairs per block for this launch: about 24 blocks per SM, so blocks of unequal
            // items even out across the SMs
            double pairs = 0;
            for (int k = 0; k < m; k++) {
                const SfBatchItem &it = g.items[b0 + k];
                pairs += (double)it.n_tiles * kTileAtoms * it.S.n_hkl;
            }
            const double block_terms = std::max<double>(kTileAtoms * 64.0, pairs / (std::max(1, e->n_sm) * 24.0));
            int blocks = 0;
            for (int k = 0; k < m; k++) {
                B.item[k] = g.items[b0 + k];
                SfLaunch &L = B.item[k].L;
                const int n_hkl = B.item[k].S.n_hkl, ht = L.ht;
                int chunk = (int)std::min<double>(n_hkl, std::max(1.0, block_terms / kTileAtoms));
                chunk = std::max(chunk, 4 * ht);
                chunk = (chunk + ht - 1) / ht * ht;
                L.hkl_chunk = chunk;
                B.block_begin[k] = blocks;
                blocks += B.item[k].n_tiles * ((n_hkl + chunk - 1) / chunk);
            }
            B.block_begin[m] = blocks;
            K3Args A;
            A.B = &B;
            A.G = &g.G;
            A.n_sym = g.n_sym;
            A.coset = g.coset;
            A.pattern = wht_pattern_of(g.G, g.n_sym, g.coset, g.model == MODEL_HC);
            A.inv = g.inv;
            A.blocks = blocks;
            A.smem = g.smem;
            A.st = (lane++ & 1) ? e->side : st;
            DSF_CUDA(launch_k3b_f32(A, g.model, g.aniso == 1));
            launches++;
        }
    DSF_CUDA(cudaEventRecord(e->ev_join, e->side));
    DSF_CUDA(cudaStreamWaitEvent(st, e->ev_join, 0));
    if ((rc = launch_prepost(true))) return rc;
    for (int i = 0; i < n; i++) structures[i]->last_launches = launches;
    return DSF_OK;
}

// host-buffer calls, staged through one pinned buffer per structure
struct HostCall {
    dsf_outputs d;      // device output block
    double *po = nullptr;
    int *pk = nullptr;
    double *raw = nullptr, *pg = nullptr;  // pinned staging of the atoms and of dT/dF
    size_t nf = 0, nout = 0;
};

// a host-buffer call in phases: checks and buffers (host_begin), the CPU copies into pinned staging
// (host_fill: no CUDA calls, thread-safe per structure), the asynchronous uploads and the atom conversion
// (host_send), then after the kernels the readback (host_readback), the status (host_status) and the
// copy-out (host_copy_out: no CUDA calls, thread-safe per structure)
static int host_begin(dsf_structure *s, const double *xyz, const double *occ, const double *dtdf, const int *include,
                      const dsf_outputs *out, HostCall &hc)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (!s->have_hkl) return fail(e, DSF_ERR_STATE, "no reflections set");
    if (s->pending) return fail(e, DSF_ERR_STATE, "a submitted call of this structure is still pending (dsf_poll)");
    if (!out || (s->n_hkl > 0 && (!out->f || !dtdf))) return fail(e, DSF_ERR_ARGUMENT, "dtdf and f are required");
    if ((xyz != nullptr) != (occ != nullptr)) return fail(e, DSF_ERR_ARGUMENT, "xyz and occupancy go together");
    cudaSetDevice(e->device);
    const int n_hkl = s->n_hkl, n = s->n_atoms;
    // inclusion mask (countAtomContribution)
    bool changed = false;
    for (int a = 0; a < n; a++) {
        const uint8_t v = include ? (include[s->perm[a]] != 0) : 1;
        if (v != s->active_host[a]) { s->active_host[a] = v; changed = true; }
    }
    if (changed)
        DSF_CUDA(cudaMemcpyAsync(s->d_active.p, s->active_host.data(), n, cudaMemcpyHostToDevice, e->stream));
    // device output block: f, xyz, adp, occ, pval, plm, kappa, kappa'
    const size_t nf = 2 * (size_t)n_hkl, per_atom = 3 + 6 + 1 + 1 + 25 + 1 + 1;
    const size_t nout = nf + per_atom * (size_t)n;
    DSF_CUDA(s->d_out.alloc(sizeof(double) * nout));
    // pinned staging: [raw atoms 10 n][dtdf 2 n_hkl][outputs nout][status]
    const size_t nin = 10 * (size_t)n + 2 * (size_t)n_hkl;
    const size_t stage_bytes = sizeof(double) * (nin + nout) + 16;
    if (s->pinned_bytes < stage_bytes) {
        if (s->pinned) cudaFreeHost(s->pinned);
        s->pinned = nullptr;
        s->pinned_bytes = 0;
        DSF_CUDA(cudaHostAlloc(&s->pinned, stage_bytes, cudaHostAllocDefault));
        s->pinned_bytes = stage_bytes;
    }
    hc.raw = (double *)s->pinned;
    hc.pg = hc.raw + 10 * (size_t)n;
    hc.po = hc.pg + 2 * (size_t)n_hkl;
    hc.pk = (int *)(hc.po + nout);
    hc.nf = nf;
    hc.nout = nout;
    double *base = s->d_out.as<double>();
    dsf_outputs &d = hc.d;
    d.f = base;
    d.d_xyz = base + nf;
    d.d_adp = d.d_xyz + 3 * (size_t)n;
    d.d_occ = d.d_adp + 6 * (size_t)n;
    d.d_pval = d.d_occ + n;
    d.d_plm = d.d_pval + n;
    d.d_kappa = d.d_plm + 25 * (size_t)n;
    d.d_kappa_prime = d.d_kappa + n;
    return DSF_OK;
}

// 0, or 1 with a non-finite coordinate
static int host_fill(const dsf_structure *s, const double *xyz, const double *adp, const double *occ,
                     const double *dtdf, const HostCall &hc)
{
    const int n = s->n_atoms;
    if (xyz) {
        double *raw = hc.raw;
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < 3; j++) {
                if (!std::isfinite(xyz[3 * i + j])) return 1;
                raw[10 * i + j] = xyz[3 * i + j];
            }
            for (int j = 0; j < 6; j++) raw[10 * i + 3 + j] = (adp && j < s->adpk[i]) ? adp[6 * i + j] : 0.0;
            raw[10 * i + 9] = occ[i];
        }
    }
    if (s->n_hkl > 0) std::memcpy(hc.pg, dtdf, sizeof(double) * 2 * (size_t)s->n_hkl);
    return 0;
}

static int host_send(dsf_structure *s, bool atoms, const HostCall &hc)
{
    dsf_engine *e = s->eng;
    const int n = s->n_atoms, n_hkl = s->n_hkl;
    if (atoms) {
        DSF_CUDA(cudaMemcpyAsync(s->d_raw.p, hc.raw, sizeof(double) * 10 * (size_t)n, cudaMemcpyHostToDevice,
                                 e->stream));
        AtomParams P;
        P.n_atoms = n;
        P.xyz_conv = s->xyz_conv;
        std::copy(s->Minv, s->Minv + 9, P.Minv);
        std::copy(s->A6, s->A6 + 36, P.A6);
        atom_convert_kernel<<<(n + 127) / 128, 128, 0, e->stream>>>(
            P, s->d_raw.as<double>(), s->d_perm.as<int>(), s->d_atom_adpk.as<int>(), s->d_multw.as<double>(),
            s->d_xq.as<uint32_t>(), s->d_xlo.as<float>(), s->d_xd.as<double>(), s->d_adp_f.as<float>(),
            s->d_adp_d.as<double>(), s->d_w_f.as<float>(), s->d_w_d.as<double>(), s->n_sym, s->d_sym_rot.as<int>(),
            s->d_sym_t24.as<int>(), s->d_step_f.as<float2>(), s->d_step_d.as<double2>());
        DSF_CUDA(cudaGetLastError());
        s->have_atoms = true;
    }
    if (n_hkl > 0)
        DSF_CUDA(cudaMemcpyAsync(s->d_dtdf.p, hc.pg, 16 * (size_t)n_hkl, cudaMemcpyHostToDevice, e->stream));
    return DSF_OK;
}

static int host_stage(dsf_structure *s, const double *xyz, const double *adp, const double *occ,
                      const double *dtdf, const int *include, const dsf_outputs *out, HostCall &hc)
{
    int rc = host_begin(s, xyz, occ, dtdf, include, out, hc);
    if (rc) return rc;
    if (host_fill(s, xyz, adp, occ, dtdf, hc)) return fail(s->eng, DSF_ERR_ARGUMENT, "non-finite coordinate");
    return host_send(s, xyz != nullptr, hc);
}

static int host_readback(dsf_structure *s, int flags, HostCall &hc)
{
    dsf_engine *e = s->eng;
    const bool mp = (flags & DSF_D_MULTIPOLE) != 0;
    const size_t nback = mp ? hc.nout : hc.nf + 10 * (size_t)s->n_atoms;  // f, xyz, adp, occ (+ multipole block)
    DSF_CUDA(cudaMemcpyAsync(hc.po, hc.d.f, sizeof(double) * nback, cudaMemcpyDeviceToHost, e->stream));
    DSF_CUDA(cudaMemcpyAsync(hc.pk, s->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    return DSF_OK;
}

// a timed-out kernel wait of the call (DSF_ERR_TIMEOUT), after the stream synchronisation
static int host_status(dsf_structure *s, const HostCall &hc)
{
    if (*hc.pk) {
        cudaMemsetAsync(s->d_err.p, 0, sizeof(int), s->eng->stream);
        return fail(s->eng, DSF_ERR_TIMEOUT, "a shared-memory pipeline wait of the kernel ran out");
    }
    return DSF_OK;
}

// copy-out of the pinned results (no CUDA calls, thread-safe per structure);
// derivative outputs that the flags do not ask for are left as the caller had them
static void host_copy_out(const dsf_structure *s, int flags, const HostCall &hc, const dsf_outputs *out)
{
    const int n = s->n_atoms;
    const int mp = s->model == MODEL_HC ? DSF_D_MULTIPOLE : 0;
    if (hc.nf) std::memcpy(out->f, hc.po, sizeof(double) * hc.nf);
    const double *q = hc.po + hc.nf;
    struct { double *dst; size_t off, n; int flag; } cp[] = {
        {out->d_xyz, 0, 3 * (size_t)n, DSF_D_XYZ}, {out->d_adp, 3 * (size_t)n, 6 * (size_t)n, DSF_D_ADP},
        {out->d_occ, 9 * (size_t)n, (size_t)n, DSF_D_OCC}, {out->d_pval, 10 * (size_t)n, (size_t)n, mp},
        {out->d_plm, 11 * (size_t)n, 25 * (size_t)n, mp}, {out->d_kappa, 36 * (size_t)n, (size_t)n, mp},
        {out->d_kappa_prime, 37 * (size_t)n, (size_t)n, mp}};
    for (auto &c : cp)
        if (c.dst && (flags & c.flag)) std::memcpy(c.dst, q + c.off, sizeof(double) * c.n);
}

static int calculate_host(dsf_structure *s, int precision, int flags, const double *xyz, const double *adp,
                          const double *occ, const double *dtdf, const int *include, const dsf_outputs *out)
{
    HostCall hc;
    int rc = host_stage(s, xyz, adp, occ, dtdf, include, out, hc);
    if (rc) return rc;
    dsf_engine *e = s->eng;
    if ((rc = dsf_calculate_device(s, precision, flags, s->d_dtdf.as<double>(), &hc.d, e->stream))) return rc;
    if ((rc = host_readback(s, flags, hc))) return rc;
    DSF_CUDA(cudaStreamSynchronize(e->stream));
    if ((rc = host_status(s, hc))) return rc;
    host_copy_out(s, flags, hc, out);
    return DSF_OK;
}

// an asynchronous host-buffer call (dsf_submit / dsf_poll)
struct dsf_ticket {
    dsf_structure *s = nullptr;
    int flags = 0;
    HostCall hc;
    dsf_outputs out{};
    cudaEvent_t done = nullptr;
};

int dsf_submit(dsf_structure *s, int precision, int flags, const double *xyz, const double *adp,
               const double *occupancy, const double *dtdf, const int *include, const dsf_outputs *out,
               dsf_ticket **ticket)
{
    if (!s || !ticket || !out) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    *ticket = nullptr;
    auto *t = new dsf_ticket;
    int rc = host_stage(s, xyz, adp, occupancy, dtdf, include, out, t->hc);
    if (!rc) rc = dsf_calculate_device(s, precision, flags, s->d_dtdf.as<double>(), &t->hc.d, e->stream);
    if (!rc) rc = host_readback(s, flags, t->hc);
    if (!rc && (cudaEventCreateWithFlags(&t->done, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventRecord(t->done, e->stream) != cudaSuccess))
        rc = fail(e, DSF_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    if (rc) {
        if (t->done) cudaEventDestroy(t->done);
        delete t;
        return rc;
    }
    t->s = s;
    t->flags = flags;
    t->out = *out;
    s->pending = 1;
    *ticket = t;
    return DSF_OK;
}

int dsf_poll(dsf_ticket *t, int timeout_ms)
{
    if (!t) return DSF_ERR_ARGUMENT;
    dsf_structure *s = t->s;
    cudaSetDevice(s->eng->device);
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = cudaEventQuery(t->done);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) {  // the call failed on the device: release the ticket, report
            s->pending = 0;
            cudaEventDestroy(t->done);
            delete t;
            return fail(s->eng, DSF_ERR_CUDA, cudaGetErrorString(q));
        }
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (ms >= timeout_ms) return DSF_PENDING;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    int rc = host_status(s, t->hc);
    if (!rc) host_copy_out(s, t->flags, t->hc, &t->out);
    s->pending = 0;
    cudaEventDestroy(t->done);
    delete t;
    return rc;
}

int dsf_reduce_to_types(dsf_structure *s, const dsf_outputs *per_atom, const dsf_outputs *per_type, void *stream)
{
    if (!s || !per_atom || !per_type) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (s->model != MODEL_HC) return fail(e, DSF_ERR_STATE, "multipole parameters exist only for HC structures");
    cudaSetDevice(e->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    const int nT = s->n_types, n = s->n_atoms;
    if (per_type->d_pval) DSF_CUDA(cudaMemsetAsync(per_type->d_pval, 0, sizeof(double) * nT, st));
    if (per_type->d_plm) DSF_CUDA(cudaMemsetAsync(per_type->d_plm, 0, sizeof(double) * 25 * (size_t)nT, st));
    if (per_type->d_kappa) DSF_CUDA(cudaMemsetAsync(per_type->d_kappa, 0, sizeof(double) * nT, st));
    if (per_type->d_kappa_prime) DSF_CUDA(cudaMemsetAsync(per_type->d_kappa_prime, 0, sizeof(double) * nT, st));
    type_reduce_kernel<<<(n * 28 + 255) / 256, 256, 0, st>>>(n, nT, s->d_atom_type0.as<int>(), per_atom->d_pval,
                                                            per_atom->d_plm, per_atom->d_kappa,
                                                            per_atom->d_kappa_prime, per_type->d_pval,
                                                            per_type->d_plm, per_type->d_kappa,
                                                            per_type->d_kappa_prime);
    DSF_CUDA(cudaGetLastError());
    return DSF_OK;
}

int dsf_structure_set_anomalous(dsf_structure *s, const double *anomalous)
{
    if (!s) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (!anomalous) return fail(e, DSF_ERR_ARGUMENT, "anomalous dispersion [n_atoms][2] is required");
    const int n = s->n_atoms;
    std::vector<double> an_d(2 * (size_t)n);
    std::vector<float> an_f(2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < 2; k++) {
            if (!std::isfinite(anomalous[2 * i + k])) return fail(e, DSF_ERR_ARGUMENT, "non-finite anomalous dispersion");
            s->anom[2 * i + k] = anomalous[2 * i + k];
        }
    }
    for (int i = 0; i < n; i++) {  // engine (sorted) order
        const int o = s->perm[i];
        an_d[2 * i] = s->anom[2 * o];
        an_d[2 * i + 1] = s->anom[2 * o + 1];
        an_f[2 * i] = (float)an_d[2 * i];
        an_f[2 * i + 1] = (float)an_d[2 * i + 1];
    }
    cudaSetDevice(e->device);
    DSF_CUDA(cudaStreamSynchronize(e->stream));  // no call of the engine's stream still reads the old values
    int rc;
    if ((rc = upload(e, s->d_anom_d, an_d.data(), an_d.size()))) return rc;
    if ((rc = upload(e, s->d_anom_f, an_f.data(), an_f.size()))) return rc;
    DSF_CUDA(cudaStreamSynchronize(e->setup));
    return DSF_OK;
}

int dsf_debug_stall_next_call(dsf_structure *s)
{
    if (!s) return DSF_ERR_ARGUMENT;
    s->debug_stall = 1;
    return DSF_OK;
}

int dsf_form_factors(dsf_structure *s, const int *hkl, const int *include, double *ff)
{
    if (!s || !hkl || !ff) return DSF_ERR_ARGUMENT;
    dsf_engine *e = s->eng;
    if (s->model == MODEL_TABLE)
        return fail(e, DSF_ERR_UNSUPPORTED, "form factors at one reflection: HC and IAM structures only");
    cudaSetDevice(e->device);
    const int n = s->n_atoms;
    double hc[3];
    for (int j = 0; j < 3; j++) hc[j] = s->B[3 * j] * hkl[0] + s->B[3 * j + 1] * hkl[1] + s->B[3 * j + 2] * hkl[2];
    struct Scratch {  // per call (not hot): freed on every return path
        DevBuf inc, ff;
        ~Scratch() { inc.release(); ff.release(); }
    } sc;
    DevBuf &d_inc = sc.inc, &d_ff = sc.ff;
    if (include) {
        DSF_CUDA(d_inc.alloc(sizeof(int) * (size_t)n));
        DSF_CUDA(cudaMemcpyAsync(d_inc.p, include, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, e->stream));
    }
    DSF_CUDA(d_ff.alloc(sizeof(double2) * (size_t)n));
    DSF_CUDA(launch_form_factors(s->dev, hc, include ? d_inc.as<int>() : nullptr, d_ff.as<double2>(), e->stream));
    DSF_CUDA(cudaMemcpyAsync(ff, d_ff.p, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost, e->stream));
    DSF_CUDA(cudaStreamSynchronize(e->stream));
    return DSF_OK;
}

int dsf_calculate_batch(dsf_structure *const *structures, int n, int precision, int flags,
                        const double *const *dtdf, const int *const *include, const dsf_outputs *out)
{
    return dsf_calculate_batch_atoms(structures, n, precision, flags, nullptr, nullptr, nullptr, dtdf, include, out);
}

int dsf_calculate_batch_atoms(dsf_structure *const *structures, int n, int precision, int flags,
                              const double *const *xyz, const double *const *adp, const double *const *occupancy,
                              const double *const *dtdf, const int *const *include, const dsf_outputs *out)
{
    if (!structures || n < 1 || !dtdf || !out || !structures[0]) return DSF_ERR_ARGUMENT;
    dsf_engine *e = structures[0]->eng;
    std::vector<HostCall> hc(n);
    std::vector<dsf_outputs> d(n);
    std::vector<const double *> g(n);
    std::vector<size_t> io(n);
    std::vector<double> work(n);
    size_t bytes_io = 0;
    double total = 0;
    for (int i = 0; i < n; i++) {
        if (!structures[i] || structures[i]->eng != e)
            return fail(e, DSF_ERR_ARGUMENT, "batch structures must belong to one engine");
        int rc = host_begin(structures[i], xyz ? xyz[i] : nullptr, occupancy ? occupancy[i] : nullptr, dtdf[i],
                            include ? include[i] : nullptr, &out[i], hc[i]);
        if (rc) return rc;
        io[i] = 16 * (size_t)structures[i]->n_hkl + (xyz ? 80 * (size_t)structures[i]->n_atoms : 0) + 8 * hc[i].nout;
        bytes_io += io[i];
        work[i] = (double)structures[i]->n_atoms * structures[i]->n_hkl * structures[i]->n_sym + 1.0;
        total += work[i];
        d[i] = hc[i].d;
        g[i] = structures[i]->d_dtdf.as<double>();
    }
    // Large batches run as groups of consecutive structures of about equal work:
    // while the GPU computes one group, the CPU copies the next group's inputs into
    // pinned staging and the previous group's results out of it.
    const int n_groups = (bytes_io >= kPipelineBytes && n >= 8) ? std::min(kPipelineGroups, n / 4) : 1;
    std::vector<int> gb(n_groups + 1, n);
    gb[0] = 0;
    {
        double acc = 0;
        int k = 1;
        for (int i = 0; i < n && k < n_groups; i++) {
            acc += work[i];
            if (acc >= total * k / n_groups) gb[k++] = i + 1;
        }
    }
    struct Events {  // one completion event per group, destroyed on every return path
        std::vector<cudaEvent_t> ev;
        ~Events()
        {
            for (cudaEvent_t x : ev)
                if (x) cudaEventDestroy(x);
        }
    } evs;
    evs.ev.assign(n_groups, nullptr);
    cudaSetDevice(e->device);
    auto group_bytes = [&](int k) {
        size_t b = 0;
        for (int i = gb[k]; i < gb[k + 1]; i++) b += io[i];
        return b;
    };
    // inputs in, the group's calculation and its read-back enqueued, the event recorded
    auto stage = [&](int k) -> int {
        const int i0 = gb[k], m = gb[k + 1] - gb[k];
        std::vector<int> bad(m, 0);
        host_parallel(m, group_bytes(k), [&](int j) {
            const int i = i0 + j;
            bad[j] = host_fill(structures[i], xyz ? xyz[i] : nullptr, adp ? adp[i] : nullptr,
                               occupancy ? occupancy[i] : nullptr, dtdf[i], hc[i]);
        });
        for (int j = 0; j < m; j++)
            if (bad[j]) return fail(e, DSF_ERR_ARGUMENT, "non-finite coordinate");
        int rc;
        for (int i = i0; i < i0 + m; i++)
            if ((rc = host_send(structures[i], xyz != nullptr && xyz[i] != nullptr, hc[i]))) return rc;
        if ((rc = dsf_calculate_batch_device(structures + i0, m, precision, flags, g.data() + i0, d.data() + i0,
                                             e->stream)))
            return rc;
        for (int i = i0; i < i0 + m; i++)
            if ((rc = host_readback(structures[i], flags, hc[i]))) return rc;
        DSF_CUDA(cudaEventCreateWithFlags(&evs.ev[k], cudaEventDisableTiming));
        DSF_CUDA(cudaEventRecord(evs.ev[k], e->stream));
        return DSF_OK;
    };
    // the group's results out of pinned staging, after its event
    auto finish = [&](int k) -> int {
        DSF_CUDA(cudaEventSynchronize(evs.ev[k]));
        int rc;
        for (int i = gb[k]; i < gb[k + 1]; i++)
            if ((rc = host_status(structures[i], hc[i]))) return rc;
        const int i0 = gb[k];
        host_parallel(gb[k + 1] - i0, group_bytes(k),
                      [&](int j) { host_copy_out(structures[i0 + j], flags, hc[i0 + j], &out[i0 + j]); });
        return DSF_OK;
    };
    int rc = DSF_OK, prev = -1;
    for (int k = 0; k < n_groups && !rc; k++) {
        if (gb[k] == gb[k + 1]) continue;
        rc = stage(k);
        if (!rc && prev >= 0) rc = finish(prev);
        prev = k;
    }
    if (!rc && prev >= 0) rc = finish(prev);
    if (rc) cudaStreamSynchronize(e->stream);  // no copy of a failed call still in flight
    return rc;
}

int dsf_calculate(dsf_structure *s, int precision, int flags, const double *dtdf, const int *include,
                  const dsf_outputs *out)
{
    return calculate_host(s, precision, flags, nullptr, nullptr, nullptr, dtdf, include, out);
}

int dsf_calculate_atoms(dsf_structure *s, int precision, int flags, const double *xyz, const double *adp,
                        const double *occupancy, const double *dtdf, const int *include, const dsf_outputs *out)
{
    if (s && (!xyz || !occupancy)) return fail(s->eng, DSF_ERR_ARGUMENT, "xyz and occupancy are required");
    return calculate_host(s, precision, flags, xyz, adp, occupancy, dtdf, include, out);
}

}  // extern "C"
