// Allocation-free IAM structure factors + derivatives.
//
// For callers that cannot allocate device memory: code running inside a
// host framework that owns every device allocation through its own pool (a
// refinement program embedding this library), or a caller that must not
// trigger allocation (and the device-wide synchronisation cudaMalloc/cudaFree
// can bring) inside its per-cycle loop.  The caller passes every input and
// output as its own device buffer; the scratch the calculation needs
// (converted atom parameters, per-reflection tables, the FP64 accumulators
// of the cross-block sums) lives in one file-scope __device__ array of
// DSF_NOALLOC_SCRATCH_BYTES that every GPU which loads this library holds
// until the process exits.  The call launches the same kernels as
// dsf_calculate_device on that scratch and allocates nothing.
//
// The first call on a device looks up the array's device address
// (cudaGetSymbolAddress, once per device, with that device current).  Under
// CUDA's lazy module loading that lookup is also what loads this file's
// module and places the array on the GPU, so the first call can fail with
// DSF_ERR_CUDA (out of memory); make it during set-up, before any stream
// capture.  The address is kept per device ordinal for the life of the
// process: after cudaDeviceReset of a device this call must not be used on
// that device again.  All calls share the array: calls that overlap on the
// GPU (different streams, or different host threads) race on it and must be
// serialised by the caller.
//
// It runs the first-generation kernel of the engine (sf_grad_kernel: the
// per-block reflection tables in shared memory, no line recurrences, no
// sign-diagonal cosets), several times slower than dsf_calculate_device.
// Atoms whose type index lies outside 0..n_types-1 contribute nothing;
// adp_components other than 1 or 6 mean no temperature factor.
#include "../../include/dsf_gb300.h"
#include "dsf_device.cuh"
#include "dsf_math.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace dsf {
cudaError_t launch_sf_grad(const DevStructure &S, const CallBuffers &C, bool fp64, bool mp, int hkl_chunk, int ht,
                           cudaStream_t st);
size_t sf_grad_smem_bytes(bool fp64, int ht, int n_sym);
void host_cell_matrices(const double *cell, double *M, double *Minv, double *B);
void host_adp_param_map(const double *A, double *A6);
cudaError_t launch_adjoint_weights(int n, const double2 *dtdf, const double *mult, const double2 *cinv, int centro,
                                   double2 *gw_d, float2 *gw_f, cudaStream_t st);
cudaError_t launch_f_epilogue(int n, const double2 *facc, const double *mult, const double2 *cinv, int centro,
                              double *f_out, cudaStream_t st);
cudaError_t launch_grad_epilogue(int n_atoms, int xyz_conv, const double *Minv, const double *A6, int flags,
                                 const double *g_acc, const int *perm, const int *adpk, const double *w,
                                 const double *mult_w, const dsf_outputs *out, cudaStream_t st);
}  // namespace dsf

using namespace dsf;

static __device__ __align__(256) unsigned char g_noalloc_scratch[DSF_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
unsigned char *g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

int report(char *err, int err_len, int code, const char *msg)
{
    if (err && err_len > 0) {
        std::strncpy(err, msg, (size_t)err_len - 1);
        err[err_len - 1] = '\0';
    }
    return code;
}

// small host tables passed by value to the set-up kernel
struct SetupParams {
    int n_sym, n_types, n_atoms, n_tiles;
    int rot[kMaxSym * 9];
    int t24[kMaxSym * 3];
    TypeRadialT<float> tf[DSF_NOALLOC_MAX_TYPES];
    TypeRadialT<double> td[DSF_NOALLOC_MAX_TYPES];
};

struct Layout {
    size_t off = 0;
    template <typename T>
    size_t take(size_t n)
    {
        const size_t o = off;
        off = (off + sizeof(T) * std::max<size_t>(n, 1) + 255) & ~(size_t)255;
        return o;
    }
};

struct Scratch {
    int *sym_rot, *sym_t24, *tile_begin, *tile_ntypes, *tile_types;
    TypeRadialT<float> *types_f;
    TypeRadialT<double> *types_d;
    uint32_t *xq;
    float *xlo, *adp_f, *w_f;
    double *xd, *adp_d, *w_d, *multw, *g_acc;
    float2 *anom_f;
    double2 *anom_d;
    uint8_t *active;
    int *ltype, *adpk, *perm;
    int4 *hkl;
    double *h2, *mult;
    float *h2f;
    double2 *cinv, *gw_d, *f_acc;
    float2 *gw_f;
    size_t bytes;
};

Scratch carve(unsigned char *base, int n_atoms, int n_hkl, int n_sym, int n_types, int n_tiles)
{
    Layout L;
    const size_t na = (size_t)n_atoms, nh = (size_t)n_hkl;
    const size_t o_rot = L.take<int>(9 * (size_t)n_sym), o_t24 = L.take<int>(3 * (size_t)n_sym);
    const size_t o_tb = L.take<int>(n_tiles + 1), o_tn = L.take<int>(n_tiles);
    const size_t o_tt = L.take<int>((size_t)n_tiles * kMaxTileTypes);
    const size_t o_tf = L.take<TypeRadialT<float> >(n_types), o_td = L.take<TypeRadialT<double> >(n_types);
    const size_t o_xq = L.take<uint32_t>(3 * na), o_xlo = L.take<float>(3 * na), o_xd = L.take<double>(3 * na);
    const size_t o_af = L.take<float>(6 * na), o_ad = L.take<double>(6 * na);
    const size_t o_wf = L.take<float>(na), o_wd = L.take<double>(na), o_mw = L.take<double>(na);
    const size_t o_anf = L.take<float2>(na), o_and = L.take<double2>(na), o_act = L.take<uint8_t>(na);
    const size_t o_lt = L.take<int>(na), o_k = L.take<int>(na), o_p = L.take<int>(na);
    const size_t o_g = L.take<double>((size_t)kNch * na);
    const size_t o_hkl = L.take<int4>(nh), o_h2 = L.take<double>(nh), o_h2f = L.take<float>(nh);
    const size_t o_m = L.take<double>(nh), o_c = L.take<double2>(nh), o_gd = L.take<double2>(nh);
    const size_t o_gf = L.take<float2>(nh), o_fa = L.take<double2>(nh);
    Scratch s;
    s.bytes = L.off;
    s.sym_rot = (int *)(base + o_rot);
    s.sym_t24 = (int *)(base + o_t24);
    s.tile_begin = (int *)(base + o_tb);
    s.tile_ntypes = (int *)(base + o_tn);
    s.tile_types = (int *)(base + o_tt);
    s.types_f = (TypeRadialT<float> *)(base + o_tf);
    s.types_d = (TypeRadialT<double> *)(base + o_td);
    s.xq = (uint32_t *)(base + o_xq);
    s.xlo = (float *)(base + o_xlo);
    s.xd = (double *)(base + o_xd);
    s.adp_f = (float *)(base + o_af);
    s.adp_d = (double *)(base + o_ad);
    s.w_f = (float *)(base + o_wf);
    s.w_d = (double *)(base + o_wd);
    s.multw = (double *)(base + o_mw);
    s.anom_f = (float2 *)(base + o_anf);
    s.anom_d = (double2 *)(base + o_and);
    s.active = (uint8_t *)(base + o_act);
    s.ltype = (int *)(base + o_lt);
    s.adpk = (int *)(base + o_k);
    s.perm = (int *)(base + o_p);
    s.g_acc = (double *)(base + o_g);
    s.hkl = (int4 *)(base + o_hkl);
    s.h2 = (double *)(base + o_h2);
    s.h2f = (float *)(base + o_h2f);
    s.mult = (double *)(base + o_m);
    s.cinv = (double2 *)(base + o_c);
    s.gw_d = (double2 *)(base + o_gd);
    s.gw_f = (float2 *)(base + o_gf);
    s.f_acc = (double2 *)(base + o_fa);
    return s;
}

__global__ void noalloc_setup_kernel(SetupParams P, Scratch S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.n_sym * 9) S.sym_rot[i] = P.rot[i];
    if (i < P.n_sym * 3) S.sym_t24[i] = P.t24[i];
    if (i < P.n_types) {
        S.types_f[i] = P.tf[i];
        S.types_d[i] = P.td[i];
    }
    if (i <= P.n_tiles) S.tile_begin[i] = min(i * kTileAtoms, P.n_atoms);
    if (i < P.n_tiles) {
        S.tile_ntypes[i] = P.n_types;
        for (int t = 0; t < kMaxTileTypes; t++) S.tile_types[i * kMaxTileTypes + t] = t < P.n_types ? t : 0;
    }
}

struct AtomIn {
    int n_atoms, n_total, n_types;
    double A6[36];
    const int *type, *adpk;
    const double *xyz, *adp, *occ, *mult, *anom;
};

// caller atoms (fractional xyz, U_cif) -> the kernel's representation (identity order)
__global__ void noalloc_atoms_kernel(AtomIn P, Scratch S)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= P.n_atoms) return;
    for (int i = 0; i < 3; i++) {
        const double x = P.xyz[3 * a + i];
        S.xd[3 * a + i] = x;
        const double xr = x - floor(x);
        const double q = rint(xr * 4294967296.0);
        S.xlo[3 * a + i] = (float)(xr - q * (1.0 / 4294967296.0));
        S.xq[3 * a + i] = (uint32_t)(unsigned long long)q;
    }
    const int k = P.adpk[a];
    const double two_pi2 = 2.0 * DSF_PI * DSF_PI, log2e = 1.4426950408889634;
    for (int i = 0; i < 6; i++) {
        S.adp_d[6 * a + i] = 0.0;
        S.adp_f[6 * a + i] = 0.0f;
    }
    if (k == 1) {
        S.adp_d[6 * a] = two_pi2 * P.adp[6 * a];
        S.adp_f[6 * a] = (float)(two_pi2 * P.adp[6 * a] * log2e);
    } else if (k == 6) {
        for (int p = 0; p < 6; p++) {
            double s = 0;
            for (int q = 0; q < 6; q++) s += P.A6[6 * p + q] * P.adp[6 * a + q];
            S.adp_d[6 * a + p] = two_pi2 * s;
            S.adp_f[6 * a + p] = (float)(two_pi2 * s * log2e);
        }
    }
    const double mw = P.mult[a] / (double)P.n_total;
    const double w = P.occ[a] * mw;
    S.multw[a] = mw;
    S.w_d[a] = w;
    S.w_f[a] = (float)w;
    const double are = P.anom ? P.anom[2 * a] : 0.0, aim = P.anom ? P.anom[2 * a + 1] : 0.0;
    S.anom_d[a] = make_double2(are, aim);
    S.anom_f[a] = make_float2((float)are, (float)aim);
    // an atom whose type index is out of range contributes nothing
    const int t = P.type[a];
    const bool ok = t >= 0 && t < P.n_types;
    S.active[a] = ok ? 1 : 0;
    S.ltype[a] = ok ? t : 0;
    S.adpk[a] = k;
    S.perm[a] = a;
}

struct HklIn {
    int n_hkl;
    double B[9];
    char centering;
    int obverse;
    int t_inv24[3];
    const int *hkl;
};

__device__ double centering_mult(char c, int obverse, int h, int k, int l)
{
    switch (c) {
    // reverse setting: (h - k + l) mod 2, as the reference and the allocating path test it
    case 'R':
        if (obverse) return (abs(-h + k + l) % 3 == 0) ? 3.0 : 0.0;
        return (abs(h - k + l) % 2 == 0) ? 3.0 : 0.0;
    case 'F': {
        const int a = abs(h % 2), b = abs(k % 2), d = abs(l % 2);
        return (a == b && a == d) ? 4.0 : 0.0;
    }
    case 'I': return ((h + k + l) % 2 == 0) ? 2.0 : 0.0;
    case 'A': return ((k + l) % 2 == 0) ? 2.0 : 0.0;
    case 'B': return ((h + l) % 2 == 0) ? 2.0 : 0.0;
    case 'C': return ((h + k) % 2 == 0) ? 2.0 : 0.0;
    default: return 1.0;
    }
}

__global__ void noalloc_hkl_kernel(HklIn P, Scratch S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n_hkl) return;
    const int h = P.hkl[3 * i], k = P.hkl[3 * i + 1], l = P.hkl[3 * i + 2];
    S.hkl[i] = make_int4(h, k, l, 0);
    double c[3];
    for (int j = 0; j < 3; j++) c[j] = P.B[3 * j] * h + P.B[3 * j + 1] * k + P.B[3 * j + 2] * l;
    const double h2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    S.h2[i] = h2;
    S.h2f[i] = (float)h2;
    S.mult[i] = centering_mult(P.centering, P.obverse, h, k, l);
    int r = (h * P.t_inv24[0] + k * P.t_inv24[1] + l * P.t_inv24[2]) % 24;
    if (r < 0) r += 24;
    double sn, cs;
    sincospi(r / 12.0, &sn, &cs);
    if (r % 6 == 0) {
        const int q = r / 6;
        cs = q == 0 ? 1.0 : q == 2 ? -1.0 : 0.0;
        sn = q == 1 ? 1.0 : q == 3 ? -1.0 : 0.0;
    }
    S.cinv[i] = make_double2(cs, sn);
}

unsigned char *scratch_base(int device, cudaError_t *status)
{
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (device < 0 || device >= kMaxDevices) {
        *status = cudaErrorInvalidDevice;
        return nullptr;
    }
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            *status = e;
            return nullptr;
        }
        g_scratch_addr[device] = (unsigned char *)p;
    }
    *status = cudaSuccess;
    return g_scratch_addr[device];
}

}  // namespace

extern "C" int dsf_iam_calculate_noalloc(const dsf_symmetry *sym, const dsf_iam_model *model, int n_atoms,
                                         const int *atom_type, const int *adp_components, const double *xyz,
                                         const double *adp, const double *occupancy, const double *multiplicity,
                                         const double *anomalous, int n_hkl, const int *hkl, const double *dtdf,
                                         int precision, int derivative_flags, const dsf_outputs *out, void *stream,
                                         char *err, int err_len)
{
    if (!sym || !model || !out || !out->f || !atom_type || !adp_components || !xyz || !adp || !occupancy ||
        !multiplicity || !hkl || !dtdf)
        return report(err, err_len, DSF_ERR_ARGUMENT, "missing argument");
    if (n_atoms < 1 || n_hkl < 1) return report(err, err_len, DSF_ERR_ARGUMENT, "need atoms and reflections");
    if (sym->n_symops < 1 || sym->n_symops > kMaxSym)
        return report(err, err_len, DSF_ERR_ARGUMENT, "n_symops must be in 1..48");
    // the symmetry checks of the allocating path, before anything is launched
    for (int i = 0; i < 3; i++)
        if (!(sym->cell[i] > 0)) return report(err, err_len, DSF_ERR_ARGUMENT, "cell lengths must be positive");
    const char centering = sym->centering ? (char)toupper(sym->centering) : 'P';
    if (!std::strchr("PABCIFR", centering))
        return report(err, err_len, DSF_ERR_ARGUMENT, "unsupported lattice centering");
    if (sym->centrosymmetric)
        for (int i = 0; i < 3; i++) {
            const double t = sym->inversion_translation[i] * 24.0;
            if (std::fabs(t - std::rint(t)) > 1e-6)
                return report(err, err_len, DSF_ERR_ARGUMENT, "inversion translation must be a multiple of 1/24");
        }
    if (model->n_types < 1 || model->n_types > DSF_NOALLOC_MAX_TYPES)
        return report(err, err_len, DSF_ERR_ARGUMENT, "IAM types must number 1..32 for the allocation-free call");
    if (precision != DSF_FP64 && precision != DSF_FP32_BULK)
        return report(err, err_len, DSF_ERR_ARGUMENT, "unknown precision");
    const int n_tiles = (n_atoms + kTileAtoms - 1) / kTileAtoms;
    {
        Scratch probe = carve(nullptr, n_atoms, n_hkl, sym->n_symops, model->n_types, n_tiles);
        if (probe.bytes > (size_t)DSF_NOALLOC_SCRATCH_BYTES) {
            char msg[200];
            std::snprintf(msg, sizeof msg,
                          "problem needs %zu bytes of scratch, over the %u-byte limit of the allocation-free call",
                          probe.bytes, (unsigned)DSF_NOALLOC_SCRATCH_BYTES);
            return report(err, err_len, DSF_ERR_ARGUMENT, msg);
        }
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return report(err, err_len, DSF_ERR_CUDA, "no current CUDA device");
    cudaError_t ce;
    unsigned char *base = scratch_base(device, &ce);
    if (!base) return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));
    Scratch S = carve(base, n_atoms, n_hkl, sym->n_symops, model->n_types, n_tiles);
    cudaStream_t st = (cudaStream_t)stream;

    // symmetry, cell and per-type constants on the host
    SetupParams P;
    std::memset(&P, 0, sizeof P);
    P.n_sym = sym->n_symops;
    P.n_types = model->n_types;
    P.n_atoms = n_atoms;
    P.n_tiles = n_tiles;
    for (int i = 0; i < 9 * P.n_sym; i++) P.rot[i] = sym->symop_rotation[i];
    for (int i = 0; i < 3 * P.n_sym; i++) {
        const double t = sym->symop_translation[i] * 24.0, r = std::rint(t);
        if (std::fabs(t - r) > 1e-6) return report(err, err_len, DSF_ERR_ARGUMENT, "translations must be multiples of 1/24");
        P.t24[i] = (((int)r % 24) + 24) % 24;
    }
    for (int t = 0; t < P.n_types; t++) {
        const int ng = model->n_gauss[t];
        if (ng < 0 || ng > 5) return report(err, err_len, DSF_ERR_ARGUMENT, "at most 5 Gaussians per type");
        TypeRadialT<float> &f = P.tf[t];
        TypeRadialT<double> &d = P.td[t];
        d.iam_n = f.iam_n = ng;
        for (int q = 0; q < ng; q++) {
            d.iam_a[q] = model->a[5 * t + q];
            d.iam_b[q] = model->b[5 * t + q];
            f.iam_a[q] = (float)d.iam_a[q];
            f.iam_b[q] = (float)d.iam_b[q];
        }
        d.iam_c = model->c[t];
        f.iam_c = (float)d.iam_c;
        d.inv_kappa = d.inv_kappa_p = 1.0;
        f.inv_kappa = f.inv_kappa_p = 1.0f;
    }
    double M[9], Minv[9], B[9], A6[36];
    host_cell_matrices(sym->cell, M, Minv, B);
    double A[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 3; i++) A[4 * i] = std::sqrt(B[i] * B[i] + B[3 + i] * B[3 + i] + B[6 + i] * B[6 + i]);
    host_adp_param_map(A, A6);  // U_cif -> U*

    const int setup_n = std::max(std::max(9 * P.n_sym, n_tiles + 1), P.n_types);
    noalloc_setup_kernel<<<(setup_n + 127) / 128, 128, 0, st>>>(P, S);
    AtomIn ai;
    ai.n_atoms = n_atoms;
    ai.n_total = sym->n_symops_total > 0 ? sym->n_symops_total : sym->n_symops;
    ai.n_types = P.n_types;
    std::copy(A6, A6 + 36, ai.A6);
    ai.type = atom_type;
    ai.adpk = adp_components;
    ai.xyz = xyz;
    ai.adp = adp;
    ai.occ = occupancy;
    ai.mult = multiplicity;
    ai.anom = anomalous;
    noalloc_atoms_kernel<<<(n_atoms + 127) / 128, 128, 0, st>>>(ai, S);
    HklIn hi;
    hi.n_hkl = n_hkl;
    std::copy(B, B + 9, hi.B);
    hi.centering = centering;
    hi.obverse = sym->obverse;
    int centro = 0;
    for (int i = 0; i < 3; i++) {
        const double t = sym->inversion_translation[i] * 24.0;
        hi.t_inv24[i] = sym->centrosymmetric ? ((((int)std::rint(t)) % 24) + 24) % 24 : 0;
    }
    if (sym->centrosymmetric) centro = (hi.t_inv24[0] | hi.t_inv24[1] | hi.t_inv24[2]) ? 2 : 1;
    hi.hkl = hkl;
    noalloc_hkl_kernel<<<(n_hkl + 255) / 256, 256, 0, st>>>(hi, S);
    if ((ce = cudaGetLastError()) != cudaSuccess) return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));

    // the per-call kernels of dsf_calculate_device on the scratch
    if ((ce = launch_adjoint_weights(n_hkl, reinterpret_cast<const double2 *>(dtdf), S.mult, S.cinv, centro, S.gw_d,
                                     S.gw_f, st)) != cudaSuccess)
        return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));
    if ((ce = cudaMemsetAsync(S.f_acc, 0, sizeof(double2) * (size_t)n_hkl, st)) != cudaSuccess ||
        (ce = cudaMemsetAsync(S.g_acc, 0, sizeof(double) * kNch * (size_t)n_atoms, st)) != cudaSuccess)
        return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));
    DevStructure D{};
    std::memset(&D, 0, sizeof D);
    D.model = MODEL_IAM;
    D.n_atoms = n_atoms;
    D.n_hkl = n_hkl;
    D.n_sym = P.n_sym;
    D.n_tiles = n_tiles;
    D.n_types = P.n_types;
    std::copy(B, B + 9, D.B);
    for (int i = 0; i < 9; i++) D.Bf[i] = (float)B[i];
    D.sym_rot = S.sym_rot;
    D.sym_t24 = S.sym_t24;
    D.tile_begin = S.tile_begin;
    D.tile_ntypes = S.tile_ntypes;
    D.tile_types = S.tile_types;
    D.atom_ltype = S.ltype;
    D.atom_adpk = S.adpk;
    D.atom_active = S.active;
    D.atom_xq = S.xq;
    D.atom_xlo = S.xlo;
    D.atom_xd = S.xd;
    D.atom_adp_f = S.adp_f;
    D.atom_adp_d = S.adp_d;
    D.atom_w_f = S.w_f;
    D.atom_w_d = S.w_d;
    D.atom_anom_f = S.anom_f;
    D.atom_anom_d = S.anom_d;
    D.types_f = S.types_f;
    D.types_d = S.types_d;
    D.hkl = S.hkl;
    D.h2 = S.h2;
    D.h2f = S.h2f;
    D.atom_orig = S.perm;
    CallBuffers C;
    C.gw_d = S.gw_d;
    C.gw_f = S.gw_f;
    C.f_acc = S.f_acc;
    C.g_acc = S.g_acc;
    const bool fp64 = precision == DSF_FP64;
    int smem_optin = 0, n_sm = 1;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
    int ht = kMaxHT;
    while (ht > 2 && sf_grad_smem_bytes(fp64, ht, D.n_sym) > std::min<size_t>((size_t)smem_optin, 110 * 1024)) ht /= 2;
    const int n_chunks = std::max(1, n_sm * 8 / n_tiles);
    int chunk = (n_hkl + n_chunks - 1) / n_chunks;
    chunk = std::max(chunk, 4 * ht);
    chunk = (chunk + ht - 1) / ht * ht;
    if ((ce = launch_sf_grad(D, C, fp64, false, chunk, ht, st)) != cudaSuccess)
        return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));
    if ((ce = launch_f_epilogue(n_hkl, S.f_acc, S.mult, S.cinv, centro, out->f, st)) != cudaSuccess)
        return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));
    if (derivative_flags & (DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC)) {
        if ((ce = launch_grad_epilogue(n_atoms, 0, Minv, A6, derivative_flags, S.g_acc, S.perm, S.adpk, S.w_d,
                                       S.multw, out, st)) != cudaSuccess)
            return report(err, err_len, DSF_ERR_CUDA, cudaGetErrorString(ce));
    }
    return DSF_OK;
}
