// Device-side data layout of a resident structure and the launch parameters
// of the structure-factor kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dsf {

constexpr int kTileAtoms = 128;   // atoms per block (one per thread)
constexpr int kMaxTileTypes = 32; // distinct atom types inside one atom tile
constexpr int kMaxHT = 16;        // reflections staged per shared-memory sub-tile
constexpr int kMaxSym = 48;
constexpr int kNch = 40;          // per-atom derivative channels
constexpr int kRad = 13;          // radial values per (reflection, type)

// per-atom accumulator channels
enum Channel {
    CH_XYZ = 0,    // 3: d/d(fractional x,y,z) before the 2 pi w factor
    CH_ADP = 3,    // 6: aniso (beta basis) or [0] iso
    CH_OCC = 9,
    CH_PV = 10,
    CH_KAPPA = 11,
    CH_KAPPA_P = 12,
    CH_PLM = 13,   // 25: global-frame P_lm
};

enum ModelKind { MODEL_HC = 0, MODEL_IAM = 1, MODEL_TABLE = 2 };

// Radial constants of one atom type in the precision R of a kernel.  The
// Fourier-Bessel integrals are evaluated as pre * s^l C_m^{(l+1)}(c) / rho^{n+1}
// (see dsf_math.cuh); every constant prefactor (4 pi, the density
// normalisation, the sign of i^l, 2^l l! m!) is folded in on the host.
template <typename R>
struct TypeRadialT {
    R pv, inv_kappa, inv_kappa_p, zeta;
    R def_pre[5];       // signed 4 pi N_l 2^l l! m_l!
    int def_m[5];       // m_l = n_l + 1 - l
    int n_def;          // number of l with a radial function
    int core_begin, core_end, val_begin, val_end;  // into the density-term arrays
    int iam_n;
    R iam_a[5], iam_b[5], iam_c;
    R e_z, e_f000;      // electron scattering: atomic number, f_e at h = 0
};

struct DevStructure {
    int model;
    int electron;                // HC form factors converted to electron scattering (Mott-Bethe)
    int n_atoms, n_hkl, n_sym, n_tiles, n_types;
    double B[9];                 // h_cart = B h_frac (row-major)
    float Bf[9];
    const int *sym_rot;          // [n_sym][9] fractional, x' = R x + t
    const int *sym_t24;          // [n_sym][3] translation in 1/24
    const int *tile_begin;       // [n_tiles+1]
    const int *tile_ntypes;      // [n_tiles]
    const int *tile_types;       // [n_tiles][kMaxTileTypes]
    const int *atom_ltype;       // sorted atoms: local type index
    const int *atom_adpk;        // 0 / 1 / 6
    const uint8_t *atom_active;  // inclusion mask of the current call
    const uint32_t *atom_xq;     // [3] fractional position, 2^32 fixed point
    const float *atom_xlo;       // [3] x - xq 2^-32
    const double *atom_xd;       // [3]
    const float *atom_adp_f;     // [6] log2(e) * beta (2 pi^2 U*) or [0] = log2(e) 2 pi^2 Uiso
    const double *atom_adp_d;    // [6] beta or [0] 2 pi^2 Uiso
    const float *atom_w_f;       // occupancy * multiplicity / n_total
    const double *atom_w_d;
    const float2 *atom_anom_f;
    const double2 *atom_anom_d;
    const float *atom_pg_f;      // [25] global-frame P_lm (HC)
    const double *atom_pg_d;
    const TypeRadialT<float> *types_f;
    const TypeRadialT<double> *types_d;
    const float *term_pre_f;     // 4 pi c m! of the Slater density terms (core and valence)
    const double *term_pre_d;
    const float *term_exp_f;
    const double *term_exp_d;
    const int *term_m;           // m = n + 1 with n the r power of the density term
    const int4 *hkl;             // [n_hkl] (h,k,l,0)
    const double *h2;            // |h_cart|^2
    const float *h2f;
    const float2 *table_f;       // tabulated model: [n_hkl_pad][table_stride][n_sym] (+16 bytes of slack)
    const double2 *table_d;
    int table_stride;            // columns per (reflection, operation) row: even
    int table_split, table_shift;  // column of sorted atom a: a + (a >= split ? shift : 0) (even tile starts)
    const int *atom_orig;        // sorted -> original atom index
    const int *atom_plm_lmax;    // highest l of the atom's P_lm parameters (-1: none)
    // per (sorted atom, operation): the line step e^{2 pi i ((R^T e_l).x + t_l)}, computed in FP64 with the
    // atom conversion (once per atom upload, not per block)
    const float2 *atom_step_f;
    const double2 *atom_step_d;
};

struct CallBuffers {
    const double2 *gw_d;   // effective adjoint weight per reflection
    const float2 *gw_f;
    double2 *f_acc;        // [n_hkl]
    double *g_acc;         // [n_atoms][kNch]
};

}  // namespace dsf
