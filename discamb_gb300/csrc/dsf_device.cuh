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
constexpr int kNch = 40;          // per-atom derivative channels (see ChannelLayout)

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

struct TypeRadial {
    double pv, kappa, kappa_p, zeta;
    double norm[5];       // density normalisation of the deformation radial functions
    int npow[5];          // n_l
    int n_def;            // number of l with a radial function
    int lmax_used;        // l used in the sum (-1: none)
    int core_begin, core_end, val_begin, val_end;
    int iam_n;
    double iam_a[5], iam_b[5], iam_c;
};

struct DevStructure {
    int model;
    int n_atoms, n_hkl, n_sym, n_tiles, n_types;
    double B[9];                 // h_cart = B h_frac (row-major)
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
    const float *atom_adp_f;     // [6] beta (2 pi^2 U*) or [0] = 2 pi^2 Uiso
    const double *atom_adp_d;
    const float *atom_w_f;       // occupancy * multiplicity / n_total
    const double *atom_w_d;
    const float2 *atom_anom_f;
    const double2 *atom_anom_d;
    const float *atom_pg_f;      // [25] global-frame P_lm (HC)
    const double *atom_pg_d;
    const TypeRadial *types;
    const double *term_coeff;    // Slater density terms of all wavefunctions
    const double *term_exp;
    const int *term_pow;
    const int4 *hkl;             // [n_hkl] (h,k,l,0)
    const double *h2;            // |h_cart|^2
    const float2 *table_f;       // tabulated model: [n_hkl][n_sym][n_atoms_orig]
    const double2 *table_d;
    const int *atom_orig;        // sorted -> original atom index
    const int *atom_plm_lmax;    // highest l of the atom's P_lm parameters (-1: none)
};

struct CallBuffers {
    const double2 *gw_d;   // effective adjoint weight per reflection
    const float2 *gw_f;
    double2 *f_acc;        // [n_hkl]
    double *g_acc;         // [n_atoms][kNch]
};

}  // namespace dsf
