/*
 * dsf_gb300 -- C ABI of the GB300 structure-factor + derivative engine.
 *
 * Drop-in boundary for the structure-factor hot path of DiSCaMB.  The
 * functions here replace, call for call:
 *
 *   dsf_structure_create_hc     HansenCoppensStructureFactorCalculator(crystal, HC_ModelParameters)
 *                               + setModel (src/Scattering/HansenCoppensStructureFactorCalculator.cpp:57-72, 157-290)
 *   dsf_structure_create_iam    AnyIamCalculator::set / IamFormFactorCalculationsManager
 *                               (src/Scattering/AnyIamCalculator.cpp:49-154)
 *   dsf_structure_create_tabulated
 *                               TscFileBasedSfCalculator + ConstFormFactorCalculationsManager
 *                               (src/Scattering/TscFileBasedSfCalculator.cpp:17-123,
 *                                src/Scattering/ConstFormFactorCalculationsManager.cpp:34-102)
 *   dsf_structure_set_hkl       the hkl argument of calculateStructureFactorsAndDerivatives, kept
 *                               resident across calls (include/discamb/Scattering/SfCalculator.h:45-67)
 *   dsf_structure_update_atoms  SfCalculator::update / the atoms argument
 *                               (prepareDataForEngine_part, HansenCoppensStructureFactorCalculator.cpp:897-990)
 *   dsf_structure_update_types  HC_ModelParameters::type_parameters (P_lm, P_val, kappa, kappa')
 *   dsf_structure_set_anomalous SfCalculator::setAnomalous (per-atom f', f'')
 *   dsf_structure_set_lcs       the localCoordinateSystems argument
 *                               (include/discamb/Scattering/HansenCoppensStructureFactorCalculator.h:148-165)
 *   dsf_calculate               calculateStructureFactorsAndDerivatives(atoms, [lcs,] hkl, f,
 *                               dTarget_dparam, dTarget_df, countAtomContribution, selector)
 *                               (HansenCoppensStructureFactorCalculator.cpp:380-508 and
 *                                AnyScattererStructureFactorCalculator.cpp:614-829), host buffers
 *   dsf_calculate_atoms         the same call with the atoms' parameters of the call (one submission)
 *   dsf_calculate_device        the same with device-resident buffers on a caller stream
 *   dsf_structure_create_tabulated_device
 *                               the tabulated model from a device table (no host copy of the table)
 *   dsf_calculate_batch, dsf_calculate_batch_atoms, dsf_calculate_batch_device
 *                               many structures in one submission (the reference's callers run one
 *                               calculator per structure in turn, HcAtomBankStructureFactorCalculator.cpp:482-520)
 *   dsf_structure_create_tsc, dsf_tsc_load
 *                               TscFileBasedSfCalculator / tsc_io::read_tsc (the .tsc reader)
 *   dsf_structure_set_electron  HansenCoppensStructureFactorCalculator::setElectronScattering
 *   dsf_reduce_to_types         per-type multipole derivatives for TAAM callers (no reference counterpart)
 *   dsf_submit, dsf_poll        asynchronous form of dsf_calculate_atoms for serving (no reference counterpart)
 *   dsf_form_factors            SfCalculator::calculateFormFactors(hkl, ff, includeAtom) (SfCalculator.h:82-93;
 *                               HansenCoppensStructureFactorCalculator.cpp:1277-1304, AnyIamCalculator.cpp:223-233)
 *   dsf_last_error              on_error::throwException messages (include/discamb/BasicUtilities/on_error.h:24-36):
 *                               every function returns a status instead of throwing; the message is the
 *                               calling thread's last one
 *
 * Conventions follow the reference: dT/dF = dT/dA + i dT/dB per reflection;
 * derivatives are returned in the crystal's xyz and ADP conventions;
 * positions fractional or Cartesian [A]; ADPs U_cif, U_cart or U_star;
 * anisotropic ADP order U11 U22 U33 U12 U13 U23.
 * Thread safety: one structure must not be used by two host threads at once
 * (as for the reference calculators); distinct structures may.
 */
#ifndef DSF_GB300_H
#define DSF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSF_ABI_VERSION 1

enum dsf_status {
    DSF_OK = 0,
    DSF_ERR_ARGUMENT = 1,   /* invalid argument (size mismatch, bad index, unsupported value) */
    DSF_ERR_CUDA = 2,       /* CUDA runtime error */
    DSF_ERR_MEMORY = 3,     /* device or host allocation failed, or over the memory budget */
    DSF_ERR_STATE = 4,      /* call not valid in the current state (e.g. no reflections set) */
    DSF_ERR_TIMEOUT = 5,    /* a bounded wait ran out */
    DSF_ERR_UNSUPPORTED = 6,
    DSF_PENDING = 7         /* dsf_poll: the submitted call has not finished within the timeout; poll again */
};

enum dsf_precision { DSF_FP64 = 0, DSF_FP32_BULK = 1 };
enum dsf_xyz_convention { DSF_XYZ_FRACTIONAL = 0, DSF_XYZ_CARTESIAN = 1 };
enum dsf_adp_convention { DSF_ADP_U_CIF = 0, DSF_ADP_U_CART = 1, DSF_ADP_U_STAR = 2 };

/* derivative selection (DerivativesSelector, include/discamb/Scattering/SF_CalcDataTypes.h:22-27,
 * plus the multipole-model parameters the reference does not differentiate).  0: structure factors only
 * (calculateStructureFactors, HansenCoppensStructureFactorCalculator.cpp:305-326): the FP32 single-structure
 * kernels then run without the adjoint; dtdf must still point to n_hkl values (any, e.g. 1) */
enum dsf_derivative_flags {
    DSF_D_XYZ = 1, DSF_D_ADP = 2, DSF_D_OCC = 4,
    DSF_D_MULTIPOLE = 8   /* P_val, P_lm, kappa, kappa' per atom */
};

typedef struct dsf_engine dsf_engine;
typedef struct dsf_structure dsf_structure;
typedef struct dsf_ticket dsf_ticket;

/* Crystal symmetry as the engine consumes it.  Either the engine subset
 * (operations modulo inversion and lattice centering, centrosymmetric = 1,
 * inversion_translation = t of the inversion -x+t; the HansenCoppens CPU
 * engine's representation) or any operation list with centrosymmetric = 0
 * (e.g. all operations modulo centering: the generic AnyScatterer
 * representation).  Lattice centering enters as the per-reflection
 * multiplier of scattering_utilities::centeringSfMultipliers.  With the
 * inversion taken by the engine, anomalous dispersion enters as the
 * reference's centrosymmetric engine takes it (F = U + c conj(U) with U the
 * sum over the listed operations, HansenCoppens_SF_Engine3.cpp:1920-1935);
 * the all-operations form sums f' + i f'' over every operation. */
typedef struct {
    double cell[6];                   /* a b c [A], alpha beta gamma [deg] */
    int n_symops;
    const int *symop_rotation;        /* [n_symops][3][3] fractional, row-major: x' = R x + t */
    const double *symop_translation;  /* [n_symops][3] fractional (multiples of 1/24) */
    int centrosymmetric;
    double inversion_translation[3];
    char centering;                   /* P A B C I F R */
    int obverse;                      /* R only: 1 obverse (-h+k+l = 3n); 0 reverse, tested as the reference
                                       * tests it, (h-k+l) even (scattering_utilities.cpp:117-134) */
    int n_symops_total;               /* full operation count; weight = multiplicity / n_symops_total */
} dsf_symmetry;

/* Hansen-Coppens model: spherical densities per wavefunction type as Slater
 * density terms c r^n exp(-z r) (CSR over wavefunction types), the
 * deformation-valence radial functions and the atom types. */
typedef struct {
    int n_wfn;
    const int *core_offset;    /* [n_wfn+1] */
    const double *core_coeff;
    const double *core_exp;
    const int *core_pow;
    const int *val_offset;     /* [n_wfn+1], valence normalised to one electron */
    const double *val_coeff;
    const double *val_exp;
    const int *val_pow;
    const double *def_val_exp;  /* [n_wfn] zeta [1/A] */
    const int *def_val_npow;    /* [n_wfn] number of n_l entries (<= 5) */
    const int *def_val_pow;     /* [n_wfn][5] n_l */
    const double *anomalous;    /* [n_wfn][2] */
    int n_types;
    const int *type_nl;          /* [n_types] number of l levels of P_lm (p_lm.size()) */
    const double *type_plm;      /* [n_types][25], index l*l + m + l, density normalised */
    const double *type_pval;
    const double *type_kappa;
    const double *type_kappa_prime;
} dsf_hc_model;

/* IAM: per scatterer type f0(|h|) = sum_i a_i exp(-b_i |h|^2/4) + c */
typedef struct {
    int n_types;
    const int *n_gauss;     /* [n_types] <= 5 */
    const double *a;        /* [n_types][5] */
    const double *b;        /* [n_types][5] */
    const double *c;        /* [n_types] */
} dsf_iam_model;

typedef struct {
    int n_atoms;
    const int *atom_wfn;         /* HC: wavefunction type */
    const int *atom_type;        /* HC / IAM: type */
    const int *adp_components;   /* 0, 1 or 6 */
    const double *lcs;           /* HC: [n_atoms][3][3] row-major, columns = local x, y, z */
    const double *multiplicity;  /* [n_atoms] */
    const double *anomalous;     /* [n_atoms][2] or NULL (HC: per wavefunction) */
    int xyz_convention;
    int adp_convention;
} dsf_atoms;

/* outputs of one call: f always written; each derivative output written only when derivative_flags asks for it
 * (the others keep what the caller had there) */
typedef struct {
    double *f;            /* [n_hkl][2] */
    double *d_xyz;        /* [n_atoms][3] or NULL */
    double *d_adp;        /* [n_atoms][6] (first 1 or 6 used) or NULL */
    double *d_occ;        /* [n_atoms] or NULL */
    double *d_pval;       /* [n_atoms] or NULL */
    double *d_plm;        /* [n_atoms][25] local frame or NULL */
    double *d_kappa;      /* [n_atoms] or NULL */
    double *d_kappa_prime;/* [n_atoms] or NULL */
} dsf_outputs;

/* ---- engine (one GPU, one stream) -------------------------------------- */
int dsf_engine_create(int device, dsf_engine **out);
int dsf_engine_destroy(dsf_engine *e);
const char *dsf_last_error(const dsf_engine *e);
int dsf_abi_version(void);

/* ---- resident structures ---------------------------------------------- */
int dsf_structure_create_hc(dsf_engine *e, const dsf_symmetry *sym, const dsf_hc_model *model,
                            const dsf_atoms *atoms, dsf_structure **out);
int dsf_structure_create_iam(dsf_engine *e, const dsf_symmetry *sym, const dsf_iam_model *model,
                             const dsf_atoms *atoms, dsf_structure **out);
/* table: complex form factors [n_hkl][n_symops][n_atoms] (re,im) for the
 * reflections passed here (they become the structure's reflection set) */
int dsf_structure_create_tabulated(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms,
                                   int n_hkl, const int *hkl, const double *table, int table_fp32,
                                   dsf_structure **out);
/* the same from a device table (the caller's buffer on the engine's device, complex64 when table_fp64 = 0,
 * else complex128; [n_hkl][n_symops][n_atoms] in the order of hkl): gathered on the device into the engine's
 * complex64 table, so tables larger than host memory never cross the host.  The caller may free its buffer when
 * the call returns.  The reference's table lives in a host std::map (ConstFormFactorCalculationsManager.cpp:9-15). */
int dsf_structure_create_tabulated_device(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms,
                                          int n_hkl, const int *hkl, const void *table_device, int table_fp64,
                                          dsf_structure **out);
/* the tabulated model from a .tsc file (TscFileBasedSfCalculator, src/Scattering/TscFileBasedSfCalculator.cpp:17-123;
 * format of tsc_io::read_tsc, src/IO/tsc_io.cpp:60-125): the file's columns are the structure's atoms in order; its
 * rows must cover h' = h R for every reflection and operation of sym (a missing h' is an error, as in the reference) */
int dsf_structure_create_tsc(dsf_engine *e, const dsf_symmetry *sym, const dsf_atoms *atoms, int n_hkl,
                             const int *hkl, const char *path, dsf_structure **out);
/* the raw contents of a .tsc file (no device needed): first call with hkl = values = NULL for the sizes, then with
 * hkl [n_rows][3] and values [n_rows][n_atoms][2] of capacity_rows rows */
int dsf_tsc_load(const char *path, int *n_atoms, int *n_rows, int *hkl, double *values, int capacity_rows);
int dsf_structure_destroy(dsf_structure *s);

int dsf_structure_set_hkl(dsf_structure *s, int n_hkl, const int *hkl);
/* atoms in the crystal's conventions; adp [n_atoms][6] (first 1 or 6 used) */
int dsf_structure_update_atoms(dsf_structure *s, const double *xyz, const double *adp, const double *occupancy);
int dsf_structure_update_types(dsf_structure *s, const double *type_plm, const double *type_pval,
                               const double *type_kappa, const double *type_kappa_prime);
int dsf_structure_set_lcs(dsf_structure *s, const double *lcs);
/* per-atom anomalous dispersion [n_atoms][2] (f', f'') in the caller's atom order, replacing the values given at
 * creation (SfCalculator::setAnomalous, include/discamb/Scattering/SfCalculator.h:43; the HC calculator's
 * set_anomalous_dispersion_per_atom, HansenCoppensStructureFactorCalculator.h:49) */
int dsf_structure_set_anomalous(dsf_structure *s, const double *anomalous);
/* bytes of device memory the structure holds */
int64_t dsf_structure_device_bytes(const dsf_structure *s);

/* ---- calculation --------------------------------------------------------- */
/* host buffers: dtdf [n_hkl][2]; include [n_atoms] (NULL = all); outputs on host */
int dsf_calculate(dsf_structure *s, int precision, int derivative_flags, const double *dtdf,
                  const int *include, const dsf_outputs *out);
/* the reference call shape: the atoms' current parameters (xyz [n][3], adp [n][6], occupancy [n], crystal's
 * conventions) with dT/dF, uploaded and computed in one call (calculateStructureFactorsAndDerivatives(atoms, hkl,
 * f, dTarget_dparam, dTarget_df, countAtomContribution), include/discamb/Scattering/SfCalculator.h:45-67) */
int dsf_calculate_atoms(dsf_structure *s, int precision, int derivative_flags, const double *xyz, const double *adp,
                        const double *occupancy, const double *dtdf, const int *include, const dsf_outputs *out);
/* device buffers, asynchronous on `stream` (cudaStream_t, NULL = engine stream) */
int dsf_calculate_device(dsf_structure *s, int precision, int derivative_flags, const double *dtdf_device,
                         const dsf_outputs *out_device, void *stream);
/* n structures of one engine in one submission (device buffers per structure, asynchronous on `stream`): the
 * FP32 structure-factor kernels of structures without the multipole adjoint run as batched launches, one per
 * kernel shape.  The same results as n dsf_calculate_device calls; the reference has no batched call (one
 * calculator per structure, SfCalculator.h:45-67, called in turn by its callers). */
int dsf_calculate_batch_device(dsf_structure *const *structures, int n, int precision, int derivative_flags,
                               const double *const *dtdf_device, const dsf_outputs *out_device, void *stream);
/* electron scattering for an HC structure (the reference's setElectronScattering,
 * HansenCoppensStructureFactorCalculator.cpp:510-514): every form factor converted by Mott-Bethe,
 * f_e = 0.023934 (Z - f_x) / s^2 + f'' terms, f_e(000) = wfn_f000 (the element's electron scattering factor at s = 0,
 * which the reference takes from its "electron-IT" table); wfn_z, wfn_f000: [n_wfn]; on = 0 switches back to X-rays */
int dsf_structure_set_electron(dsf_structure *s, int on, const int *wfn_z, const double *wfn_f000);
/* TAAM-style types: the multipole-parameter derivatives of dsf_calculate_device (per_atom: device buffers in the
 * caller's atom order) summed over the atoms of each type into per_type (device buffers [n_types], [n_types][25];
 * NULL members are skipped); asynchronous on `stream`.  The reference computes no multipole derivatives; its TAAM
 * callers refine per-type parameters (HcAtomBankStructureFactorCalculator.cpp:482-520). */
int dsf_reduce_to_types(dsf_structure *s, const dsf_outputs *per_atom, const dsf_outputs *per_type, void *stream);
/* form factors of every atom at one reflection hkl[3] (the reference's single-h calculateFormFactors): ff[2 n_atoms]
 * (re, im) in the caller's atom order, no anomalous dispersion, 0 for atoms with include[a] == 0 (include may be
 * NULL); FP64, synchronous.  HC and IAM structures; DSF_ERR_UNSUPPORTED for the tabulated model. */
int dsf_form_factors(dsf_structure *s, const int *hkl, const int *include, double *ff);
/* test hook of the failure path: the next single-structure FP32/FP64 call of s issues no copies for its first
 * reflection sub-tile, so every block's bounded wait runs out (about 4 s), the kernel sets its error flag and exits,
 * and a host-buffer call returns DSF_ERR_TIMEOUT; the engine stays usable.  No reference counterpart (the reference
 * GPU code exit()s on errors, src/GPU/cuda/globals.h:22). */
int dsf_debug_stall_next_call(dsf_structure *s);
/* asynchronous dsf_calculate_atoms for serving (xyz/adp/occupancy may be NULL: the resident atoms): the inputs are
 * staged before the call returns (the caller may reuse its input buffers at once), the kernels and the readback
 * are queued on the engine's stream, and *ticket identifies the call.  The output buffers are written by dsf_poll.
 * One pending call per structure (DSF_ERR_STATE otherwise); other structures of the engine may be submitted
 * meanwhile.  The reference calls synchronously (SfCalculator.h:45-67); a serving caller overlaps its own work. */
int dsf_submit(dsf_structure *s, int precision, int derivative_flags, const double *xyz, const double *adp,
               const double *occupancy, const double *dtdf, const int *include, const dsf_outputs *out,
               dsf_ticket **ticket);
/* waits up to timeout_ms (0: test only) for a submitted call: DSF_OK with the outputs written (the ticket is
 * released), DSF_PENDING (the ticket stays valid: poll again), or the call's error (the ticket is released) */
int dsf_poll(dsf_ticket *ticket, int timeout_ms);
/* the same with host buffers (dtdf[i] [n_hkl_i][2], include[i] NULL = all atoms, outputs on the host).  A batch
 * of 8 or more structures with at least 64 MB of inputs and outputs runs as up to four groups of consecutive
 * structures, so that the host copies of one group overlap the GPU work of another; smaller ones take one stream
 * synchronisation */
int dsf_calculate_batch(dsf_structure *const *structures, int n, int precision, int derivative_flags,
                        const double *const *dtdf, const int *const *include, const dsf_outputs *out);
/* the same with every structure's atomic parameters of this call (xyz[i] NULL: the resident ones), as
 * dsf_calculate_atoms does for one structure: a serving loop's least-squares cycles in one submission */
int dsf_calculate_batch_atoms(dsf_structure *const *structures, int n, int precision, int derivative_flags,
                              const double *const *xyz, const double *const *adp, const double *const *occupancy,
                              const double *const *dtdf, const int *const *include, const dsf_outputs *out);

/* ---- tile-shape autotuner -------------------------------------------------
 * No reference counterpart (the reference's threads take fixed contiguous shares of the reflections,
 * scattering_utilities::splitHklLines, src/Scattering/scattering_utilities.cpp:463-517).  dsf_autotune times
 * the structure's call (these precision and derivative flags) over a few tile shapes -- reflection chunks aiming
 * at 24, 48, 75 or 150 blocks per SM, the longest shared-memory sub-tile or at most 8 reflections, and for the
 * FP32 multipole-adjoint kernels the compiler's registers or a cap for three blocks per SM -- on a zero dT/dF
 * in scratch buffers it allocates and frees, and keeps the fastest for every later call of structures with the
 * same shape key (model, precision, multipole adjoint, derivative pass, operation count, coset form, atoms and
 * reflections in half-octaves, SM count).  Results do not depend on the shape beyond the order of the
 * cross-block sums.  Synchronous.  dsf_tuning_lookup: the shape the next call would take (ht 0: the longest
 * sub-tile; occupancy 3: the register-capped form, 0: the compiler's registers; *tuned 0: the rule, 75 blocks
 * per SM).  dsf_tuning_save / dsf_tuning_load: the engine's tuned shapes to and from a text file. */
int dsf_autotune(dsf_structure *s, int precision, int derivative_flags, int *blocks_per_sm, int *ht,
                 int *occupancy, double *best_ms);
int dsf_tuning_lookup(dsf_structure *s, int precision, int derivative_flags, int *blocks_per_sm, int *ht,
                      int *occupancy, int *tuned);
int dsf_tuning_save(dsf_engine *e, const char *path);
int dsf_tuning_load(dsf_engine *e, const char *path);

/* number of kernel launches issued by the last calculation (for accounting) */
int dsf_last_launch_count(const dsf_structure *s);
/* device time [ms] of the fused SF+adjoint kernel of the last calculation,
 * from CUDA events recorded around it on its launch stream; -1 while that
 * stream has not finished it */
double dsf_last_kernel_ms(dsf_structure *s);

/* ---- allocation-free call ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: a host program that owns every device allocation through its own
 * pool, or a per-cycle refinement loop that must not trigger allocation.
 * IAM structure factors and derivatives with every input and output in the
 * caller's own device buffers; the scratch lives in one static device array
 * of DSF_NOALLOC_SCRATCH_BYTES (32 MiB) that every GPU which loads the
 * library holds until exit, enough for roughly 500 bytes per atom plus 100
 * bytes per reflection (e.g. 20,000 atoms with 200,000 reflections).  Larger
 * problems are rejected with DSF_ERR_ARGUMENT and a message in err.  No
 * cudaMalloc, cudaFree or other allocating call is made.
 * The first call on a device does a one-time set-up: it looks up the device
 * address of the array.  Under CUDA's lazy module loading (the default) that
 * lookup is also what loads the module and places the 32 MiB array on the
 * GPU, so the first call can fail with DSF_ERR_CUDA (out of memory); make it
 * during set-up, before any stream capture.  The address is kept per device
 * for the life of the process: after cudaDeviceReset of a device, do not call
 * this entry point on that device again.
 * All calls share the array, which keeps the last call's contents: calls
 * that overlap on the GPU (other streams, other host threads) race on it and
 * must be serialised by the caller.
 * The symmetry is checked as dsf_structure_create_* checks it (positive cell
 * lengths, centering one of P A B C I F R, translations in multiples of
 * 1/24).  Atoms whose atom_type is outside 0..n_types-1 contribute nothing;
 * adp_components other than 1 or 6 mean no temperature factor.  It runs the
 * engine's first-generation kernel, several times slower than
 * dsf_calculate_device.
 * Device inputs: atom_type [n], adp_components [n] (0/1/6), xyz [n][3]
 * fractional, adp [n][6] U_cif (Uiso in [0]), occupancy [n], multiplicity
 * [n], anomalous [n][2] or NULL, hkl [n_hkl][3], dtdf [n_hkl][2]; device
 * outputs in out (f required; d_xyz, d_adp, d_occ or NULL).  sym and model
 * are host structures (at most DSF_NOALLOC_MAX_TYPES types). */
#define DSF_NOALLOC_SCRATCH_BYTES (32u << 20)
#define DSF_NOALLOC_MAX_TYPES 32
int dsf_iam_calculate_noalloc(const dsf_symmetry *sym, const dsf_iam_model *model, int n_atoms,
                              const int *atom_type, const int *adp_components, const double *xyz,
                              const double *adp, const double *occupancy, const double *multiplicity,
                              const double *anomalous, int n_hkl, const int *hkl, const double *dtdf,
                              int precision, int derivative_flags, const dsf_outputs *out, void *stream,
                              char *err, int err_len);

#ifdef __cplusplus
}
#endif
#endif
