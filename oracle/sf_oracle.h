/*
 * CPU oracle for the structure-factor + derivative path.  TEST
 * INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline leg
 * of the benchmark call it as the checker; nothing in the shipped library
 * links or calls it.
 *
 * Plain FP64 C restatement of the reference engine's per-reflection sum
 * and adjoint, evaluated directly (no line recurrences):
 *   - HansenCoppens_SF_Engine3::calculateSF and its three serial kernels
 *     (src/Scattering/HansenCoppens_SF_Engine3.cpp:678-950, 1030-1509,
 *      1511-1992, 2649-2894);
 *   - pre_hkl_loop_sf_calc / pre_atom_loop_sf_calc (same file :195-256, 319-418);
 *   - calculateDeformationValence in the atom's local frame (same file :150-184)
 *     with combine_multipolar_terms (include/discamb/Scattering/
 *     HansenCoppens_SF_Engine3.h:986-1074);
 *   - the generic all-operations loop of AnyScattererStructureFactorCalculator
 *     (src/Scattering/AnyScattererStructureFactorCalculator.cpp:614-829) for
 *     the IAM and tabulated-form-factor models.
 * Multipole-parameter derivatives (P_val, P_lm, kappa, kappa') have no
 * counterpart in the reference; they are the analytic derivatives of the
 * same sum and are checked against finite differences of the reference F.
 *
 * Conventions (engine level, like the reference engine): Cartesian
 * positions [A], ADPs as U_cart * 2 pi^2, Cartesian reflection vectors
 * [1/A], dtdf already conjugated and multiplied by the centering factor.
 */
#ifndef DSF_SF_ORACLE_H
#define DSF_SF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { SFO_MODEL_HC = 0, SFO_MODEL_IAM = 1, SFO_MODEL_TABLE = 2 };

typedef struct {
    int model;
    /* wavefunction types (HC) : CSR over density terms */
    int n_wfn;
    const int *core_off; const double *core_coeff; const double *core_exp; const int *core_pow;
    const int *val_off; const double *val_coeff; const double *val_exp; const int *val_pow;
    const double *def_exp;      /* [n_wfn] zeta */
    const int *def_npow;        /* [n_wfn] number of n_l entries */
    const int *def_pow;         /* [n_wfn*5] */
    const double *wfn_anom;     /* [n_wfn*2] */
    /* atom types (HC) */
    int n_types;
    const int *type_nl;         /* p_lm.size() */
    const double *type_plm;     /* [n_types*25], index l*l+m+l */
    const double *type_pval, *type_kappa, *type_kappa_p;
    /* IAM: per type n-Gaussian: a[5], b[5], c, n_gauss */
    const int *iam_ngauss;      /* [n_types] */
    const double *iam_a, *iam_b, *iam_c;   /* [n_types*5], [n_types*5], [n_types] */
    /* tabulated: f[h][s][atom] complex (re,im) */
    const double *table;
    /* atoms */
    int n_atoms;
    const int *atom_wfn, *atom_type;
    const double *pos;          /* [n*3] Cartesian */
    const int *n_adp;           /* 0,1,6 */
    const double *adp;          /* [n*6] U_cart*2pi^2 (iso in [0]) */
    const double *occ, *mult_w; /* occupancy, multiplicity/n_sym_total */
    const double *lcs;          /* [n*9] row-major, columns = local axes */
    const double *atom_anom;    /* [n*2] or NULL */
    const int *include;         /* [n] */
    /* symmetry */
    int n_sym;
    const double *rot;          /* [n_sym*9] Cartesian, row-major */
    const double *trans;        /* [n_sym*3] Cartesian */
    int centro;
    double inv_trans[3];        /* Cartesian translation of the inversion op */
    /* reflections */
    int n_hkl;
    const double *h;            /* [n_hkl*3] Cartesian */
    const double *dtdf;         /* [n_hkl*2] conj(dT/dF) * centering */
    /* derivative switches */
    int d_xyz, d_adp, d_occ, d_mp;
    /* electron scattering (HC, Mott-Bethe, HansenCoppens_SF_Engine3.cpp:1387-1397):
     * per wavefunction atomic number and f_e at s = 0 */
    int electron;
    const int *wfn_z;
    const double *wfn_f000;
} sfo_problem;

typedef struct {
    double *f;        /* [n_hkl*2] */
    double *d_xyz;    /* [n*3] Cartesian */
    double *d_adp;    /* [n*6] U_cart */
    double *d_occ;    /* [n] */
    double *d_pval;   /* [n] */
    double *d_plm;    /* [n*25] local frame, density normalised */
    double *d_kappa;  /* [n] */
    double *d_kappa_p;/* [n] */
} sfo_result;

/* Structure factors and target-function derivatives; returns 0 on success. */
int sfo_compute(const sfo_problem *p, sfo_result *r, int n_threads);

/* The same for the HC model in the reference engine's line-ordered loop
 * (recurrences along (h, k, l) lines, harmonics per (reflection, operation),
 * P_lm rotated once per atom): the benchmark's CPU baseline.  hkl: the
 * integer indices of p->h; b3: the Cartesian third reciprocal axis. */
int sfo_compute_lines(const sfo_problem *p, const int *hkl, const double *b3, sfo_result *r, int n_threads);

/* int_0^inf r^n exp(-z r) j_l(2 pi h r) dr, 0<=l<=5, l+1<=n<=12 */
double sfo_g(int l, int n, double h, double z);
/* form factors of every atom at one Cartesian reciprocal vector h[3]: ff[n_atoms][re, im] (HC, IAM) */
int sfo_form_factors(const sfo_problem *p, const double h[3], double *ff);

/* density-normalised real spherical harmonics d_lm(u), l<=4, u normalised */
void sfo_dlm(const double u[3], double out[25]);

#ifdef __cplusplus
}
#endif
#endif
