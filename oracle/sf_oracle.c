/*
 * CPU oracle for the structure-factor + derivative path: TEST
 * INFRASTRUCTURE, see sf_oracle.h for the scope and the reference functions
 * it restates.  Plain FP64, OpenMP over reflections with per-thread
 * derivative buffers merged at the end (the reference engine's own scheme,
 * src/Scattering/HansenCoppens_SF_Engine3.cpp:773-946).
 */
#include "sf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846

/* ------------------------------------------------------------------------
 * Radial Fourier-Bessel integrals of Slater functions
 *   G(n,l,K,Z) = int_0^inf r^n e^{-Z r} j_l(K r) dr ,  K = 2 pi |h|
 * (closed forms of sto_scattering::gFunction, include/discamb/Scattering/
 * SlaterTypeOrbitalScattering.h:51-183).  The closed forms are generated
 * here rather than tabulated: G(l+1,l) = (2K)^l l! / (Z^2+K^2)^{l+1} and
 * G(n+1,l) = -dG(n,l)/dZ.  Writing G(n,l) = K^l P_{n,l}(Z,K^2) / d^n with
 * d = Z^2+K^2 gives the integer recurrence
 *   P_{n+1} = 2 n Z P_n - d dP_n/dZ .
 * ------------------------------------------------------------------------ */
#define G_LMAX 5
#define G_NMAX 12
#define G_NTERM 16
/* nonzero coefficients of P_{n,l}: c Z^i (K^2)^j */
static int g_nterm[G_LMAX + 1][G_NMAX + 1];
static int g_zi[G_LMAX + 1][G_NMAX + 1][G_NTERM], g_kj[G_LMAX + 1][G_NMAX + 1][G_NTERM];
static double g_c[G_LMAX + 1][G_NMAX + 1][G_NTERM];
static int g_ready = 0;

static void g_init(void)
{
    if (g_ready) return;
    static double poly[G_NMAX + 1][G_NMAX + 2][G_NMAX + 2];
    for (int l = 0; l <= G_LMAX; l++) {
        memset(poly, 0, sizeof(poly));
        double base = 1.0;
        for (int k = 1; k <= l; k++) base *= 2.0 * k;  /* 2^l l! */
        poly[l + 1][0][0] = base;
        for (int n = l + 1; n < G_NMAX; n++)
            for (int i = 0; i <= G_NMAX; i++)
                for (int j = 0; j <= G_NMAX; j++) {
                    double c = poly[n][i][j];
                    if (c == 0.0) continue;
                    poly[n + 1][i + 1][j] += (2.0 * n - i) * c;
                    if (i >= 1) poly[n + 1][i - 1][j + 1] -= i * c;
                }
        for (int n = 0; n <= G_NMAX; n++) {
            int q = 0;
            for (int i = 0; i <= G_NMAX; i++)
                for (int j = 0; j <= G_NMAX; j++)
                    if (poly[n][i][j] != 0.0 && q < G_NTERM) {
                        g_zi[l][n][q] = i; g_kj[l][n][q] = j; g_c[l][n][q] = poly[n][i][j]; q++;
                    }
            g_nterm[l][n] = q;
        }
    }
    g_ready = 1;
}

double sfo_g(int l, int n, double h, double z)
{
    g_init();
    if (l < 0 || l > G_LMAX || n < l + 1 || n > G_NMAX) return 0.0;
    const double k = 2.0 * PI * h;
    const double k2 = k * k;
    const double d = z * z + k2;
    double s = 0.0;
    for (int q = 0; q < g_nterm[l][n]; q++) {
        double t = g_c[l][n][q];
        for (int i = 0; i < g_zi[l][n][q]; i++) t *= z;
        for (int j = 0; j < g_kj[l][n][q]; j++) t *= k2;
        s += t;
    }
    double kl = 1.0;
    for (int i = 0; i < l; i++) kl *= k;
    double dn = 1.0;
    for (int i = 0; i < n; i++) dn *= d;
    return kl * s / dn;
}

/* dG(n,l)/dK = (l/K) G(n,l) - G(n+1,l+1)  (from j_l' = (l/x) j_l - j_{l+1}),
 * returned as derivative with respect to h = K/(2 pi) */
static double g_dh(int l, int n, double h, double z)
{
    double k = 2.0 * PI * h;
    double v = -sfo_g(l + 1, n + 1, h, z);
    if (l > 0 && k > 0.0) v += (double)l / k * sfo_g(l, n, h, z);
    return v * 2.0 * PI;
}

/* ------------------------------------------------------------------------
 * density-normalised real spherical harmonics d_lm, l <= 4
 * polynomials and ordering of real_spherical_harmonics::getPolynomials
 * (include/discamb/MathUtilities/real_spherical_harmonics.h:136-190),
 * normalisation N_lm = (2 - delta_l0) / int |y_lm| dOmega (Paturle &
 * Coppens 1988); values obtained here by piecewise Gauss-Legendre
 * quadrature of |y_lm| over the sphere.
 * ------------------------------------------------------------------------ */
static const double DNORM[25] = {
    0.07957747154594767,
    0.3183098861837907, 0.3183098861837907, 0.3183098861837907,
    0.75, 0.75, 0.2067483357831728, 0.75, 0.375,
    0.4244131815783876, 2.0, 0.3203330895838574, 0.2448537586029175, 0.3203330895838574, 1.0,
    0.4244131815783876,
    1.875, 1.25, 0.6611826845788106, 0.4740025188689597, 0.06941752438437611, 0.4740025188689597,
    0.3305913422894053, 1.25, 0.46875};

void sfo_dlm(const double u[3], double v[25])
{
    const double x = u[0], y = u[1], z = u[2];
    const double xx = x * x, yy = y * y, zz = z * z;
    const double xy = x * y, xz = x * z, yz = y * z;
    v[0] = 1.0;
    v[1] = y; v[2] = z; v[3] = x;
    v[4] = xy; v[5] = yz; v[6] = 2.0 * zz - xx - yy; v[7] = xz; v[8] = xx - yy;
    v[9] = (3.0 * xx - yy) * y; v[10] = xy * z; v[11] = y * (4.0 * zz - xx - yy);
    v[12] = z * (2.0 * zz - 3.0 * xx - 3.0 * yy); v[13] = x * (4.0 * zz - xx - yy);
    v[14] = (xx - yy) * z; v[15] = (xx - 3.0 * yy) * x;
    v[16] = xy * (xx - yy); v[17] = (3.0 * xx - yy) * yz; v[18] = xy * (7.0 * zz - 1.0);
    v[19] = yz * (7.0 * zz - 3.0); v[20] = (35.0 * zz - 30.0) * zz + 3.0; v[21] = xz * (7.0 * zz - 3.0);
    v[22] = (xx - yy) * (7.0 * zz - 1.0); v[23] = (xx - 3.0 * yy) * xz;
    v[24] = xx * (xx - 3.0 * yy) - yy * (3.0 * xx - yy);
    for (int i = 0; i < 25; i++) v[i] *= DNORM[i];
}

/* ------------------------------------------------------------------------ */

typedef struct { double re, im; } cplx;
static inline cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cplx cscale(cplx a, double s) { cplx r = {a.re * s, a.im * s}; return r; }
static inline cplx cconj(cplx a) { cplx r = {a.re, -a.im}; return r; }

/* i^l */
static const cplx IPOW[5] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, 0}};

#define NCH 40  /* per-atom derivative channels: xyz 3, adp 6, occ, pval, plm 25, kappa, kappa' */
enum { CH_XYZ = 0, CH_ADP = 3, CH_OCC = 9, CH_PV = 10, CH_PLM = 11, CH_K = 36, CH_KP = 37 };

/* highest l for which P_lm exist in the model of a type */
static int type_lmax_params(const sfo_problem *p, int t, int w)
{
    int lm = p->type_nl[t] - 1;
    if (p->def_npow[w] - 1 < lm) lm = p->def_npow[w] - 1;
    if (lm > 4) lm = 4;
    return lm;
}

/* l used in the sum: pre_hkl_loop_sf_calc (HansenCoppens_SF_Engine3.cpp:238-255) */
static int type_lmax_used(const sfo_problem *p, int t, int w)
{
    int lp = -1;
    for (int l = 0; l < p->type_nl[t] && l <= 4; l++)
        for (int m = 0; m < 2 * l + 1; m++)
            if (p->type_plm[t * 25 + l * l + m] != 0.0) lp = l;
    int lm = p->def_npow[w] - 1;
    if (lm > 4) lm = 4;
    return lp < lm ? lp : lm;
}

/* radial terms at |h| = hl per wavefunction / type: HC f_core[w], f_val[t] (and d/dkappa), the normalised
 * deformation radial functions g_l[t][5] (and d/dkappa'); IAM: f0[t] in fval (the reference's pre_hkl_loop_sf_calc,
 * HansenCoppens_SF_Engine3.cpp:195-256, and NGaussianFormFactor::calculate_h) */
static void radial_terms(const sfo_problem *p, const int *type_wfn, double hl, double *fcore, double *fval,
                         double *dfval, double *gl, double *dgl)
{
    if (p->model == SFO_MODEL_HC) {
        for (int w = 0; w < p->n_wfn; w++) {
            double s = 0.0;
            for (int k = p->core_off[w]; k < p->core_off[w + 1]; k++)
                s += p->core_coeff[k] * sfo_g(0, p->core_pow[k] + 2, hl, p->core_exp[k]);
            fcore[w] = 4.0 * PI * s;
        }
        for (int ty = 0; ty < p->n_types; ty++) {
            const int w = type_wfn[ty];
            const double kap = p->type_kappa[ty], kp = p->type_kappa_p[ty];
            double s = 0.0, ds = 0.0;
            for (int k = p->val_off[w]; k < p->val_off[w + 1]; k++) {
                s += p->val_coeff[k] * sfo_g(0, p->val_pow[k] + 2, hl / kap, p->val_exp[k]);
                ds += p->val_coeff[k] * g_dh(0, p->val_pow[k] + 2, hl / kap, p->val_exp[k]);
            }
            fval[ty] = 4.0 * PI * s;
            dfval[ty] = 4.0 * PI * ds * (-hl / (kap * kap)); /* d f_val / d kappa */
            const double zeta = p->def_exp[w];
            for (int l = 0; l < 5; l++) {
                gl[ty * 5 + l] = 0.0;
                dgl[ty * 5 + l] = 0.0;
                if (l < p->def_npow[w]) {
                    const int nl = p->def_pow[w * 5 + l];
                    double norm = pow(zeta, nl + 3);
                    for (int q = 2; q <= nl + 2; q++) norm /= q;
                    gl[ty * 5 + l] = norm * sfo_g(l, nl + 2, hl / kp, zeta);
                    dgl[ty * 5 + l] = norm * g_dh(l, nl + 2, hl / kp, zeta) * (-hl / (kp * kp));
                }
            }
        }
    } else if (p->model == SFO_MODEL_IAM) {
        for (int ty = 0; ty < p->n_types; ty++) {
            double s = p->iam_c[ty];
            const double x2 = hl * hl / 4.0;
            for (int q = 0; q < p->iam_ngauss[ty]; q++) s += p->iam_a[ty * 5 + q] * exp(-p->iam_b[ty * 5 + q] * x2);
            fval[ty] = s;
        }
    }
}

/* form factors of every atom at one Cartesian reciprocal vector h (the reference's single-h calculateFormFactors:
 * HansenCoppens_SF_Engine::calculateFormFactors, HansenCoppens_SF_Engine.cpp:383-500; IAM through
 * IamFormFactorCalculationsManager::calculateCart, IamFormFactorCalculationsManager.cpp:147-161): no anomalous
 * dispersion, no deformation term at h = 0, 0 for excluded atoms; ff [n_atoms][re, im] */
int sfo_form_factors(const sfo_problem *p, const double h[3], double *ff)
{
    if (p->model != SFO_MODEL_HC && p->model != SFO_MODEL_IAM) return 1;
    g_init();
    const int nA = p->n_atoms;
    const int nT = p->n_types > 0 ? p->n_types : 1, nW = p->n_wfn > 0 ? p->n_wfn : 1;
    int *type_wfn = (int *)calloc((size_t)nT, sizeof(int));
    double *fcore = (double *)calloc((size_t)nW, sizeof(double));
    double *fval = (double *)calloc((size_t)nT, sizeof(double));
    double *dfval = (double *)calloc((size_t)nT, sizeof(double));
    double *gl = (double *)calloc((size_t)nT * 5, sizeof(double));
    double *dgl = (double *)calloc((size_t)nT * 5, sizeof(double));
    if (!type_wfn || !fcore || !fval || !dfval || !gl || !dgl) return 1;
    for (int a = 0; a < nA; a++) /* HC types only: the other models carry no per-type wavefunctions */
        if (p->model == SFO_MODEL_HC && p->atom_type[a] >= 0 && p->atom_type[a] < p->n_types)
            type_wfn[p->atom_type[a]] = p->atom_wfn[a];
    const double hl = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    radial_terms(p, type_wfn, hl, fcore, fval, dfval, gl, dgl);
    for (int a = 0; a < nA; a++) {
        cplx f = {0.0, 0.0};
        if (p->include[a]) {
            const int w = p->atom_wfn[a], ty = p->atom_type[a];
            if (p->model == SFO_MODEL_IAM) {
                f.re = fval[ty];
            } else {
                f.re = fcore[w] + fval[ty] * p->type_pval[ty];
                const int lmax_use = type_lmax_used(p, ty, w);
                if (hl >= 1e-10 && type_lmax_params(p, ty, w) >= 0) {
                    const double *L = p->lcs + 9 * a, *P = p->type_plm + 25 * ty;
                    double u[3], d[25];
                    for (int j = 0; j < 3; j++) u[j] = (L[0 + j] * h[0] + L[3 + j] * h[1] + L[6 + j] * h[2]) / hl;
                    sfo_dlm(u, d);
                    for (int l = 0; l <= lmax_use; l++) {
                        double ang = 0.0;
                        for (int m = 0; m < 2 * l + 1; m++) ang += P[l * l + m] * d[l * l + m];
                        f = cadd(f, cscale(IPOW[l], 4.0 * PI * gl[ty * 5 + l] * ang));
                    }
                }
            }
        }
        ff[2 * a] = f.re;
        ff[2 * a + 1] = f.im;
    }
    free(type_wfn); free(fcore); free(fval); free(dfval); free(gl); free(dgl);
    return 0;
}

int sfo_compute(const sfo_problem *p, sfo_result *r, int n_threads)
{
    g_init();
    const int nA = p->n_atoms, nH = p->n_hkl, nS = p->n_sym;
    if (n_threads < 1) n_threads = 1;
#ifndef _OPENMP
    n_threads = 1;
#endif
    double *acc = (double *)calloc((size_t)n_threads * nA * NCH, sizeof(double));
    if (!acc) return 1;
    /* type -> wfn (HC): the wfn of any atom using the type */
    int *type_wfn = (int *)malloc(sizeof(int) * (p->n_types > 0 ? p->n_types : 1));
    for (int t = 0; t < p->n_types; t++) type_wfn[t] = 0;
    for (int a = 0; a < nA; a++) /* HC types only: the other models carry no per-type wavefunctions */
        if (p->model == SFO_MODEL_HC && p->atom_type[a] >= 0 && p->atom_type[a] < p->n_types)
            type_wfn[p->atom_type[a]] = p->atom_wfn[a];

#pragma omp parallel num_threads(n_threads)
    {
#ifdef _OPENMP
        const int tid = omp_get_thread_num();
#else
        const int tid = 0;
#endif
        double *A = acc + (size_t)tid * nA * NCH;
        const int nT = p->n_types > 0 ? p->n_types : 1;
        const int nW = p->n_wfn > 0 ? p->n_wfn : 1;
        double *fcore = (double *)malloc(sizeof(double) * nW);
        double *fval = (double *)malloc(sizeof(double) * nT);
        double *dfval = (double *)malloc(sizeof(double) * nT);
        double *gl = (double *)malloc(sizeof(double) * nT * 5);
        double *dgl = (double *)malloc(sizeof(double) * nT * 5);
        double *hr = (double *)malloc(sizeof(double) * nS * 3);
        double *tf = (double *)malloc(sizeof(double) * nS);

#pragma omp for schedule(dynamic, 16)
        for (int ih = 0; ih < nH; ih++) {
            const double *h = p->h + 3 * ih;
            const double h2 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
            const double hl = sqrt(h2);
            const int h000 = hl < 1e-10;
            const cplx g = {p->dtdf[2 * ih], p->dtdf[2 * ih + 1]};
            for (int s = 0; s < nS; s++) {
                const double *R = p->rot + 9 * s, *t = p->trans + 3 * s;
                for (int j = 0; j < 3; j++) hr[3 * s + j] = h[0] * R[j] + h[1] * R[3 + j] + h[2] * R[6 + j];
                tf[s] = h[0] * t[0] + h[1] * t[1] + h[2] * t[2];
            }
            radial_terms(p, type_wfn, hl, fcore, fval, dfval, gl, dgl);
            /* centrosymmetric handling: e^{2 pi i h.t_inv} */
            double ph_inv = 2.0 * PI * (h[0] * p->inv_trans[0] + h[1] * p->inv_trans[1] + h[2] * p->inv_trans[2]);
            const cplx cinv = {cos(ph_inv), sin(ph_inv)};
            const int at_origin = p->inv_trans[0] == 0.0 && p->inv_trans[1] == 0.0 && p->inv_trans[2] == 0.0;
            /* effective adjoint weight: g_eff = g (acentric), 2 Re g (centre at origin),
             * g + conj(g c_inv) otherwise -- the three serial kernels of the engine */
            cplx ge = g;
            if (p->centro) {
                if (at_origin) { ge.re = 2.0 * g.re; ge.im = 0.0; }
                else ge = cadd(g, cconj(cmul(g, cinv)));
            }
            /* electron scattering: f_e = C (Z - f_x) / s^2 + anomalous, linear in f_x with slope -C/s^2 */
            const double esc = (p->electron && p->model == SFO_MODEL_HC) ? (h000 ? 0.0 : -0.023934 / (0.25 * h2)) : 1.0;
            cplx Ftot = {0, 0};
            for (int a = 0; a < nA; a++) {
                if (!p->include[a]) continue;
                const int w = p->atom_wfn[a], ty = p->atom_type[a];
                const double wgt = p->occ[a] * p->mult_w[a];
                const int nadp = p->n_adp[a];
                const double *adp = p->adp + 6 * a;
                const double *L = p->lcs + 9 * a;
                const double *pos = p->pos + 3 * a;
                cplx anom;
                if (p->atom_anom) { anom.re = p->atom_anom[2 * a]; anom.im = p->atom_anom[2 * a + 1]; }
                else if (p->model == SFO_MODEL_HC) { anom.re = p->wfn_anom[2 * w]; anom.im = p->wfn_anom[2 * w + 1]; }
                else { anom.re = 0.0; anom.im = 0.0; }
                int lmax_use = -1, lmax_par = -1;
                double fsph = 0.0;
                const double *P = NULL;
                if (p->model == SFO_MODEL_HC) {
                    fsph = fcore[w] + fval[ty] * p->type_pval[ty];
                    lmax_use = type_lmax_used(p, ty, w);
                    lmax_par = type_lmax_params(p, ty, w);
                    P = p->type_plm + 25 * ty;
                } else if (p->model == SFO_MODEL_IAM) {
                    fsph = fval[ty];
                }
                cplx U = {0, 0};          /* sum_s f e^{i theta} T_s */
                cplx Ex = {0, 0};         /* sum_s e^{i theta} T_s (for P_val, kappa) */
                cplx X[3] = {{0, 0}, {0, 0}, {0, 0}};
                cplx Ad[6] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
                cplx Pd[25];
                cplx Kp = {0, 0};
                for (int q = 0; q < 25; q++) { Pd[q].re = 0; Pd[q].im = 0; }
                for (int s = 0; s < nS; s++) {
                    const double *hs = hr + 3 * s;
                    const double th = 2.0 * PI * (hs[0] * pos[0] + hs[1] * pos[1] + hs[2] * pos[2] + tf[s]);
                    cplx e = {cos(th), sin(th)};
                    double T = 1.0, mlt[6];
                    if (nadp == 6) {
                        mlt[0] = hs[0] * hs[0]; mlt[1] = hs[1] * hs[1]; mlt[2] = hs[2] * hs[2];
                        mlt[3] = 2.0 * hs[0] * hs[1]; mlt[4] = 2.0 * hs[0] * hs[2]; mlt[5] = 2.0 * hs[1] * hs[2];
                        T = exp(-mlt[0] * adp[0] - mlt[1] * adp[1] - mlt[2] * adp[2]
                                - mlt[3] * adp[3] - mlt[4] * adp[4] - mlt[5] * adp[5]);
                    }
                    cplx f = {fsph + anom.re, anom.im};
                    double d[25];
                    int have_d = 0;
                    if (p->model == SFO_MODEL_TABLE) {
                        const double *tb = p->table + 2 * (((size_t)ih * nS + s) * nA + a);
                        f.re = tb[0] + anom.re; f.im = tb[1] + anom.im;
                    } else if (p->model == SFO_MODEL_HC && !h000 && lmax_par >= 0) {
                        /* unit vector of the rotated h in the atom's local frame */
                        double u[3];
                        for (int j = 0; j < 3; j++)
                            u[j] = (L[0 + j] * hs[0] + L[3 + j] * hs[1] + L[6 + j] * hs[2]) / hl;
                        sfo_dlm(u, d);
                        have_d = 1;
                        cplx fd = {0, 0};
                        for (int l = 0; l <= lmax_use; l++) {
                            double ang = 0.0;
                            for (int m = 0; m < 2 * l + 1; m++) ang += P[l * l + m] * d[l * l + m];
                            fd = cadd(fd, cscale(IPOW[l], 4.0 * PI * gl[ty * 5 + l] * ang));
                        }
                        f = cadd(f, fd);
                    }
                    if (p->electron && p->model == SFO_MODEL_HC) {
                        if (h000) { f.re = p->wfn_f000[w] + anom.re; f.im = anom.im; }
                        else {
                            f.re = esc * (f.re - anom.re) - esc * p->wfn_z[w] + anom.re;
                            f.im = esc * (f.im - anom.im) + anom.im;
                        }
                    }
                    cplx eT = cscale(e, T);
                    cplx u_s = cmul(f, eT);
                    U = cadd(U, u_s);
                    if (nadp == 6)
                        for (int k = 0; k < 6; k++) Ad[k] = cadd(Ad[k], cscale(u_s, -mlt[k]));
                    for (int j = 0; j < 3; j++) X[j] = cadd(X[j], cscale(u_s, hs[j]));
                    if (p->d_mp && p->model == SFO_MODEL_HC) {
                        Ex = cadd(Ex, eT);
                        if (have_d) {
                            for (int l = 0; l <= lmax_par; l++)
                                for (int m = 0; m < 2 * l + 1; m++)
                                    Pd[l * l + m] = cadd(Pd[l * l + m],
                                        cmul(IPOW[l], cscale(eT, 4.0 * PI * gl[ty * 5 + l] * d[l * l + m])));
                            cplx kd = {0, 0};
                            for (int l = 0; l <= lmax_use; l++) {
                                double ang = 0.0;
                                for (int m = 0; m < 2 * l + 1; m++) ang += P[l * l + m] * d[l * l + m];
                                kd = cadd(kd, cscale(IPOW[l], 4.0 * PI * dgl[ty * 5 + l] * ang));
                            }
                            Kp = cadd(Kp, cmul(kd, eT));
                        }
                    }
                }
                double Tiso = 1.0;
                if (nadp == 1) {
                    Tiso = exp(-h2 * adp[0]);
                    U = cscale(U, Tiso);
                    for (int j = 0; j < 3; j++) X[j] = cscale(X[j], Tiso);
                    Ex = cscale(Ex, Tiso);
                    for (int q = 0; q < 25; q++) Pd[q] = cscale(Pd[q], Tiso);
                    Kp = cscale(Kp, Tiso);
                }
                /* forward: F = sum_a w U (+ c conj for centrosymmetric, applied after the atom loop) */
                Ftot = cadd(Ftot, cscale(U, wgt));
                /* adjoint: dT/dp = Re(g_eff * dU/dp) with the engine's scalings */
                double *Aa = A + (size_t)a * NCH;
                if (p->d_occ) Aa[CH_OCC] += cmul(ge, U).re * p->mult_w[a];
                if (p->d_adp) {
                    if (nadp == 1) Aa[CH_ADP] += -h2 * cmul(ge, U).re * 2.0 * PI * PI * wgt;
                    else if (nadp == 6)
                        for (int k = 0; k < 6; k++) Aa[CH_ADP + k] += cmul(ge, Ad[k]).re * 2.0 * PI * PI * wgt;
                }
                if (p->d_xyz)
                    for (int j = 0; j < 3; j++)
                        Aa[CH_XYZ + j] += -cmul(ge, X[j]).im * 2.0 * PI * wgt;
                if (p->d_mp && p->model == SFO_MODEL_HC) {
                    Aa[CH_PV] += cmul(ge, cscale(Ex, esc * fval[ty])).re * wgt;
                    Aa[CH_K] += cmul(ge, cscale(Ex, esc * p->type_pval[ty] * dfval[ty])).re * wgt;
                    for (int q = 0; q < 25; q++) Aa[CH_PLM + q] += esc * cmul(ge, Pd[q]).re * wgt;
                    Aa[CH_KP] += esc * cmul(ge, Kp).re * wgt;
                }
            }
            if (p->centro) {
                if (at_origin) { Ftot.re = 2.0 * Ftot.re; Ftot.im = 0.0; }
                else Ftot = cadd(Ftot, cmul(cinv, cconj(Ftot)));
            }
            r->f[2 * ih] = Ftot.re;
            r->f[2 * ih + 1] = Ftot.im;
        }
        free(fcore); free(fval); free(dfval); free(gl); free(dgl); free(hr); free(tf);
    }
    /* merge per-thread buffers */
    for (int a = 0; a < nA; a++) {
        double s[NCH];
        for (int c = 0; c < NCH; c++) s[c] = 0.0;
        for (int t = 0; t < n_threads; t++)
            for (int c = 0; c < NCH; c++) s[c] += acc[((size_t)t * nA + a) * NCH + c];
        if (r->d_xyz) for (int j = 0; j < 3; j++) r->d_xyz[3 * a + j] = s[CH_XYZ + j];
        if (r->d_adp) for (int j = 0; j < 6; j++) r->d_adp[6 * a + j] = s[CH_ADP + j];
        if (r->d_occ) r->d_occ[a] = s[CH_OCC];
        if (r->d_pval) r->d_pval[a] = s[CH_PV];
        if (r->d_plm) for (int j = 0; j < 25; j++) r->d_plm[25 * a + j] = s[CH_PLM + j];
        if (r->d_kappa) r->d_kappa[a] = s[CH_K];
        if (r->d_kappa_p) r->d_kappa_p[a] = s[CH_KP];
    }
    free(acc);
    free(type_wfn);
    return 0;
}

/* ========================================================================
 * Line-ordered evaluation of the HC model: the reference engine's own loop
 * structure (HansenCoppens_SF_Engine3::calculateSF_Serial*, src/Scattering/
 * HansenCoppens_SF_Engine3.cpp:1030-1509, 1511-1992, 2649-2894):
 *   - reflections grouped in lattice lines (h, k, l), (h, k, l+1), ...
 *     (scattering_utilities::splitHklLines, src/Scattering/scattering_utilities.cpp:463-517);
 *   - per line: h' = h R and h.t per (reflection, operation), the harmonics of
 *     h' in the crystal frame, the radial terms per (reflection, type);
 *   - per (atom, operation): the phase factor and the anisotropic temperature
 *     factor by recurrences along the line (calculate_line_phase_factors,
 *     calculate_line_temperature_factors, scattering_utilities.cpp:575-756),
 *     re-anchored every 32 reflections;
 *   - P_lm rotated once per atom to the crystal frame
 *     (calculateGlobalCoordinatesPlm, HansenCoppens_SF_Engine3.cpp:594-654),
 *     here by a least-squares fit of the rotated harmonics over 40 directions.
 * The CPU baseline of the benchmark; the same sums as sfo_compute.
 * ======================================================================== */
#define FIT_K 40
static double fit_u[FIT_K][3];
static double fit_pinv[5][9 * FIT_K];
static int fit_ready = 0;

static void fit_init(void)
{
    if (fit_ready) return;
    const double ga = PI * (3.0 - sqrt(5.0));
    for (int k = 0; k < FIT_K; k++) {
        const double z = 1.0 - (2.0 * k + 1.0) / FIT_K, rr = sqrt(1.0 - z * z);
        fit_u[k][0] = rr * cos(ga * k);
        fit_u[k][1] = rr * sin(ga * k);
        fit_u[k][2] = z;
    }
    for (int l = 0; l <= 4; l++) {
        const int n = 2 * l + 1;
        double A[FIT_K * 9], M[9 * 18];
        for (int k = 0; k < FIT_K; k++) {
            double v[25];
            sfo_dlm(fit_u[k], v);
            for (int m = 0; m < n; m++) A[k * n + m] = v[l * l + m];
        }
        /* [A^T A | I] -> [I | (A^T A)^-1] by Gauss-Jordan */
        for (int i = 0; i < n; i++)
            for (int j = 0; j < 2 * n; j++) {
                double s = 0.0;
                if (j < n)
                    for (int k = 0; k < FIT_K; k++) s += A[k * n + i] * A[k * n + j];
                else
                    s = (j - n == i) ? 1.0 : 0.0;
                M[i * 2 * n + j] = s;
            }
        for (int c = 0; c < n; c++) {
            int piv = c;
            for (int i = c + 1; i < n; i++)
                if (fabs(M[i * 2 * n + c]) > fabs(M[piv * 2 * n + c])) piv = i;
            for (int j = 0; j < 2 * n; j++) {
                double t = M[c * 2 * n + j];
                M[c * 2 * n + j] = M[piv * 2 * n + j];
                M[piv * 2 * n + j] = t;
            }
            const double d = M[c * 2 * n + c];
            for (int j = 0; j < 2 * n; j++) M[c * 2 * n + j] /= d;
            for (int i = 0; i < n; i++)
                if (i != c) {
                    const double f = M[i * 2 * n + c];
                    for (int j = 0; j < 2 * n; j++) M[i * 2 * n + j] -= f * M[c * 2 * n + j];
                }
        }
        /* pinv = (A^T A)^-1 A^T : [n][K] */
        for (int i = 0; i < n; i++)
            for (int k = 0; k < FIT_K; k++) {
                double s = 0.0;
                for (int j = 0; j < n; j++) s += M[i * 2 * n + n + j] * A[k * n + j];
                fit_pinv[l][i * FIT_K + k] = s;
            }
    }
    fit_ready = 1;
}

/* D_l blocks (165 values, [i][j] per l) with d(L^T u) = D d(u) (L: columns = local axes) */
static void rotation_blocks_cpu(const double *L, double *D)
{
    double B[FIT_K][25];
    for (int k = 0; k < FIT_K; k++) {
        double v[3];
        for (int j = 0; j < 3; j++) v[j] = L[0 + j] * fit_u[k][0] + L[3 + j] * fit_u[k][1] + L[6 + j] * fit_u[k][2];
        sfo_dlm(v, B[k]);
    }
    int off = 0;
    for (int l = 0; l <= 4; l++) {
        const int n = 2 * l + 1;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double s = 0.0;
                for (int k = 0; k < FIT_K; k++) s += fit_pinv[l][j * FIT_K + k] * B[k][l * l + i];
                D[off + i * n + j] = s;
            }
        off += n * n;
    }
}

typedef struct { int h, k, l, idx; } hkl_key;
static int hkl_cmp(const void *a, const void *b)
{
    const hkl_key *x = (const hkl_key *)a, *y = (const hkl_key *)b;
    if (x->h != y->h) return x->h < y->h ? -1 : 1;
    if (x->k != y->k) return x->k < y->k ? -1 : 1;
    if (x->l != y->l) return x->l < y->l ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

int sfo_compute_lines(const sfo_problem *p, const int *hkl, const double *b3, sfo_result *r, int n_threads)
{
    if (p->model != SFO_MODEL_HC) return 2;
    g_init();
    fit_init();
    const int nA = p->n_atoms, nH = p->n_hkl, nS = p->n_sym, nT = p->n_types > 0 ? p->n_types : 1;
    const int nW = p->n_wfn > 0 ? p->n_wfn : 1;
    if (n_threads < 1) n_threads = 1;
#ifndef _OPENMP
    n_threads = 1;
#endif
    /* lines */
    hkl_key *key = (hkl_key *)malloc(sizeof(hkl_key) * (nH > 0 ? nH : 1));
    for (int i = 0; i < nH; i++) {
        key[i].h = hkl[3 * i]; key[i].k = hkl[3 * i + 1]; key[i].l = hkl[3 * i + 2]; key[i].idx = i;
    }
    qsort(key, nH, sizeof(hkl_key), hkl_cmp);
    int *line_start = (int *)malloc(sizeof(int) * (nH + 1));
    int n_lines = 0, max_len = 1;
    for (int i = 0; i < nH; i++) {
        const int cont = i > 0 && key[i].h == key[i - 1].h && key[i].k == key[i - 1].k && key[i].l == key[i - 1].l + 1;
        if (!cont) line_start[n_lines++] = i;
    }
    line_start[n_lines] = nH;
    for (int q = 0; q < n_lines; q++)
        if (line_start[q + 1] - line_start[q] > max_len) max_len = line_start[q + 1] - line_start[q];
    /* one contiguous share of the ordered reflections per thread, lines cut at the share boundaries (the
     * reference's splitHklLines, scattering_utilities.cpp:463-513): segments [seg_i0, seg_i0 + seg_len),
     * thread c takes segments share[c] .. share[c + 1] - 1 */
    int *seg_i0 = (int *)malloc(sizeof(int) * (n_lines + n_threads + 1));
    int *seg_len = (int *)malloc(sizeof(int) * (n_lines + n_threads + 1));
    int *share = (int *)malloc(sizeof(int) * (n_threads + 1));
    int n_seg = 0;
    {
        int q = 0;
        for (int c = 0; c < n_threads; c++) {
            const int b0 = (int)((long long)nH * c / n_threads), b1 = (int)((long long)nH * (c + 1) / n_threads);
            share[c] = n_seg;
            while (q < n_lines && line_start[q + 1] <= b0) q++;
            for (int k = q; k < n_lines && line_start[k] < b1; k++) {
                const int i0 = line_start[k] > b0 ? line_start[k] : b0;
                const int i1 = line_start[k + 1] < b1 ? line_start[k + 1] : b1;
                if (i1 > i0) {
                    seg_i0[n_seg] = i0;
                    seg_len[n_seg] = i1 - i0;
                    n_seg++;
                }
            }
        }
        share[n_threads] = n_seg;
    }
    /* per atom: crystal-frame P_lm and rotation blocks */
    int *type_wfn = (int *)malloc(sizeof(int) * nT);
    for (int t = 0; t < nT; t++) type_wfn[t] = 0;
    for (int a = 0; a < nA; a++) /* HC types only: the other models carry no per-type wavefunctions */
        if (p->model == SFO_MODEL_HC && p->atom_type[a] >= 0 && p->atom_type[a] < p->n_types)
            type_wfn[p->atom_type[a]] = p->atom_wfn[a];
    double *pg = (double *)calloc((size_t)nA * 25, sizeof(double));
    double *Dm = (double *)calloc((size_t)nA * 165, sizeof(double));
    int *lmu = (int *)malloc(sizeof(int) * nA), *lmp = (int *)malloc(sizeof(int) * nA);
    for (int a = 0; a < nA; a++) {
        const int t = p->atom_type[a], w = p->atom_wfn[a];
        lmu[a] = type_lmax_used(p, t, w);
        lmp[a] = type_lmax_params(p, t, w);
        rotation_blocks_cpu(p->lcs + 9 * a, Dm + 165 * (size_t)a);
        int off = 0;
        for (int l = 0; l <= 4; l++) {
            const int n = 2 * l + 1;
            if (l <= lmu[a])
                for (int j = 0; j < n; j++) {
                    double v = 0.0;
                    for (int i = 0; i < n; i++) v += Dm[165 * (size_t)a + off + i * n + j] * p->type_plm[25 * t + l * l + i];
                    pg[25 * (size_t)a + l * l + j] = v;
                }
            off += n * n;
        }
    }
    double *acc = (double *)calloc((size_t)n_threads * nA * NCH, sizeof(double));
    const int at_origin = p->inv_trans[0] == 0.0 && p->inv_trans[1] == 0.0 && p->inv_trans[2] == 0.0;

#pragma omp parallel num_threads(n_threads)
    {
#ifdef _OPENMP
        const int tid = omp_get_thread_num();
#else
        const int tid = 0;
#endif
        double *A = acc + (size_t)tid * nA * NCH;
        const size_t L = (size_t)max_len;
        double *hr = (double *)malloc(sizeof(double) * L * nS * 3);
        double *tf = (double *)malloc(sizeof(double) * L * nS);
        double *dd = (double *)malloc(sizeof(double) * L * nS * 25);
        double *h2v = (double *)malloc(sizeof(double) * L);
        double *fcore = (double *)malloc(sizeof(double) * L * nW);
        double *fval = (double *)malloc(sizeof(double) * L * nT), *dfval = (double *)malloc(sizeof(double) * L * nT);
        double *gl = (double *)malloc(sizeof(double) * L * nT * 5), *dgl = (double *)malloc(sizeof(double) * L * nT * 5);
        cplx *gev = (cplx *)malloc(sizeof(cplx) * L), *Fl = (cplx *)malloc(sizeof(cplx) * L);
        cplx *cinvv = (cplx *)malloc(sizeof(cplx) * L);
        cplx *e = (cplx *)malloc(sizeof(cplx) * nS), *st = (cplx *)malloc(sizeof(cplx) * nS);
        double *Tn = (double *)malloc(sizeof(double) * nS), *Tr = (double *)malloc(sizeof(double) * nS);
        double *Trho = (double *)malloc(sizeof(double) * nS);
        int *is000 = (int *)malloc(sizeof(int) * L);

#pragma omp for schedule(static, 1)
        for (int c = 0; c < n_threads; c++)
        for (int q = share[c]; q < share[c + 1]; q++) {
            const int i0 = seg_i0[q], len = seg_len[q];
            for (int j = 0; j < len; j++) {
                const double *h = p->h + 3 * key[i0 + j].idx;
                const double h2 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2], hl = sqrt(h2);
                h2v[j] = h2;
                is000[j] = hl < 1e-10;
                for (int s = 0; s < nS; s++) {
                    const double *R = p->rot + 9 * s, *t = p->trans + 3 * s;
                    double *x = hr + ((size_t)j * nS + s) * 3;
                    for (int c = 0; c < 3; c++) x[c] = h[0] * R[c] + h[1] * R[3 + c] + h[2] * R[6 + c];
                    tf[(size_t)j * nS + s] = h[0] * t[0] + h[1] * t[1] + h[2] * t[2];
                    double *d = dd + ((size_t)j * nS + s) * 25;
                    if (!is000[j]) {
                        const double u[3] = {x[0] / hl, x[1] / hl, x[2] / hl};
                        sfo_dlm(u, d);
                    } else {
                        for (int c = 0; c < 25; c++) d[c] = 0.0;
                    }
                }
                for (int w = 0; w < p->n_wfn; w++) {
                    double s = 0.0;
                    for (int k = p->core_off[w]; k < p->core_off[w + 1]; k++)
                        s += p->core_coeff[k] * sfo_g(0, p->core_pow[k] + 2, hl, p->core_exp[k]);
                    fcore[(size_t)j * nW + w] = 4.0 * PI * s;
                }
                for (int ty = 0; ty < p->n_types; ty++) {
                    const int w = type_wfn[ty];
                    const double kap = p->type_kappa[ty], kp = p->type_kappa_p[ty];
                    double s = 0.0, ds = 0.0;
                    for (int k = p->val_off[w]; k < p->val_off[w + 1]; k++) {
                        s += p->val_coeff[k] * sfo_g(0, p->val_pow[k] + 2, hl / kap, p->val_exp[k]);
                        if (p->d_mp) ds += p->val_coeff[k] * g_dh(0, p->val_pow[k] + 2, hl / kap, p->val_exp[k]);
                    }
                    fval[(size_t)j * nT + ty] = 4.0 * PI * s;
                    dfval[(size_t)j * nT + ty] = 4.0 * PI * ds * (-hl / (kap * kap));
                    const double zeta = p->def_exp[w];
                    for (int l = 0; l < 5; l++) {
                        double gv = 0.0, dg = 0.0;
                        if (l < p->def_npow[w]) {
                            const int nl = p->def_pow[w * 5 + l];
                            double norm = pow(zeta, nl + 3);
                            for (int c = 2; c <= nl + 2; c++) norm /= c;
                            gv = norm * sfo_g(l, nl + 2, hl / kp, zeta);
                            if (p->d_mp) dg = norm * g_dh(l, nl + 2, hl / kp, zeta) * (-hl / (kp * kp));
                        }
                        gl[((size_t)j * nT + ty) * 5 + l] = gv;
                        dgl[((size_t)j * nT + ty) * 5 + l] = dg;
                    }
                }
                const cplx g = {p->dtdf[2 * key[i0 + j].idx], p->dtdf[2 * key[i0 + j].idx + 1]};
                const double ph_inv = 2.0 * PI * (h[0] * p->inv_trans[0] + h[1] * p->inv_trans[1] + h[2] * p->inv_trans[2]);
                cinvv[j].re = cos(ph_inv);
                cinvv[j].im = sin(ph_inv);
                cplx ge = g;
                if (p->centro) {
                    if (at_origin) { ge.re = 2.0 * g.re; ge.im = 0.0; }
                    else ge = cadd(g, cconj(cmul(g, cinvv[j])));
                }
                gev[j] = ge;
                Fl[j].re = Fl[j].im = 0.0;
            }
            const double *h0 = p->h + 3 * key[i0].idx;
            for (int a = 0; a < nA; a++) {
                if (!p->include[a]) continue;
                const int w = p->atom_wfn[a], ty = p->atom_type[a], nadp = p->n_adp[a];
                const double wgt = p->occ[a] * p->mult_w[a];
                const double *adp = p->adp + 6 * a, *pos = p->pos + 3 * a, *P = pg + 25 * (size_t)a;
                const double U[9] = {adp[0], adp[3], adp[4], adp[3], adp[1], adp[5], adp[4], adp[5], adp[2]};
                cplx anom;
                if (p->atom_anom) { anom.re = p->atom_anom[2 * a]; anom.im = p->atom_anom[2 * a + 1]; }
                else { anom.re = p->wfn_anom[2 * w]; anom.im = p->wfn_anom[2 * w + 1]; }
                double *Aa = A + (size_t)a * NCH;
                for (int j = 0; j < len; j++) {
                    cplx Us = {0, 0}, Ex = {0, 0}, Kp = {0, 0};
                    cplx X[3] = {{0, 0}, {0, 0}, {0, 0}}, Ad[6] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
                    cplx Pd[25];
                    if (p->d_mp)
                        for (int c = 0; c < 25; c++) Pd[c].re = Pd[c].im = 0.0;
                    const double fsph = fcore[(size_t)j * nW + w] + fval[(size_t)j * nT + ty] * p->type_pval[ty];
                    const double esc = p->electron ? (is000[j] ? 0.0 : -0.023934 / (0.25 * h2v[j])) : 1.0;
                    for (int s = 0; s < nS; s++) {
                        const double *hs = hr + ((size_t)j * nS + s) * 3;
                        /* phase and temperature factor: exact at the line start and every 32 reflections,
                         * otherwise one step of the recurrences */
                        if (j % 32 == 0) {
                            const double th = 2.0 * PI * (hs[0] * pos[0] + hs[1] * pos[1] + hs[2] * pos[2] + tf[(size_t)j * nS + s]);
                            e[s].re = cos(th); e[s].im = sin(th);
                            if (j == 0) {
                                const double *R = p->rot + 9 * s, *t = p->trans + 3 * s;
                                double d3[3];
                                for (int c = 0; c < 3; c++) d3[c] = b3[0] * R[c] + b3[1] * R[3 + c] + b3[2] * R[6 + c];
                                const double ps = 2.0 * PI * (d3[0] * pos[0] + d3[1] * pos[1] + d3[2] * pos[2] +
                                                              b3[0] * t[0] + b3[1] * t[1] + b3[2] * t[2]);
                                st[s].re = cos(ps); st[s].im = sin(ps);
                                if (nadp == 6) {
                                    double Ud[3];
                                    for (int c = 0; c < 3; c++) Ud[c] = U[3 * c] * d3[0] + U[3 * c + 1] * d3[1] + U[3 * c + 2] * d3[2];
                                    Trho[s] = exp(-2.0 * (d3[0] * Ud[0] + d3[1] * Ud[1] + d3[2] * Ud[2]));
                                }
                            }
                            if (nadp == 6) {
                                const double *R = p->rot + 9 * s;
                                double d3[3], Uh[3], Ud[3];
                                for (int c = 0; c < 3; c++) d3[c] = b3[0] * R[c] + b3[1] * R[3 + c] + b3[2] * R[6 + c];
                                for (int c = 0; c < 3; c++) {
                                    Uh[c] = U[3 * c] * hs[0] + U[3 * c + 1] * hs[1] + U[3 * c + 2] * hs[2];
                                    Ud[c] = U[3 * c] * d3[0] + U[3 * c + 1] * d3[1] + U[3 * c + 2] * d3[2];
                                }
                                Tn[s] = exp(-(hs[0] * Uh[0] + hs[1] * Uh[1] + hs[2] * Uh[2]));
                                Tr[s] = exp(-(2.0 * (hs[0] * Ud[0] + hs[1] * Ud[1] + hs[2] * Ud[2]) +
                                              (d3[0] * Ud[0] + d3[1] * Ud[1] + d3[2] * Ud[2])));
                            }
                        }
                        const cplx es = e[s];
                        const double T = nadp == 6 ? Tn[s] : 1.0;
                        /* advance to the next reflection of the line */
                        e[s] = cmul(e[s], st[s]);
                        if (nadp == 6) { Tn[s] *= Tr[s]; Tr[s] *= Trho[s]; }
                        cplx f = {fsph + anom.re, anom.im};
                        const double *d = dd + ((size_t)j * nS + s) * 25;
                        double ang[5] = {0, 0, 0, 0, 0};
                        if (!is000[j] && lmp[a] >= 0) {
                            cplx fd = {0, 0};
                            for (int l = 0; l <= lmu[a]; l++) {
                                double sum = 0.0;
                                for (int m = 0; m < 2 * l + 1; m++) sum += P[l * l + m] * d[l * l + m];
                                ang[l] = sum;
                                fd = cadd(fd, cscale(IPOW[l], 4.0 * PI * gl[((size_t)j * nT + ty) * 5 + l] * sum));
                            }
                            f = cadd(f, fd);
                        }
                        if (p->electron) {
                            if (is000[j]) { f.re = p->wfn_f000[w] + anom.re; f.im = anom.im; }
                            else {
                                f.re = esc * (f.re - anom.re) - esc * p->wfn_z[w] + anom.re;
                                f.im = esc * (f.im - anom.im) + anom.im;
                            }
                        }
                        const cplx eT = cscale(es, T);
                        const cplx u = cmul(f, eT);
                        Us = cadd(Us, u);
                        if (nadp == 6) {
                            const double m6[6] = {hs[0] * hs[0], hs[1] * hs[1], hs[2] * hs[2], 2.0 * hs[0] * hs[1],
                                                  2.0 * hs[0] * hs[2], 2.0 * hs[1] * hs[2]};
                            for (int c = 0; c < 6; c++) Ad[c] = cadd(Ad[c], cscale(u, -m6[c]));
                        }
                        for (int c = 0; c < 3; c++) X[c] = cadd(X[c], cscale(u, hs[c]));
                        if (p->d_mp) {
                            Ex = cadd(Ex, eT);
                            if (!is000[j] && lmp[a] >= 0) {
                                for (int l = 0; l <= lmp[a]; l++)
                                    for (int m = 0; m < 2 * l + 1; m++)
                                        Pd[l * l + m] = cadd(Pd[l * l + m],
                                            cmul(IPOW[l], cscale(eT, 4.0 * PI * gl[((size_t)j * nT + ty) * 5 + l] * d[l * l + m])));
                                cplx kd = {0, 0};
                                for (int l = 0; l <= lmu[a]; l++)
                                    kd = cadd(kd, cscale(IPOW[l], 4.0 * PI * dgl[((size_t)j * nT + ty) * 5 + l] * ang[l]));
                                Kp = cadd(Kp, cmul(kd, eT));
                            }
                        }
                    }
                    if (nadp == 1) {
                        const double Ti = exp(-h2v[j] * adp[0]);
                        Us = cscale(Us, Ti);
                        for (int c = 0; c < 3; c++) X[c] = cscale(X[c], Ti);
                        Ex = cscale(Ex, Ti);
                        if (p->d_mp)
                            for (int c = 0; c < 25; c++) Pd[c] = cscale(Pd[c], Ti);
                        Kp = cscale(Kp, Ti);
                    }
                    Fl[j] = cadd(Fl[j], cscale(Us, wgt));
                    const cplx ge = gev[j];
                    if (p->d_occ) Aa[CH_OCC] += cmul(ge, Us).re * p->mult_w[a];
                    if (p->d_adp) {
                        if (nadp == 1) Aa[CH_ADP] += -h2v[j] * cmul(ge, Us).re * 2.0 * PI * PI * wgt;
                        else if (nadp == 6)
                            for (int c = 0; c < 6; c++) Aa[CH_ADP + c] += cmul(ge, Ad[c]).re * 2.0 * PI * PI * wgt;
                    }
                    if (p->d_xyz)
                        for (int c = 0; c < 3; c++) Aa[CH_XYZ + c] += -cmul(ge, X[c]).im * 2.0 * PI * wgt;
                    if (p->d_mp) {
                        Aa[CH_PV] += cmul(ge, cscale(Ex, esc * fval[(size_t)j * nT + ty])).re * wgt;
                        Aa[CH_K] += cmul(ge, cscale(Ex, esc * p->type_pval[ty] * dfval[(size_t)j * nT + ty])).re * wgt;
                        for (int c = 0; c < 25; c++) Aa[CH_PLM + c] += esc * cmul(ge, Pd[c]).re * wgt;  /* crystal frame */
                        Aa[CH_KP] += esc * cmul(ge, Kp).re * wgt;
                    }
                }
            }
            for (int j = 0; j < len; j++) {
                cplx F = Fl[j];
                if (p->centro) {
                    if (at_origin) { F.re = 2.0 * F.re; F.im = 0.0; }
                    else F = cadd(F, cmul(cinvv[j], cconj(F)));
                }
                r->f[2 * key[i0 + j].idx] = F.re;
                r->f[2 * key[i0 + j].idx + 1] = F.im;
            }
            (void)h0;
        }
        free(hr); free(tf); free(dd); free(h2v); free(fcore); free(fval); free(dfval); free(gl); free(dgl);
        free(gev); free(Fl); free(cinvv); free(e); free(st); free(Tn); free(Tr); free(Trho); free(is000);
    }
    for (int a = 0; a < nA; a++) {
        double s[NCH];
        for (int c = 0; c < NCH; c++) s[c] = 0.0;
        for (int t = 0; t < n_threads; t++)
            for (int c = 0; c < NCH; c++) s[c] += acc[((size_t)t * nA + a) * NCH + c];
        if (r->d_xyz) for (int j = 0; j < 3; j++) r->d_xyz[3 * a + j] = s[CH_XYZ + j];
        if (r->d_adp) for (int j = 0; j < 6; j++) r->d_adp[6 * a + j] = s[CH_ADP + j];
        if (r->d_occ) r->d_occ[a] = s[CH_OCC];
        if (r->d_pval) r->d_pval[a] = s[CH_PV];
        if (r->d_kappa) r->d_kappa[a] = s[CH_K];
        if (r->d_kappa_p) r->d_kappa_p[a] = s[CH_KP];
        if (r->d_plm) {  /* back to the local frame: dT/dP_local = D dT/dP_glob, zero above the parameters' l */
            const double *D = Dm + 165 * (size_t)a;
            int off = 0;
            for (int l = 0; l <= 4; l++) {
                const int n = 2 * l + 1;
                for (int i = 0; i < n; i++) {
                    double v = 0.0;
                    for (int j = 0; j < n; j++) v += D[off + i * n + j] * s[CH_PLM + l * l + j];
                    r->d_plm[25 * a + l * l + i] = l <= lmp[a] ? v : 0.0;
                }
                off += n * n;
            }
        }
    }
    free(acc); free(pg); free(Dm); free(lmu); free(lmp); free(type_wfn); free(key); free(line_start);
    free(seg_i0); free(seg_len); free(share);
    return 0;
}
