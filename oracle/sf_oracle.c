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
    for (int a = 0; a < nA; a++) type_wfn[p->atom_type[a]] = p->atom_wfn[a];

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
            /* radial terms per wavefunction / type */
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
                    for (int q = 0; q < p->iam_ngauss[ty]; q++)
                        s += p->iam_a[ty * 5 + q] * exp(-p->iam_b[ty * 5 + q] * x2);
                    fval[ty] = s;
                }
            }
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
                    Aa[CH_PV] += cmul(ge, cscale(Ex, fval[ty])).re * wgt;
                    Aa[CH_K] += cmul(ge, cscale(Ex, p->type_pval[ty] * dfval[ty])).re * wgt;
                    for (int q = 0; q < 25; q++) Aa[CH_PLM + q] += cmul(ge, Pd[q]).re * wgt;
                    Aa[CH_KP] += cmul(ge, Kp).re * wgt;
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
