// Device/host math shared by the structure-factor kernels.
//
//  * density-normalised real spherical harmonics d_lm, l <= 4, in the
//    ordering and polynomial form of real_spherical_harmonics::getPolynomials
//    (include/discamb/MathUtilities/real_spherical_harmonics.h:136-190);
//  * Slater-function Fourier-Bessel integrals
//      G(n,l,K,Z) = int_0^inf r^n e^{-Zr} j_l(Kr) dr
//    (the quantity sto_scattering::gFunction returns,
//    include/discamb/Scattering/SlaterTypeOrbitalScattering.h:51-183) in a
//    cancellation-free form: with rho^2 = Z^2 + K^2, c = Z/rho, s = K/rho and
//    m = n - l - 1,
//      G = 2^l l! m! s^l C_m^{(l+1)}(c) / rho^{n+1},
//    C_m^{(lambda)} the Gegenbauer polynomial, from
//    G(l+1,l) = (2K)^l l!/rho^{2l+2}, G(n+1,l) = -dG(n,l)/dZ and the
//    Gegenbauer generating function.  The three-term recurrence for C_m is
//    stable on [0,1], so the same code is accurate in FP32 (the expanded
//    polynomial with coefficients up to 1e8 is not).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define DSF_PI 3.14159265358979323846
#define DSF_HD __host__ __device__ __forceinline__

namespace dsf {

// (2 - delta_l0) / int |y_lm| dOmega  (Paturle & Coppens 1988), l*l + m + l
__device__ __constant__ double kDensityNorm[25] = {
    0.07957747154594767,
    0.3183098861837907, 0.3183098861837907, 0.3183098861837907,
    0.75, 0.75, 0.2067483357831728, 0.75, 0.375,
    0.4244131815783876, 2.0, 0.3203330895838574, 0.2448537586029175, 0.3203330895838574, 1.0,
    0.4244131815783876,
    1.875, 1.25, 0.6611826845788106, 0.4740025188689597, 0.06941752438437611, 0.4740025188689597,
    0.3305913422894053, 1.25, 0.46875};

static const double kDensityNormHost[25] = {
    0.07957747154594767,
    0.3183098861837907, 0.3183098861837907, 0.3183098861837907,
    0.75, 0.75, 0.2067483357831728, 0.75, 0.375,
    0.4244131815783876, 2.0, 0.3203330895838574, 0.2448537586029175, 0.3203330895838574, 1.0,
    0.4244131815783876,
    1.875, 1.25, 0.6611826845788106, 0.4740025188689597, 0.06941752438437611, 0.4740025188689597,
    0.3305913422894053, 1.25, 0.46875};

// harmonic polynomials (unnormalised) of a unit vector, 25 values
template <typename R>
DSF_HD void harmonic_polys(R x, R y, R z, R *v)
{
    const R xx = x * x, yy = y * y, zz = z * z;
    const R xy = x * y, xz = x * z, yz = y * z;
    v[0] = R(1);
    v[1] = y; v[2] = z; v[3] = x;
    v[4] = xy; v[5] = yz; v[6] = R(2) * zz - xx - yy; v[7] = xz; v[8] = xx - yy;
    v[9] = (R(3) * xx - yy) * y; v[10] = xy * z; v[11] = y * (R(4) * zz - xx - yy);
    v[12] = z * (R(2) * zz - R(3) * xx - R(3) * yy); v[13] = x * (R(4) * zz - xx - yy);
    v[14] = (xx - yy) * z; v[15] = (xx - R(3) * yy) * x;
    v[16] = xy * (xx - yy); v[17] = (R(3) * xx - yy) * yz; v[18] = xy * (R(7) * zz - R(1));
    v[19] = yz * (R(7) * zz - R(3)); v[20] = (R(35) * zz - R(30)) * zz + R(3); v[21] = xz * (R(7) * zz - R(3));
    v[22] = (xx - yy) * (R(7) * zz - R(1)); v[23] = (xx - R(3) * yy) * xz;
    v[24] = xx * (xx - R(3) * yy) - yy * (R(3) * xx - yy);
}

// 2^l l! m! for l <= 5, m <= 11
DSF_HD double g_prefactor(int l, int m)
{
    double p = 1.0;
    for (int k = 1; k <= l; k++) p *= 2.0 * k;
    for (int k = 2; k <= m; k++) p *= k;
    return p;
}

template <typename R>
DSF_HD R rsqrt_(R x);
template <>
DSF_HD float rsqrt_<float>(float x)
{
#ifdef __CUDA_ARCH__
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}
template <>
DSF_HD double rsqrt_<double>(double x) { return 1.0 / sqrt(x); }

// G(n,l,K,Z); n >= l+1
template <typename R>
DSF_HD R gfun(int l, int n, R K, R Z)
{
    const R irho = rsqrt_<R>(Z * Z + K * K);
    const R c = Z * irho, s = K * irho;
    const int m = n - l - 1;
    const R lam = R(l + 1);
    R cm = R(1);
    if (m >= 1) {
        R c0 = R(1), c1 = R(2) * lam * c;
        for (int k = 2; k <= m; k++) {
            const R c2 = (R(2) * c * (R(k) + lam - R(1)) * c1 - (R(k) + R(2) * lam - R(2)) * c0) / R(k);
            c0 = c1;
            c1 = c2;
        }
        cm = c1;
    }
    R sl = R(1);
    for (int k = 0; k < l; k++) sl *= s;
    R ir = irho;
    for (int k = 0; k < n; k++) ir *= irho;
    return R(g_prefactor(l, m)) * sl * cm * ir;
}

// dG(n,l,K,Z)/dK = (l/K) G(n,l) - G(n+1,l+1)
template <typename R>
DSF_HD R gfun_dk(int l, int n, R K, R Z)
{
    R v = -gfun<R>(l + 1, n + 1, K, Z);
    if (l > 0 && K > R(0)) v += R(l) / K * gfun<R>(l, n, K, Z);
    return v;
}

// s^l C_m^{(l+1)}(c) / rho^{l+m+2}: G(n,l,K,Z) without its constant
// prefactor 2^l l! m!, n = l + m + 1.  No division (reciprocals of k from a
// small table), so the FP32 form runs on the FP32 pipe only.
__device__ __constant__ float kInvF[13] = {0.f, 1.f, 0.5f, 0.33333334f, 0.25f, 0.2f, 0.16666667f, 0.14285715f,
                                           0.125f, 0.11111111f, 0.1f, 0.09090909f, 0.083333336f};
__device__ __constant__ double kInvD[13] = {0.0, 1.0, 0.5, 1.0 / 3, 0.25, 0.2, 1.0 / 6, 1.0 / 7, 0.125, 1.0 / 9, 0.1,
                                            1.0 / 11, 1.0 / 12};

template <typename R>
__device__ __forceinline__ R inv_k(int k);
template <>
__device__ __forceinline__ float inv_k<float>(int k) { return kInvF[k]; }
template <>
__device__ __forceinline__ double inv_k<double>(int k) { return kInvD[k]; }

template <typename R>
__device__ __forceinline__ R gcore(int l, int m, R K, R Z)
{
    const R irho = rsqrt_<R>(Z * Z + K * K);
    const R c = Z * irho, s = K * irho;
    R c0 = R(1), c1 = R(2 * (l + 1)) * c;
    R cm = m == 0 ? R(1) : c1;
    for (int k = 2; k <= m; k++) {
        const R c2 = (R(2 * (k + l)) * c * c1 - R(k + 2 * l) * c0) * inv_k<R>(k);
        c0 = c1;
        c1 = c2;
    }
    if (m >= 2) cm = c1;
    R p = irho * irho;
    for (int k = 0; k < l + m; k++) p *= irho;
    for (int k = 0; k < l; k++) p *= s;
    return cm * p;
}

template <typename R>
struct cx {
    R re, im;
};

template <typename R>
DSF_HD cx<R> cmul(cx<R> a, cx<R> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

}  // namespace dsf
