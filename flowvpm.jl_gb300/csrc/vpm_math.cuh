// vpm_math.cuh -- device-side regularizing-kernel math for the UJ and Estr
// kernels.
//
// Two forms are provided:
//
//  * FP64, the reference formula: (g, dg/dr) of src/FLOWVPM_kernel.jl:45-84 and
//    zeta of the same file, used by the plain FP64 kernels.  The only change is
//    an exact far-field shortcut for the Gaussian-erf kernel: for rho > 9 the
//    terms erf(rho/sqrt2)-1 and sqrt(2/pi)*rho*exp(-rho^2/2) are below 2^-56, so
//    g = 1 and dg = 0 to FP64 rounding.
//
//  * FP32, a regular reformulation used by the mixed kernels.  With
//    s = rho^2 = r^2/sigma^2 the pair terms of src/FLOWVPM_fmm.jl:130-160 are
//        g/r^3                          = G(s) / sigma^3
//        dg/(sigma r^4) - 3 g / r^5     = H(s) / sigma^5
//    with G(s) = g(rho)/rho^3 and H(s) = (rho g'(rho) - 3 g(rho)) / rho^5.
//    G and H are smooth at s = 0, so the cancellation of erf(rho/sqrt2) against
//    sqrt(2/pi)*rho*exp(-rho^2/2) that the literal formula suffers for small
//    rho in FP32 never happens.  For the Gaussian-erf kernel G and H come from
//    their series of positive terms for s < 2 (< 1e-8 relative), from
//    e^{-s/2} and a fit of erfcx for 2 <= s <= 50 (no erf call), and from the
//    singular form G = s^-1.5, H = -3 s^-2.5 for s > 50 (rho > 7.07), where the
//    neglected terms are below 2e-9 relative (gerf_GQ below).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vpm {

// src/FLOWVPM.jl:62-66
constexpr double C1 = 0.063493635934240969;   // 1/(2*pi)^1.5
constexpr double C2 = 0.79788456080286541;    // sqrt(2/pi)
constexpr double C3 = 0.23873241463784300;    // 3/(4*pi)
constexpr double C4 = 0.079577471545947673;   // 1/(4*pi)
constexpr double INV_SQRT2 = 0.70710678118654752;

enum : int { K_SING = 0, K_GAUS = 1, K_GAUSERF = 2, K_WNKLMNS = 3 };

// Normalisation of zeta per kernel: zeta(rho) = ZNORM * zhat(s).
__host__ __device__ constexpr double zeta_norm(int K)
{
    return K == K_GAUS ? C3 : K == K_GAUSERF ? C1 : K == K_WNKLMNS ? C4 * 7.5 : 1.0;
}

// ------------------------------------------------------------------ FP64
template <int K>
__device__ __forceinline__ void g_dgdr_f64(double rho, double& g, double& dg)
{
    if constexpr (K == K_SING) {
        g = 1.0; dg = 0.0;
    } else if constexpr (K == K_GAUS) {
        const double aux = exp(-rho * rho * rho);
        g = 1.0 - aux; dg = 3.0 * rho * rho * aux;
    } else if constexpr (K == K_GAUSERF) {
        if (rho > 9.0) { g = 1.0; dg = 0.0; }
        else {
            const double aux = C2 * rho * exp(-0.5 * rho * rho);
            g = erf(rho * INV_SQRT2) - aux; dg = rho * aux;
        }
    } else {  // Winckelmans
        const double q = rho * rho + 1.0;
        const double q2 = q * q;
        const double q25 = sqrt(q2 * q2 * q);
        g = rho * rho * rho * (rho * rho + 2.5) / q25;
        dg = 7.5 * rho * rho / (q25 * q);
    }
}

template <int K>
__device__ __forceinline__ double zeta_f64(double rho)
{
    if constexpr (K == K_SING) return rho == 0.0 ? 1.0 : 0.0;
    else if constexpr (K == K_GAUS) return C3 * exp(-rho * rho * rho);
    else if constexpr (K == K_GAUSERF) return C1 * exp(-0.5 * rho * rho);
    else {
        const double t = rho * rho + 1.0;
        const double t3 = t * t * t;
        return C4 * 7.5 / sqrt(t3 * t3 * t);
    }
}

// ------------------------------------------------------------------ FP32
constexpr float F_C2 = 0.7978845608028654f;
constexpr float F_C4 = 0.07957747154594767f;   // 1/(4 pi)
constexpr float S_SERIES = 2.0f;      // positive series below this s (Gaussian-erf, gerf_GQ)
constexpr float S_FAR_GERF = 50.0f;   // singular form above this s (rho > 7.07)
constexpr float S_FAR_GAUS = 8.0f;    // singular form above this s (rho^3 > 22.6)

#ifndef VPM_FTZ_UNARY
#define VPM_FTZ_UNARY 1
#endif
// 1/sqrt(x), 2^x and 1/x of the FP32 pair forms: the hardware approximations with
// subnormal arguments and results flushed to zero (PTX rsqrt.approx.ftz.f32,
// ex2.approx.ftz.f32, rcp.approx.ftz.f32).  The arguments on the pair paths are
// normal numbers (s, r^2 and 1 + s are at least 1e-30, or the pair is masked out),
// and a 2^x flushed below 2^-126 is far under the FP32 resolution of the sums; the
// forms that keep subnormals guard every call.  0 selects rsqrtf, exp2f, __frcp_rn.
__device__ __forceinline__ float frsqrt(float x)
{
#if VPM_FTZ_UNARY
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return rsqrtf(x);
#endif
}
__device__ __forceinline__ float fexp2(float x)
{
#if VPM_FTZ_UNARY
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return exp2f(x);
#endif
}
__device__ __forceinline__ float frcp(float x)
{
#if VPM_FTZ_UNARY
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return __frcp_rn(x);
#endif
}

// Gaussian kernel, t = rho^3: G = (1 - e^-t)/t = sum (-t)^k/(k+1)!,
// H = 3 rho sum_{k>=2} (-1)^(k+1) (k-1)/k! t^(k-2).
__device__ __forceinline__ float gaus_G_series(float t)
{
    float p = -2.08767569878681e-09f;
    p = fmaf(p, t, 2.505210838544172e-08f);
    p = fmaf(p, t, -2.755731922398589e-07f);
    p = fmaf(p, t, 2.7557319223985893e-06f);
    p = fmaf(p, t, -2.48015873015873e-05f);
    p = fmaf(p, t, 0.0001984126984126984f);
    p = fmaf(p, t, -0.001388888888888889f);
    p = fmaf(p, t, 0.008333333333333333f);
    p = fmaf(p, t, -0.041666666666666664f);
    p = fmaf(p, t, 0.16666666666666666f);
    p = fmaf(p, t, -0.5f);
    p = fmaf(p, t, 1.0f);
    return p;
}
__device__ __forceinline__ float gaus_H_series(float t)
{
    float p = 1.9270852604185937e-09f;
    p = fmaf(p, t, -2.296443268665491e-08f);
    p = fmaf(p, t, 2.505210838544172e-07f);
    p = fmaf(p, t, -2.48015873015873e-06f);
    p = fmaf(p, t, 2.2045855379188714e-05f);
    p = fmaf(p, t, -0.00017361111111111112f);
    p = fmaf(p, t, 0.0011904761904761906f);
    p = fmaf(p, t, -0.006944444444444444f);
    p = fmaf(p, t, 0.03333333333333333f);
    p = fmaf(p, t, -0.125f);
    p = fmaf(p, t, 0.3333333333333333f);
    p = fmaf(p, t, -0.5f);
    return p;
}

// The mixed kernels accumulate, per pair,
//     U += G c,   W += G gam,   J' += Q c_i dx_j,
// with c = dx x gam, gam = -Gamma/(4 pi sigma^3), and Q = -H/(3 sigma^2), so
// that J = -3 J' + (Kronecker term from W) once per target.  In the singular
// (far) form Q = G / r^2.

// s above which the kernel equals its singular form to FP32 resolution; 0 for
// the singular kernel (every pair with r > 0), +inf for Winckelmans (never).
template <int K>
__host__ __device__ constexpr float s_far()
{
    return K == K_SING ? 0.0f : K == K_GAUSERF ? S_FAR_GERF : K == K_GAUS ? S_FAR_GAUS : 3.0e38f;
}

// Singular form: G = s^-1.5, Q = G / r^2 = G s^-1 / sigma^2.
__device__ __forceinline__ void far_GQ(float s, float isig2, float& G, float& Q)
{
    const float rs = frsqrt(s);
    const float rs2 = rs * rs;
    G = rs * rs2;
    Q = G * (rs2 * isig2);
}

// G = g/rho^3 of Gaussian-erf for s >= 2 from the erfcx fit, given e = e^{-s/2}, rs = s^-1/2
__device__ __forceinline__ float gerf_G_erfcx(float s, float e, float rs)
{
    const float rho = s * rs;
    const float t = __fdividef(1.0f, fmaf(0.5f, fminf(rho, 10.0f), 1.0f));
    const float w = fmaf(4.77190564267067f, t, -1.795317607111778f);
    float p = -5.1560079373370265e-06f;
    p = fmaf(p, w, 5.998428003101994e-06f);
    p = fmaf(p, w, 0.00010125038777505872f);
    p = fmaf(p, w, -0.00030713426402493693f);
    p = fmaf(p, w, -0.0023330098304451836f);
    p = fmaf(p, w, 0.009623567049071946f);
    p = fmaf(p, w, 0.13016216050000662f);
    p = fmaf(p, w, 0.5926831417002281f);
    const float h = fmaf(F_C2, rho, p * t);
    return fmaf(-e, h, 1.0f) * rs * (rs * rs);
}

// Gaussian-erf G and Q = -H/(3 sigma^2) of one lane at any s >= 0, with
// e = e^{-s/2} (coefficients from fit_gerf.py):
//   s < 2:  G = c2 e (1/3 + s S2(s)), -H/3 = c2 e S2(s), S2(s) = sum_m s^m/(2m+5)!!
//           (Kummer's series of erf: positive terms, no cancellation);
//   s >= 2: g = 1 - e (erfcx(rho/sqrt2) + c2 rho) with erfcx(rho/sqrt2) = P(w) t,
//           t = 1/(1 + rho/2), w = A t + B, P of degree 7 (rho capped at 10, beyond
//           which e < 2e-22 and G is its singular form s^-1.5); G = g/rho^3,
//           -H/3 = (G - c2 e/3)/s.
// No erf call.  FAR adds a third branch, the singular form beyond s = 50, for
// callers whose near groups hold many lanes past the kernel's reach (the
// all-pairs kernels); without it those lanes take the s >= 2 form, which is
// valid there.
template <bool FAR>
__device__ __forceinline__ void gerf_GQ(float s, float isig2, float& G, float& Q)
{
    if (FAR && s > S_FAR_GERF) {
        far_GQ(s, isig2, G, Q);
        return;
    }
    const float e = fexp2(s * -0.72134752044448170f);
    if (s < S_SERIES) {
        float p = 3.1622138893727926e-12f;
        p = fmaf(p, s, 7.273091945557423e-11f);
        p = fmaf(p, s, 1.5273493085670588e-09f);
        p = fmaf(p, s, 2.901963686277412e-08f);
        p = fmaf(p, s, 4.9333382666716e-07f);
        p = fmaf(p, s, 7.4000074000074e-06f);
        p = fmaf(p, s, 9.62000962000962e-05f);
        p = fmaf(p, s, 0.0010582010582010583f);
        p = fmaf(p, s, 0.009523809523809525f);
        p = fmaf(p, s, 0.06666666666666667f);
        const float ce = F_C2 * e;
        G = ce * fmaf(s, p, 0.33333333333333333f);
        Q = ce * p * isig2;
    } else {
        const float rs = frsqrt(s);
        const float rs2 = rs * rs;
        G = gerf_G_erfcx(s, e, rs);
        Q = fmaf(F_C2 * -0.33333333333333333f, e, G) * rs2 * isig2;
    }
}

// gerf_GQ for four pairs of one lane, with the choice of forms made for the
// whole warp so that the four pairs' chains interleave: every lane past s = 50
// (FAR only): the singular form; otherwise the s >= 2 form for all four (valid
// at any s > 0), replaced by the series, per pair, where s < 2 when any lane
// of the warp has such a pair.  All 32 lanes must call it.
template <bool FAR>
__device__ __forceinline__ void gerf_GQ4(const float (&s)[4], const float (&isig2)[4], float (&G)[4], float (&Q)[4])
{
    bool allfar = FAR, anyser = false;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        allfar = allfar && s[q] > S_FAR_GERF;
        anyser = anyser || s[q] < S_SERIES;
    }
    if (FAR && __all_sync(0xffffffffu, allfar)) {
#pragma unroll
        for (int q = 0; q < 4; q++) far_GQ(s[q], isig2[q], G[q], Q[q]);
        return;
    }
    float e[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        e[q] = fexp2(s[q] * -0.72134752044448170f);
        const float rs = frsqrt(s[q]);
        G[q] = gerf_G_erfcx(s[q], e[q], rs);
        Q[q] = fmaf(F_C2 * -0.33333333333333333f, e[q], G[q]) * (rs * rs) * isig2[q];
    }
    if (__any_sync(0xffffffffu, anyser)) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float p = 3.1622138893727926e-12f;
            p = fmaf(p, s[q], 7.273091945557423e-11f);
            p = fmaf(p, s[q], 1.5273493085670588e-09f);
            p = fmaf(p, s[q], 2.901963686277412e-08f);
            p = fmaf(p, s[q], 4.9333382666716e-07f);
            p = fmaf(p, s[q], 7.4000074000074e-06f);
            p = fmaf(p, s[q], 9.62000962000962e-05f);
            p = fmaf(p, s[q], 0.0010582010582010583f);
            p = fmaf(p, s[q], 0.009523809523809525f);
            p = fmaf(p, s[q], 0.06666666666666667f);
            const float ce = F_C2 * e[q];
            const bool ser = s[q] < S_SERIES;
            G[q] = ser ? ce * fmaf(s[q], p, 0.33333333333333333f) : G[q];
            Q[q] = ser ? ce * p * isig2[q] : Q[q];
        }
    }
}

// Full form of kernel K for one lane (any s > 0); FAR as in gerf_GQ.
template <int K, bool FAR = true>
__device__ __forceinline__ void near_GQ(float s, float isig2, float& G, float& Q)
{
    if constexpr (K == K_WNKLMNS) {
        // g/rho^3 = (s+2.5)(s+1)^-2.5 ; -H/3 = (s+3.5)(s+1)^-3.5
        const float q = s + 1.0f;
        const float t = frcp(q);
        const float t2u = t * t * frsqrt(q);
        G = (s + 2.5f) * t2u;
        Q = (s + 3.5f) * t * t2u * isig2;
    } else if constexpr (K == K_SING) {
        far_GQ(s, isig2, G, Q);
    } else if constexpr (K == K_GAUSERF) {
        gerf_GQ<FAR>(s, isig2, G, Q);
    } else {  // Gaussian
        if (s > S_FAR_GAUS) {
            far_GQ(s, isig2, G, Q);
        } else {
            const float rs = frsqrt(s);
            const float rho = s * rs;
            const float t = s * rho;
            if (t < 1.0f) {
                G = gaus_G_series(t);
                Q = -rho * gaus_H_series(t) * isig2;
            } else {
                const float e = expf(-t);
                G = (1.0f - e) * frcp(t);
                const float rs2 = rs * rs;
                Q = fmaf(-t, e, 1.0f - e) * rs2 * rs2 * rs * isig2;   // -H/3 = (1 - e - t e)/rho^5
            }
        }
    }
}

// near_GQ for four pairs of one lane; all 32 lanes must call it.
template <int K, bool FAR = true>
__device__ __forceinline__ void near_GQ4(const float (&s)[4], const float (&isig2)[4], float (&G)[4], float (&Q)[4])
{
    if constexpr (K == K_GAUSERF) {
        gerf_GQ4<FAR>(s, isig2, G, Q);
    } else {
#pragma unroll
        for (int q = 0; q < 4; q++) near_GQ<K, FAR>(s[q], isig2[q], G[q], Q[q]);
    }
}

// (a + b) - (oh + ol) for two double-floats (hi a / oh, lo b / ol) in FP32: the
// difference of the high parts is made exact by TwoSum (s + e), the rest added
// after, so the result is rounded once, nearly correctly.  The same operations
// on the same inputs give the same bits: a point's offset from an origin
// equals itself wherever it is formed (the self pair has r^2 == 0 exactly).
__device__ __forceinline__ float df_offset(float a, float b, float oh, float ol)
{
    const float s = a - oh;
    const float v = s - a;
    const float e = (a - (s - v)) - (oh + v);
    return s + (e + (b - ol));
}

// s += y, with the rounding error of the addition accumulated in c (Fast2Sum;
// exact when |s| >= |y|, which a running sum of like terms keeps after its
// first additions).  s + c is the compensated sum.
__device__ __forceinline__ void comp_add(float& s, float& c, float y)
{
    const float t = s + y;
    c += (s - t) + y;
    s = t;
}

// zeta(rho)/ZNORM as a function of s = rho^2 (FP32).
template <int K>
__device__ __forceinline__ float zhat_f32(float s)
{
    if constexpr (K == K_SING) return s == 0.0f ? 1.0f : 0.0f;
    else if constexpr (K == K_GAUS) { const float rho = sqrtf(s); return expf(-s * rho); }
    else if constexpr (K == K_GAUSERF) return fexp2(s * -0.72134752044448170f);  // e^{-s/2}
    else {
        const float q = s + 1.0f;
        const float t = frcp(q);
        return t * t * t * frsqrt(q);
    }
}

// s above which zeta/zeta(0) < 1e-13 for the Gaussian kernels (contribution
// skipped when every lane of a warp is past it); 0 = never skip.
template <int K>
__host__ __device__ constexpr float zeta_skip_s()
{
    return K == K_GAUSERF ? 60.0f : K == K_GAUS ? 10.0f : 0.0f;
}

}  // namespace vpm
