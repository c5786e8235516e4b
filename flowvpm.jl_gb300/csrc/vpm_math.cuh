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
//    their Taylor series for s < 2 (11 terms, < 1e-8 relative), from erf/exp for
//    2 <= s <= 50, and from the singular form G = s^-1.5, H = -3 s^-2.5 for
//    s > 50 (rho > 7.07), where the neglected terms are below 2e-9 relative.
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
constexpr float S_SERIES = 2.0f;      // Taylor series below this s (Gaussian-erf)
constexpr float S_FAR_GERF = 50.0f;   // singular form above this s (rho > 7.07)
constexpr float S_FAR_GAUS = 8.0f;    // singular form above this s (rho^3 > 22.6)

// Taylor coefficients of G(s) = sqrt(2/pi) sum (-1/2)^k s^k / (k! (2k+3))
// and H(s) = -sqrt(2/pi) sum (-1/2)^k s^k / (k! (2k+5)).
__device__ __forceinline__ float gerf_G_series(float s)
{
    float p = 9.335750486555003e-12f;
    p = fmaf(p, s, -2.0449739161025244e-10f);
    p = fmaf(p, s, 4.0684217909829174e-09f);
    p = fmaf(p, s, -7.275295437992981e-08f);
    p = fmaf(p, s, 1.1543468761615528e-06f);
    p = fmaf(p, s, -1.5983264439159964e-05f);
    p = fmaf(p, s, 0.00018889312519007232f);
    p = fmaf(p, s, -0.0018469550018584847f);
    p = fmaf(p, s, 0.014247938585765453f);
    p = fmaf(p, s, -0.07978845608028655f);
    p = fmaf(p, s, 0.26596152026762176f);
    return p;
}
__device__ __forceinline__ float gerf_H_series(float s)
{
    float p = -8.588890447630603e-12f;
    p = fmaf(p, s, 1.8671500973110005e-10f);
    p = fmaf(p, s, -3.680953048984544e-09f);
    p = fmaf(p, s, 6.509474865572668e-08f);
    p = fmaf(p, s, -1.0185413613190173e-06f);
    p = fmaf(p, s, 1.3852162513938635e-05f);
    p = fmaf(p, s, -0.00015983264439159965f);
    p = fmaf(p, s, 0.0015111450015205786f);
    p = fmaf(p, s, -0.011081730011150908f);
    p = fmaf(p, s, 0.056991754343061814f);
    p = fmaf(p, s, -0.1595769121605731f);
    return p;
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
    const float rs = rsqrtf(s);
    const float rs2 = rs * rs;
    G = rs * rs2;
    Q = G * (rs2 * isig2);
}

// Full form of kernel K for one lane (any s > 0).
template <int K>
__device__ __forceinline__ void near_GQ(float s, float isig2, float& G, float& Q)
{
    if constexpr (K == K_WNKLMNS) {
        // g/rho^3 = (s+2.5)(s+1)^-2.5 ; -H/3 = (s+3.5)(s+1)^-3.5
        const float q = s + 1.0f;
        const float t = __frcp_rn(q);
        const float t2u = t * t * rsqrtf(q);
        G = (s + 2.5f) * t2u;
        Q = (s + 3.5f) * t * t2u * isig2;
    } else if constexpr (K == K_SING) {
        far_GQ(s, isig2, G, Q);
    } else if constexpr (K == K_GAUSERF) {
        if (s > S_FAR_GERF) {
            far_GQ(s, isig2, G, Q);
        } else if (s < S_SERIES) {
            G = gerf_G_series(s);
            Q = gerf_H_series(s) * (isig2 * -0.33333333333333333f);
        } else {
            const float rs = rsqrtf(s);
            const float rs2 = rs * rs;
            const float rho = s * rs;
            const float e = expf(-0.5f * s);
            const float g = erff(rho * 0.70710678118654752f) - F_C2 * rho * e;
            G = g * rs * rs2;
            Q = fmaf(F_C2 * -0.33333333333333333f, e, G) * rs2 * isig2;   // -H/3 = (G - c2 e / 3)/s
        }
    } else {  // Gaussian
        if (s > S_FAR_GAUS) {
            far_GQ(s, isig2, G, Q);
        } else {
            const float rs = rsqrtf(s);
            const float rho = s * rs;
            const float t = s * rho;
            if (t < 1.0f) {
                G = gaus_G_series(t);
                Q = -rho * gaus_H_series(t) * isig2;
            } else {
                const float e = expf(-t);
                G = (1.0f - e) * __frcp_rn(t);
                const float rs2 = rs * rs;
                Q = fmaf(-t, e, 1.0f - e) * rs2 * rs2 * rs * isig2;   // -H/3 = (1 - e - t e)/rho^5
            }
        }
    }
}

// (G, Q) of one pair for the whole warp: the singular form when every lane is
// past s_far (no divergence), else each lane's full form; pairs with r^2 == 0
// contribute nothing (src/FLOWVPM_fmm.jl:118).  All 32 lanes must call it.
template <int K>
__device__ __forceinline__ void pair_GQ(float r2, float s, float isig2, float& G, float& Q)
{
    if constexpr (K == K_WNKLMNS) {
        near_GQ<K>(s, isig2, G, Q);
        const bool nz = r2 > 0.0f;
        G = nz ? G : 0.0f;
        Q = nz ? Q : 0.0f;
    } else {
        if (__all_sync(0xffffffffu, s > s_far<K>())) {
            far_GQ(s, isig2, G, Q);
        } else {
            near_GQ<K>(s, isig2, G, Q);
            const bool nz = r2 > 0.0f;
            G = nz ? G : 0.0f;
            Q = nz ? Q : 0.0f;
        }
    }
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
    else if constexpr (K == K_GAUSERF) return exp2f(s * -0.72134752044448170f);  // e^{-s/2}
    else {
        const float q = s + 1.0f;
        const float t = __frcp_rn(q);
        return t * t * t * rsqrtf(q);
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
