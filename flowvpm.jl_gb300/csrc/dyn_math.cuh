// dyn_math.cuh -- per-pair test-filter differences of the dynamic SFS
// procedure (dynamic.cu, estr.cu, leaflist.cu): g'(t), g''(t) of each kernel in
// FP32, their Gauss-Legendre integrals over [rho, rho/alpha], and the Estr
// weight ratio zeta~(r, alpha sigma) / zeta~(r, sigma) - 1.
#pragma once
#include "internal.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

#include <cmath>

namespace vpm {

// g'(t) and g''(t) of kernel K in FP32 (src/FLOWVPM_kernel.jl:45-84, differentiated)
template <int K>
__device__ __forceinline__ void g_d1_d2_f32(float t, float& d1, float& d2)
{
    if constexpr (K == K_GAUSERF) {
        const float e = F_C2 * fexp2(t * t * -0.72134752044448170f);   // sqrt(2/pi) e^{-t^2/2}
        d1 = t * t * e;
        d2 = t * (2.0f - t * t) * e;
    } else if constexpr (K == K_GAUS) {
        const float t3 = t * t * t;
        const float e = fexp2(t3 * -1.4426950408889634f);              // e^{-t^3}
        d1 = 3.0f * t * t * e;
        d2 = t * (6.0f - 9.0f * t3) * e;
    } else if constexpr (K == K_WNKLMNS) {
        const float q = fmaf(t, t, 1.0f);
        const float iq = frcp(q);
        const float iq35 = iq * iq * iq * frsqrt(q);                   // q^-3.5
        d1 = 7.5f * t * t * iq35;
        d2 = 7.5f * t * (2.0f - 5.0f * t * t) * iq35 * iq;
    } else {
        d1 = 0.0f;
        d2 = 0.0f;
    }
}

// s = rho^2 beyond which a pair's filter differences are below 1e-12 of the
// near pairs' (warp-wide skip); +inf: never skipped
template <int K>
__host__ __device__ constexpr float dyn_skip_s()
{
    return K == K_GAUSERF ? 60.0f : K == K_GAUS ? 9.0f : 3.0e38f;
}

// (dg, dg1) of one pair at rho for the filter factor alpha: m two-point
// Gauss-Legendre panels on [rho, rho/alpha], hm = (1/alpha - 1)/m (m warp-uniform;
// one panel for alpha = 0.999, eight for alpha = 0.667).  M > 0 fixes m = M at
// compile time.
template <int K, int M = 0>
__device__ __forceinline__ void filter_diff(float rho, float hm, int m, float& dg, float& dg1)
{
    const float h = rho * hm;
    const float o = 0.28867513459481287f * h;    // h / (2 sqrt 3)
    float s1 = 0.0f, s2 = 0.0f;
    auto panel = [&](int k) {
        const float c = fmaf((float)k + 0.5f, h, rho);
        float a1, a2, b1, b2;
        g_d1_d2_f32<K>(c - o, a1, a2);
        g_d1_d2_f32<K>(c + o, b1, b2);
        s1 += a1 + b1;
        s2 += fmaf(c - o, a2, a1) + fmaf(c + o, b2, b1);
    };
    if constexpr (M > 0) {
#pragma unroll
        for (int k = 0; k < M; k++) panel(k);
    } else {
        for (int k = 0; k < m; k++) panel(k);
    }
    dg = 0.5f * h * s1;
    dg1 = __fdividef(0.5f * h * s2, rho);
}

// e^x - 1 and log(1 + x): Taylor series for |x| <= 1/8 (truncation below 1e-9
// relative: the dynamic procedure's alpha = 0.999 keeps every argument there),
// the library functions beyond
__device__ __forceinline__ float expm1_small(float x)
{
    if (fabsf(x) <= 0.125f) {
        float p = 1.9841269841269841e-4f;     // 1/5040
        p = fmaf(p, x, 1.3888888888888889e-3f);
        p = fmaf(p, x, 8.3333333333333333e-3f);
        p = fmaf(p, x, 4.1666666666666667e-2f);
        p = fmaf(p, x, 0.16666666666666667f);
        p = fmaf(p, x, 0.5f);
        p = fmaf(p, x, 1.0f);
        return p * x;
    }
    return expm1f(x);
}
__device__ __forceinline__ float log1p_small(float x)
{
    if (fabsf(x) <= 0.125f) {
        float p = -0.1f;        // log(1 + x)/x = sum_k (-x)^k/(k + 1)
        p = fmaf(p, x, 0.11111111111111111f);
        p = fmaf(p, x, -0.125f);
        p = fmaf(p, x, 0.14285714285714286f);
        p = fmaf(p, x, -0.16666666666666667f);
        p = fmaf(p, x, 0.2f);
        p = fmaf(p, x, -0.25f);
        p = fmaf(p, x, 0.33333333333333333f);
        p = fmaf(p, x, -0.5f);
        p = fmaf(p, x, 1.0f);
        return p * x;
    }
    return log1pf(x);
}

// zeta~(r, alpha sigma) / zeta~(r, sigma) - 1 at s = (r/sigma)^2, zeta~(r, sigma) =
// zeta(r/sigma)/sigma^3 (src/FLOWVPM_kernel.jl:45-84); fd = (alpha^-3 - 1, alpha^-3, alpha^-2 - 1)
template <int K>
__device__ __forceinline__ float zeta_ratio_m1(float s, float3 fd)
{
    if constexpr (K == K_GAUSERF) {          // zeta ~ e^{-rho^2/2}
        return fmaf(fd.y, expm1_small(-0.5f * s * fd.z), fd.x);
    } else if constexpr (K == K_GAUS) {      // zeta ~ e^{-rho^3}
        return fmaf(fd.y, expm1_small(-s * sqrtf(s) * fd.x), fd.x);
    } else if constexpr (K == K_WNKLMNS) {   // zeta ~ (rho^2 + 1)^-3.5
        const float eps = s * fd.z / fmaf(s, 1.0f + fd.z, 1.0f);
        return fmaf(fd.y, expm1_small(3.5f * log1p_small(-eps)), fd.x);
    } else {
        return 0.0f;
    }
}

// One pair's dJ (the pair's J term of src/FLOWVPM_fmm.jl:112-160 differenced
// in sigma, column-major 3x3), added to f: e = x_t - x_s (|e|^2 = r2 > 0),
// isig = 1/sigma_s, gam = the packed Gamma_s * (-1/(4 pi)) (over sigma_s^3 unless
// singular_tail<K>), panels as in filter_diff.  on = false adds zero (r2 must
// still be positive and finite), so that callers can run four pairs without
// branches.
template <int K, int M = 0>
__device__ __forceinline__ void filter_diff_pair(float ex, float ey, float ez, float r2, float isig, float4 gam,
                                                 float hm, int m, bool on, float (&f)[9])
{
    const float rinv = frsqrt(r2);
    const float rho = r2 * rinv * isig;
    float dg, dg1;
    filter_diff<K, M>(rho, hm, m, dg, dg1);
    dg = on ? dg : 0.0f;
    dg1 = on ? dg1 : 0.0f;
    float gx = gam.x, gy = gam.y, gz = gam.z;
    if constexpr (!singular_tail<K>()) {
        const float sig3 = __fdividef(1.0f, isig * isig * isig);
        gx *= sig3; gy *= sig3; gz *= sig3;
    }
    const float ri2 = rinv * rinv, ri3 = ri2 * rinv;
    // c = -(e x Gamma)/(4 pi r^3); the U difference would be dg c; a = daux c with
    // daux = dg1 / (sigma r) - 3 dg / r^2; daux2 = -dg / (4 pi r^3)
    const float cx = ri3 * (ey * gz - ez * gy), cy = ri3 * (ez * gx - ex * gz), cz = ri3 * (ex * gy - ey * gx);
    const float daux = fmaf(dg1 * isig, rinv, -3.0f * dg * ri2);
    const float dax2 = dg * ri3;   // times -Gamma/(4 pi): the packed gam
    const float a1 = daux * cx, a2 = daux * cy, a3 = daux * cz;
    f[0] = fmaf(a1, ex, f[0]);
    f[1] = fmaf(a2, ex, fmaf(-dax2, gz, f[1]));
    f[2] = fmaf(a3, ex, fmaf(dax2, gy, f[2]));
    f[3] = fmaf(a1, ey, fmaf(dax2, gz, f[3]));
    f[4] = fmaf(a2, ey, f[4]);
    f[5] = fmaf(a3, ey, fmaf(-dax2, gx, f[5]));
    f[6] = fmaf(a1, ez, fmaf(-dax2, gy, f[6]));
    f[7] = fmaf(a2, ez, fmaf(dax2, gx, f[7]));
    f[8] = fmaf(a3, ez, f[8]);
}

// Gauss-Legendre panels for the filter factor: the two-point rule's error per
// panel ~ (h/m)^5, so m grows with ha = 1/alpha - 1
inline int filter_panels(double ha) { return ha <= 0.0625 ? 1 : (int)std::ceil(ha * 16.0); }

}  // namespace vpm
