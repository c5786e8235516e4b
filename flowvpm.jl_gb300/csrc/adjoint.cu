// adjoint.cu -- reverse mode of the UJ pair sum (replaces the unwired rrule
// of src/FLOWVPM_rrules.jl:179-330).
//
// For L with dL/dU = Ubar and dL/dJ = Jbar, each pair (t, s) contributes
//     phi = Ubar_t . u(dx, Gamma_s, sigma_s) + Jbar_t : j(dx, Gamma_s, sigma_s),
// dx = x_t - x_s, with u and j the pair terms of src/FLOWVPM_fmm.jl:112-160.
// Writing q(r) = -g(rho)/(4 pi r^3), A = q, B = q'/r, c = dx x Gamma:
//     u = A c,   j_ab = B c_a dx_b + A eps_abl Gamma_l,
//     phi = A P + B Q,  P = Ubar.c + wbar.Gamma,  Q = c.(Jbar dx),  wbar_l = eps_abl Jbar_ab
// and
//     dphi/d(dx)   = (B P + (B'/r) Q) dx + A (Gamma x Ubar) + B (Gamma x Jbar dx + Jbar^T c)
//     dphi/dGamma  = A (Ubar x dx + wbar) + B ((Jbar dx) x dx)
//     dphi/dsigma  = (dA/dsigma) P + (dB/dsigma) Q
// with q'' (hence the kernels' g'') in B'.  x_t gets +dphi/d(dx), x_s gets
// -dphi/d(dx).
//
// Layout: one target per thread (Morton order, as in uj.cu), sources staged in
// shared memory.  Target-side sums stay in registers; each source's 7 sums
// (x, Gamma, sigma) are reduce-scattered across the warp with shuffles, four
// sources at a time (adj_reduce4), summed across the
// block's 4 warps in shared memory, then added to the outputs with one FP64
// atomic per source and block (so the summation order of those sums is not
// fixed).  Arithmetic is FP64 throughout.
#include "internal.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

namespace vpm {

// (g, g', g'') of kernel K at rho, FP64 (derivatives of src/FLOWVPM_kernel.jl:45-84).
// Beyond rho = 9 (Gaussian-erf) / 3.5 (Gaussian) g = 1 and g' = g'' = 0 to FP64.
template <int K>
__device__ __forceinline__ void g_d1_d2_f64(double rho, double& g, double& d1, double& d2)
{
    if constexpr (K == K_SING) {
        g = 1.0; d1 = 0.0; d2 = 0.0;
    } else if constexpr (K == K_GAUS) {
        if (rho > 3.5) { g = 1.0; d1 = 0.0; d2 = 0.0; }
        else {
            const double r3 = rho * rho * rho;
            const double e = exp(-r3);
            g = 1.0 - e; d1 = 3.0 * rho * rho * e; d2 = (6.0 * rho - 9.0 * r3 * rho) * e;
        }
    } else if constexpr (K == K_GAUSERF) {
        if (rho > 9.0) { g = 1.0; d1 = 0.0; d2 = 0.0; }
        else {
            const double e = C2 * exp(-0.5 * rho * rho);
            g = erf(rho * INV_SQRT2) - rho * e;
            d1 = rho * rho * e;
            d2 = (2.0 * rho - rho * rho * rho) * e;
        }
    } else {
        const double q = rho * rho + 1.0;
        const double iq = 1.0 / q;
        const double iq25 = iq * iq * sqrt(iq);           // q^-2.5
        g = rho * rho * rho * (rho * rho + 2.5) * iq25;
        d1 = 7.5 * rho * rho * iq25 * iq;
        d2 = 7.5 * rho * (2.0 - 5.0 * rho * rho) * iq25 * iq * iq;
    }
}

// r^2 past which kernel K has g = 1, g' = g'' = 0 to FP64 (g_d1_d2_f64's cuts), as a
// multiple of sigma^2; 0 = never (the singular kernel takes that form at every r).
template <int K>
__host__ __device__ constexpr double adj_far_s()
{
    return K == K_GAUSERF ? 81.0 : K == K_GAUS ? 12.25 : 0.0;
}

// The 7 derivatives of phi for one pair: o[0..2] = dphi/d(dx), o[3..5] = dphi/dGamma,
// o[6] = dphi/dsigma.  Pairs with r^2 == 0 give zeros.  Pairs past the kernel's cut
// (s.gz_sig.y = adj_far_s sigma^2, from pack_src_adj) and every pair of the singular
// kernel take A = -C4/r^3, B = 3 C4/r^5, B'/r = -15 C4/r^7, dA = dB = 0: the general
// coefficients at g = 1, g' = g'' = 0.
template <int K>
__device__ __forceinline__ void adj_pair_f64(double dx, double dy, double dz, const SrcF64& s,
                                             const double (&Ub)[3], const double (&Jb)[9], const double (&wb)[3],
                                             double (&o)[7])
{
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 == 0.0) {
#pragma unroll
        for (int k = 0; k < 7; k++) o[k] = 0.0;
        return;
    }
    const double rinv = rsqrt(r2);
    const double ri2 = rinv * rinv, ri3 = ri2 * rinv;
    double A, B, Bpr, dA = 0.0, dB = 0.0;
    if (K == K_SING || (adj_far_s<K>() > 0.0 && r2 > s.gz_sig.y)) {
        const double ri5 = ri3 * ri2;
        A = -C4 * ri3;
        B = (3.0 * C4) * ri5;
        Bpr = (-15.0 * C4) * ri5 * ri2;
    } else {
        const double isig = s.z_isig.y;
        const double rho = r2 * rinv * isig;
        double g, g1, g2;
        g_d1_d2_f64<K>(rho, g, g1, g2);
        const double ri4 = ri2 * ri2, ri5 = ri4 * rinv;
        A = -C4 * g * ri3;
        B = -C4 * (g1 * isig * ri4 - 3.0 * g * ri5);
        const double qpp = -C4 * (g2 * isig * isig * ri3 - 6.0 * g1 * isig * ri4 + 12.0 * g * ri5);
        Bpr = (qpp - B) * ri2;
        dA = C4 * g1 * rho * isig * ri3;
        dB = -C4 * (2.0 * g1 - rho * g2) * isig * isig * ri4;
    }
    const double Gx = s.gxy.x, Gy = s.gxy.y, Gz = s.gz_sig.x;
    const double cx = dy * Gz - dz * Gy, cy = dz * Gx - dx * Gz, cz = dx * Gy - dy * Gx;
    const double JDx = Jb[0] * dx + Jb[3] * dy + Jb[6] * dz;
    const double JDy = Jb[1] * dx + Jb[4] * dy + Jb[7] * dz;
    const double JDz = Jb[2] * dx + Jb[5] * dy + Jb[8] * dz;
    const double JTcx = Jb[0] * cx + Jb[1] * cy + Jb[2] * cz;
    const double JTcy = Jb[3] * cx + Jb[4] * cy + Jb[5] * cz;
    const double JTcz = Jb[6] * cx + Jb[7] * cy + Jb[8] * cz;
    const double P = Ub[0] * cx + Ub[1] * cy + Ub[2] * cz + wb[0] * Gx + wb[1] * Gy + wb[2] * Gz;
    const double Q = cx * JDx + cy * JDy + cz * JDz;
    const double sc = B * P + Bpr * Q;
    o[0] = sc * dx + A * (Gy * Ub[2] - Gz * Ub[1]) + B * (Gy * JDz - Gz * JDy + JTcx);
    o[1] = sc * dy + A * (Gz * Ub[0] - Gx * Ub[2]) + B * (Gz * JDx - Gx * JDz + JTcy);
    o[2] = sc * dz + A * (Gx * Ub[1] - Gy * Ub[0]) + B * (Gx * JDy - Gy * JDx + JTcz);
    o[3] = A * (Ub[1] * dz - Ub[2] * dy + wb[0]) + B * (JDy * dz - JDz * dy);
    o[4] = A * (Ub[2] * dx - Ub[0] * dz + wb[1]) + B * (JDz * dx - JDx * dz);
    o[5] = A * (Ub[0] * dy - Ub[1] * dx + wb[2]) + B * (JDx * dy - JDy * dx);
    o[6] = (K == K_SING) ? 0.0 : dA * P + dB * Q;
}

// Source-side sums of four pairs, reduce-scattered over the warp: v0..v3 are this lane's
// 7 terms of sources 0..3.  Lanes exchange half of the sources 16 apart, then half of the rest
// 8 apart, then add the remaining source's 7 terms across the 8 lanes left (42 FP64 adds
// a lane for the four sources, against 140 for a full reduction of each).  On return
// every lane of the 8-lane group of source q = 2 (lane/16 % 2) + (lane/8 % 2) holds its
// 7 sums in w; q is returned.
__device__ __forceinline__ int adj_reduce4(const double (&v0)[7], const double (&v1)[7], const double (&v2)[7],
                                           const double (&v3)[7], int lane, double (&w)[7])
{
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    double a[7], b[7];
#pragma unroll
    for (int k = 0; k < 7; k++) {   // sources {0, 2} -> lanes without / with bit 16; {1, 3} likewise
        a[k] = (h16 ? v2[k] : v0[k]) + __shfl_xor_sync(0xffffffffu, h16 ? v0[k] : v2[k], 16);
        b[k] = (h16 ? v3[k] : v1[k]) + __shfl_xor_sync(0xffffffffu, h16 ? v1[k] : v3[k], 16);
    }
#pragma unroll
    for (int k = 0; k < 7; k++) w[k] = (h8 ? b[k] : a[k]) + __shfl_xor_sync(0xffffffffu, h8 ? a[k] : b[k], 8);
#pragma unroll
    for (int m = 4; m > 0; m >>= 1)
#pragma unroll
        for (int k = 0; k < 7; k++) w[k] += __shfl_xor_sync(0xffffffffu, w[k], m);
    return (h16 ? 2 : 0) + (h8 ? 1 : 0);
}

template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
uj_adjoint_f64_kernel(int64_t nt, const TgtPos* __restrict__ tgt, const double* __restrict__ Ubar,
                      const double* __restrict__ Jbar, int64_t ns, int64_t ns_pad,
                      const SrcF64* __restrict__ src, int64_t per_split, double* xbar, double* gbar,
                      double* sbar)
{
    __shared__ SrcF64 tile[UJ_TILE];
    __shared__ double red[UJ_WARPS][UJ_TILE][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 3.0e4, ty = 3.0e4, tz = 3.0e4;
    int64_t idx = 0;
    double Ub[3] = {0.0, 0.0, 0.0}, Jb[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Jb[k] = 0.0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
#pragma unroll
        for (int k = 0; k < 3; k++) Ub[k] = Ubar[3 * idx + k];
#pragma unroll
        for (int k = 0; k < 9; k++) Jb[k] = Jbar[9 * idx + k];
    }
    // wbar_l = eps_abl Jbar_ab with Jbar_ab at Jb[a + 3b]
    const double wb[3] = {Jb[1 + 3 * 2] - Jb[2 + 3 * 1], Jb[2 + 3 * 0] - Jb[0 + 3 * 2], Jb[0 + 3 * 1] - Jb[1 + 3 * 0]};
    double acc[3] = {0.0, 0.0, 0.0};
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
        for (int j = 0; j < UJ_TILE; j += 4) {
            double o0[7], o1[7], o2[7], o3[7];
            {
                const SrcF64& s = tile[j];
                adj_pair_f64<K>(tx - s.xy.x, ty - s.xy.y, tz - s.z_isig.x, s, Ub, Jb, wb, o0);
            }
            {
                const SrcF64& s = tile[j + 1];
                adj_pair_f64<K>(tx - s.xy.x, ty - s.xy.y, tz - s.z_isig.x, s, Ub, Jb, wb, o1);
            }
            {
                const SrcF64& s = tile[j + 2];
                adj_pair_f64<K>(tx - s.xy.x, ty - s.xy.y, tz - s.z_isig.x, s, Ub, Jb, wb, o2);
            }
            {
                const SrcF64& s = tile[j + 3];
                adj_pair_f64<K>(tx - s.xy.x, ty - s.xy.y, tz - s.z_isig.x, s, Ub, Jb, wb, o3);
            }
#pragma unroll
            for (int k = 0; k < 3; k++) acc[k] += (o0[k] + o1[k]) + (o2[k] + o3[k]);
            double w[7];
            const int q = adj_reduce4(o0, o1, o2, o3, lane, w);
            if ((lane & 7) == 0) {   // x_s gets -dphi/d(dx)
#pragma unroll
                for (int k = 0; k < 7; k++) red[warp][j + q][k] = k < 3 ? -w[k] : w[k];
            }
        }
        __syncthreads();
        const int64_t si = base + threadIdx.x;
        if (si < ns) {
            double v[7];
#pragma unroll
            for (int k = 0; k < 7; k++) v[k] = red[0][threadIdx.x][k] + red[1][threadIdx.x][k] +
                                              red[2][threadIdx.x][k] + red[3][threadIdx.x][k];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                atomicAdd(&xbar[3 * si + k], v[k]);
                atomicAdd(&gbar[3 * si + k], v[3 + k]);
            }
            if (K != K_SING) atomicAdd(&sbar[si], v[6]);
        }
    }
    if (valid) {
#pragma unroll
        for (int k = 0; k < 3; k++) atomicAdd(&xbar[3 * idx + k], acc[k]);
    }
}

template <int K>
__global__ void pack_src_adj(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
                             const double* __restrict__ gs, const double* __restrict__ sgs,
                             SrcF64* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ns_pad) return;
    SrcF64 p;
    if (i < ns) {
        const double sig = (K == K_SING) ? 1.0 : sgs[i];
        p.xy = make_double2(xs[3 * i], xs[3 * i + 1]);
        p.z_isig = make_double2(xs[3 * i + 2], 1.0 / sig);
        p.gxy = make_double2(gs[3 * i], gs[3 * i + 1]);
        // .y: the r^2 of adj_pair_f64's cut
        p.gz_sig = make_double2(gs[3 * i + 2], adj_far_s<K>() * sig * sig);
    } else {  // padding: far away, no strength
        p.xy = make_double2(1.0e6, 1.0e6);
        p.z_isig = make_double2(1.0e6, 1.0);
        p.gxy = make_double2(0.0, 0.0);
        p.gz_sig = make_double2(0.0, adj_far_s<K>());
    }
    out[i] = p;
}

// ------------------------------------------------------------- FP32-comp adjoint
// The same pair derivatives in FP32 with the forward mixed kernel's layout:
// targets and sources in Morton order, FP32 offsets from the warp's first
// target, four-source votes between the singular form (every lane's pairs
// beyond s_far and twice the warp radius) and the full form on the
// double-float displacement.  With s = r^2/sigma^2 and e = e^{-s/2}, the
// coefficients of the pair term are written so that nothing cancels at small s:
//   A   = -C4 sigma^-3 G(s),   G = g/rho^3
//   B   = -C4 sigma^-5 H(s),   H = (g'/rho^2 - 3 g/rho^3)/s
//   B'/r= -C4 sigma^-7 K(s),   K = (g'' rho^2 - 7 g' rho + 15 g)/(rho^3 s^2)
//   dA/dsigma = C4 sigma^-4 a(s),  a = g'/rho^2
//   dB/dsigma = -C4 sigma^-6 b(s), b = (2 g' - rho g'')/rho^4
// (Gaussian-erf: G, H and K from one series of positive terms below s = 6, G
// from the erfcx fit above; a = b = sqrt(2/pi) e.  Winckelmans: rational, q = s + 1:
// G = (s+2.5) q^-2.5, H = -3 (s+3.5) q^-3.5, K = (15 s + 67.5) q^-4.5,
// a = 7.5 q^-3.5, b = 52.5 q^-4.5.  Singular form: G = s^-1.5, H = -3 s^-2.5,
// K = 15 s^-3.5, a = b = 0.)  Source-side sums are reduced across the warp in
// FP32, across the block's warps, then added with one FP64 atomic per source
// and block; target-side sums in FP32 blocks of 64 sources, then FP64.

// S3(s) = sum_m s^m/(2m+7)!! (16 terms: 1e-9 relative at s = 6).  Kummer's series
// of erf gives Gaussian-erf's G = c2 e (1/3 + s S2), H = -3 c2 e S2, K = 15 c2 e S3
// with S2 = 1/15 + s S3 and e = e^{-s/2}: positive terms, where the closed forms
// H = (a - 3G)/s and K = (15 G - a (5 + s))/s^2 lose up to 20x (s = 2) to cancellation.
__device__ __forceinline__ float gerf_S3_series(float s)
{
    float p = 3.1266513920057787e-24f;
    p = fmaf(p, s, 1.2193940428822536e-22f);
    p = fmaf(p, s, 4.5117579586643385e-21f);
    p = fmaf(p, s, 1.5791152855325184e-19f);
    p = fmaf(p, s, 5.211080442257311e-18f);
    p = fmaf(p, s, 1.6154349370997664e-16f);
    p = fmaf(p, s, 4.684761317589322e-15f);
    p = fmaf(p, s, 1.264885555749117e-13f);
    p = fmaf(p, s, 3.1622138893727926e-12f);
    p = fmaf(p, s, 7.273091945557423e-11f);
    p = fmaf(p, s, 1.5273493085670588e-09f);
    p = fmaf(p, s, 2.901963686277412e-08f);
    p = fmaf(p, s, 4.9333382666716e-07f);
    p = fmaf(p, s, 7.4000074000074e-06f);
    p = fmaf(p, s, 9.62000962000962e-05f);
    p = fmaf(p, s, 0.0010582010582010583f);
    p = fmaf(p, s, 0.009523809523809525f);
    return p;
}
constexpr float S_SERIES_ADJ = 6.0f;   // Gaussian-erf adjoint: series below this s (closed forms lose < 3x above)

// (G, H, K, a, b) of kernel K at s (any s > 0) in FP32
template <int K>
__device__ __forceinline__ void adj_coeffs_f32(float s, float& G, float& H, float& Kc, float& a, float& b)
{
    if constexpr (K == K_GAUSERF) {
        if (s > S_FAR_GERF) {
            const float rs = frsqrt(s), rs2 = rs * rs;
            G = rs * rs2; H = -3.0f * G * rs2; Kc = -5.0f * H * rs2; a = 0.0f; b = 0.0f;
        } else {
            const float e = fexp2(s * -0.72134752044448170f);
            a = F_C2 * e;
            b = a;
            if (s < S_SERIES_ADJ) {
                const float p3 = gerf_S3_series(s);
                const float p2 = fmaf(s, p3, 0.066666666666666667f);
                G = a * fmaf(s, p2, 0.33333333333333333f);
                H = -3.0f * a * p2;
                Kc = 15.0f * a * p3;
            } else {
                const float rs = frsqrt(s), rs2 = rs * rs;
                G = gerf_G_erfcx(s, e, rs);
                H = (a - 3.0f * G) * rs2;
                Kc = fmaf(15.0f, G, -a * (5.0f + s)) * rs2 * rs2;
            }
        }
    } else if constexpr (K == K_WNKLMNS) {
        const float q = s + 1.0f;
        const float iq = frcp(q);
        const float iq25 = iq * iq * frsqrt(q);
        const float iq35 = iq25 * iq, iq45 = iq35 * iq;
        G = (s + 2.5f) * iq25;
        H = -3.0f * (s + 3.5f) * iq35;
        Kc = fmaf(15.0f, s, 67.5f) * iq45;
        a = 7.5f * iq35;
        b = 52.5f * iq45;
    } else {   // singular
        const float rs = frsqrt(s), rs2 = rs * rs;
        G = rs * rs2; H = -3.0f * G * rs2; Kc = -5.0f * H * rs2; a = 0.0f; b = 0.0f;
    }
}

// adj_coeffs_f32 for four pairs of one lane with the forms chosen for the whole
// warp, so that the four pairs' chains interleave: the singular form for all
// four, then (Gaussian-erf) the s >= 6 form where any lane of the warp has such a
// pair within the kernel's reach and the series where any has s < 6, each kept
// per pair by its range.  s must be positive and finite (callers pass 1 for
// pairs that contribute nothing).  All 32 lanes must call it.
template <int K>
__device__ __forceinline__ void adj_coeffs4_f32(const float (&s)[4], float (&G)[4], float (&H)[4], float (&Kc)[4],
                                                float (&a)[4], float (&b)[4])
{
    if constexpr (K == K_GAUSERF) {
        float rs[4], rs2[4];
        bool anyser = false, anymid = false;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            rs[q] = frsqrt(s[q]);
            rs2[q] = rs[q] * rs[q];
            G[q] = rs[q] * rs2[q];
            H[q] = -3.0f * G[q] * rs2[q];
            Kc[q] = -5.0f * H[q] * rs2[q];
            a[q] = 0.0f;
            b[q] = 0.0f;
            anyser = anyser || s[q] < S_SERIES_ADJ;
            anymid = anymid || (s[q] >= S_SERIES_ADJ && s[q] <= S_FAR_GERF);
        }
        anyser = __any_sync(0xffffffffu, anyser);
        anymid = __any_sync(0xffffffffu, anymid);
        if (!anyser && !anymid) return;
        float e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            e[q] = fexp2(s[q] * -0.72134752044448170f);
            const bool near = s[q] <= S_FAR_GERF;
            a[q] = near ? F_C2 * e[q] : 0.0f;
            b[q] = a[q];
        }
        if (anymid) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float g = gerf_G_erfcx(s[q], e[q], rs[q]);
                const float h = (a[q] - 3.0f * g) * rs2[q];
                const float k = fmaf(15.0f, g, -a[q] * (5.0f + s[q])) * rs2[q] * rs2[q];
                const bool mid = s[q] >= S_SERIES_ADJ && s[q] <= S_FAR_GERF;
                G[q] = mid ? g : G[q];
                H[q] = mid ? h : H[q];
                Kc[q] = mid ? k : Kc[q];
            }
        }
        if (anyser) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float p3 = gerf_S3_series(s[q]);
                const float p2 = fmaf(s[q], p3, 0.066666666666666667f);
                const bool ser = s[q] < S_SERIES_ADJ;
                G[q] = ser ? a[q] * fmaf(s[q], p2, 0.33333333333333333f) : G[q];
                H[q] = ser ? -3.0f * a[q] * p2 : H[q];
                Kc[q] = ser ? 15.0f * a[q] * p3 : Kc[q];
            }
        }
    } else {
#pragma unroll
        for (int q = 0; q < 4; q++) adj_coeffs_f32<K>(s[q], G[q], H[q], Kc[q], a[q], b[q]);
    }
}

// The seven derivatives of phi for one pair in FP32 (o[0..2] d/d(dx), o[3..5]
// d/dGamma, o[6] d/dsigma), from the coefficients of the pair.
__device__ __forceinline__ void adj_pair_f32(float dx, float dy, float dz, float Gx, float Gy, float Gz, float A,
                                             float B, float Bpr, float dA, float dB, const float (&Ub)[3],
                                             const float (&Jb)[9], const float (&wb)[3], float (&o)[7])
{
    const float cx = fmaf(dy, Gz, -dz * Gy), cy = fmaf(dz, Gx, -dx * Gz), cz = fmaf(dx, Gy, -dy * Gx);
    const float JDx = fmaf(Jb[0], dx, fmaf(Jb[3], dy, Jb[6] * dz));
    const float JDy = fmaf(Jb[1], dx, fmaf(Jb[4], dy, Jb[7] * dz));
    const float JDz = fmaf(Jb[2], dx, fmaf(Jb[5], dy, Jb[8] * dz));
    const float JTcx = fmaf(Jb[0], cx, fmaf(Jb[1], cy, Jb[2] * cz));
    const float JTcy = fmaf(Jb[3], cx, fmaf(Jb[4], cy, Jb[5] * cz));
    const float JTcz = fmaf(Jb[6], cx, fmaf(Jb[7], cy, Jb[8] * cz));
    const float P = fmaf(Ub[0], cx, fmaf(Ub[1], cy, fmaf(Ub[2], cz, fmaf(wb[0], Gx, fmaf(wb[1], Gy, wb[2] * Gz)))));
    const float Q = fmaf(cx, JDx, fmaf(cy, JDy, cz * JDz));
    const float sc = fmaf(B, P, Bpr * Q);
    o[0] = fmaf(sc, dx, fmaf(A, fmaf(Gy, Ub[2], -Gz * Ub[1]), B * (fmaf(Gy, JDz, -Gz * JDy) + JTcx)));
    o[1] = fmaf(sc, dy, fmaf(A, fmaf(Gz, Ub[0], -Gx * Ub[2]), B * (fmaf(Gz, JDx, -Gx * JDz) + JTcy)));
    o[2] = fmaf(sc, dz, fmaf(A, fmaf(Gx, Ub[1], -Gy * Ub[0]), B * (fmaf(Gx, JDy, -Gy * JDx) + JTcz)));
    o[3] = fmaf(A, fmaf(Ub[1], dz, fmaf(-Ub[2], dy, wb[0])), B * fmaf(JDy, dz, -JDz * dy));
    o[4] = fmaf(A, fmaf(Ub[2], dx, fmaf(-Ub[0], dz, wb[1])), B * fmaf(JDz, dx, -JDx * dz));
    o[5] = fmaf(A, fmaf(Ub[0], dy, fmaf(-Ub[1], dx, wb[2])), B * fmaf(JDx, dy, -JDy * dx));
    o[6] = fmaf(dA, P, dB * Q);
}

// Packed source of the FP32-comp adjoint, 48 B: position as a double-float,
// 1/sigma, Gamma, and the particle's index.
struct __align__(16) SrcAdjMixed { float4 a; float4 b; float4 g; };

template <int K>
__global__ void pack_src_adj_mixed(int64_t n, int64_t ns_pad, const double* __restrict__ xs,
                                   const double* __restrict__ gs, const double* __restrict__ sgs,
                                   const TgtPos* __restrict__ order, SrcAdjMixed* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= ns_pad) return;
    SrcAdjMixed p;
    if (o < n) {
        const int64_t i = order[o].idx;
        const double x = xs[3 * i], y = xs[3 * i + 1], z = xs[3 * i + 2];
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        const double sig = (K == K_SING) ? 1.0 : sgs[i];
        p.a = make_float4(xh, yh, zh, (float)(1.0 / sig));
        p.b = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
        p.g = make_float4((float)gs[3 * i], (float)gs[3 * i + 1], (float)gs[3 * i + 2], __int_as_float((int)i));
    } else {   // padding: far away, no strength
        p.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
        p.b = make_float4(0.f, 0.f, 0.f, 0.f);
        p.g = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    }
    out[o] = p;
}

template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
uj_adjoint_mixed_kernel(int64_t nt, const TgtPos* __restrict__ tgt, const double* __restrict__ Ubar,
                        const double* __restrict__ Jbar, int64_t ns_pad, const SrcAdjMixed* __restrict__ src,
                        int64_t per_split, double* xbar, double* gbar, double* sbar)
{
    __shared__ SrcAdjMixed tile[UJ_TILE];
    __shared__ float4 off[UJ_WARPS][UJ_TILE];
    __shared__ float red[UJ_WARPS][UJ_TILE][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 3.0e4, ty = 3.0e4, tz = 3.0e4;
    int64_t idx = 0;
    float Ub[3] = {0.f, 0.f, 0.f}, Jb[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Jb[k] = 0.f;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
#pragma unroll
        for (int k = 0; k < 3; k++) Ub[k] = (float)Ubar[3 * idx + k];
#pragma unroll
        for (int k = 0; k < 9; k++) Jb[k] = (float)Jbar[9 * idx + k];
    }
    const float wb[3] = {Jb[1 + 3 * 2] - Jb[2 + 3 * 1], Jb[2 + 3 * 0] - Jb[0 + 3 * 2], Jb[0 + 3 * 1] - Jb[1 + 3 * 0]};
    const float3 th = make_float3((float)tx, (float)ty, (float)tz);
    const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y), (float)(tz - (double)th.z));
    const double ox = __shfl_sync(0xffffffffu, tx, 0);
    const double oy = __shfl_sync(0xffffffffu, ty, 0);
    const double oz = __shfl_sync(0xffffffffu, tz, 0);
    const float3 oh = make_float3((float)ox, (float)oy, (float)oz);
    const float3 ol = make_float3((float)(ox - (double)oh.x), (float)(oy - (double)oh.y), (float)(oz - (double)oh.z));
    const float3 to = valid ? make_float3((float)(tx - ox), (float)(ty - oy), (float)(tz - oz))
                            : make_float3(3.0e4f, 3.0e4f, 3.0e4f);
    float b2 = valid ? fmaf(to.x, to.x, fmaf(to.y, to.y, to.z * to.z)) : 0.0f;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, m));
    const float r2n = fmaxf(4.0f * b2, 1.0e-30f);
    const float sfar = singular_tail<K>() ? s_far<K>() : 3.0e38f;

    double accd[3] = {0.0, 0.0, 0.0};
    float acc[3] = {0.f, 0.f, 0.f};
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < UJ_TILE / 32; q++) {
            const int j = lane + 32 * q;
            const float4 a = tile[j].a, b = tile[j].b;
            const float sg2 = 1.0f / (a.w * a.w);
            off[warp][j] = make_float4((a.x - oh.x) + (b.x - ol.x), (a.y - oh.y) + (b.y - ol.y),
                                       (a.z - oh.z) + (b.z - ol.z), fmaxf(sfar * sg2, r2n));
        }
        __syncwarp();
#pragma unroll 1
        for (int sb = 0; sb < UJ_TILE; sb += 64) {
#pragma unroll 1
            for (int j0 = sb; j0 < sb + 64; j0 += 4) {
                float dx[4], dy[4], dz[4], r2[4];
                bool far = true;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float4 h = off[warp][j0 + q];
                    dx[q] = to.x - h.x; dy[q] = to.y - h.y; dz[q] = to.z - h.z;
                    r2[q] = fmaf(dx[q], dx[q], fmaf(dy[q], dy[q], dz[q] * dz[q]));
                    far = far && r2[q] > h.w;
                }
                const bool allfar = __all_sync(0xffffffffu, far);
                float ex[4], ey[4], ez[4];
                float A[4], B[4], Bpr[4], dA[4], dB[4];
                if (allfar) {
                    // singular form, in r directly: A = -C4/r^3, B = 3 C4/r^5 = -3 A/r^2,
                    // B'/r = -15 C4/r^7 = -5 B/r^2, no sigma derivative.  Every pair is past
                    // (2 b)^2 > 0, and a lane without a target has zero Ubar, Jbar: all its terms
                    // vanish without the `on` weight.
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        ex[q] = dx[q]; ey[q] = dy[q]; ez[q] = dz[q];
                        const float rs = frsqrt(r2[q]), rs2 = rs * rs;
                        A[q] = -F_C4 * rs * rs2;
                        B[q] = -3.0f * A[q] * rs2;
                        Bpr[q] = -5.0f * B[q] * rs2;
                        dA[q] = 0.0f;
                        dB[q] = 0.0f;
                    }
                } else {
                    float i2[4], sq[4];
                    bool on[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {   // double-float displacement
                        const SrcAdjMixed& sp = tile[j0 + q];
                        ex[q] = (th.x - sp.a.x) + (tl.x - sp.b.x);
                        ey[q] = (th.y - sp.a.y) + (tl.y - sp.b.y);
                        ez[q] = (th.z - sp.a.z) + (tl.z - sp.b.z);
                        const float e2 = fmaf(ex[q], ex[q], fmaf(ey[q], ey[q], ez[q] * ez[q]));
                        on[q] = valid && e2 > 0.0f;
                        i2[q] = sp.a.w * sp.a.w;
                        sq[q] = on[q] ? e2 * i2[q] : 1.0f;
                    }
                    float G[4], H[4], Kc[4], ca[4], cb[4];
                    adj_coeffs4_f32<K>(sq, G, H, Kc, ca, cb);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const float isig = tile[j0 + q].a.w;
                        const float w = on[q] ? 1.0f : 0.0f;
                        const float i3 = i2[q] * isig;
                        A[q] = -F_C4 * i3 * G[q] * w;
                        B[q] = -F_C4 * i3 * i2[q] * H[q] * w;
                        Bpr[q] = -F_C4 * i3 * i2[q] * i2[q] * Kc[q] * w;
                        dA[q] = F_C4 * i2[q] * i2[q] * ca[q] * w;
                        dB[q] = -F_C4 * i3 * i3 * cb[q] * w;
                    }
                }
                float o[4][7];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const SrcAdjMixed& sp = tile[j0 + q];
#pragma unroll
                    for (int k = 0; k < 7; k++) o[q][k] = 0.f;
                    adj_pair_f32(ex[q], ey[q], ez[q], sp.g.x, sp.g.y, sp.g.z, A[q], B[q], Bpr[q], dA[q], dB[q], Ub, Jb,
                                 wb, o[q]);
                    acc[0] += o[q][0]; acc[1] += o[q][1]; acc[2] += o[q][2];
                    o[q][0] = -o[q][0]; o[q][1] = -o[q][1]; o[q][2] = -o[q][2];
                }
                // source-side sums of the four sources over the warp's 32 targets, by reduce-scatter:
                // lanes 16-31 / 0-15 keep sources {2,3} / {0,1}, then lanes with bit 3 set / clear
                // keep the odd / even one, then a butterfly over the remaining 8 lanes; lane 8 g
                // ends with source g's seven sums (21 + 21 shuffles per four sources, not 4 x 35)
                const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0;
                float r[7];
#pragma unroll
                for (int k = 0; k < 7; k++) {
                    const float p0 = (b4 ? o[2][k] : o[0][k]) + __shfl_xor_sync(0xffffffffu, b4 ? o[0][k] : o[2][k], 16);
                    const float p1 = (b4 ? o[3][k] : o[1][k]) + __shfl_xor_sync(0xffffffffu, b4 ? o[1][k] : o[3][k], 16);
                    float v = (b3 ? p1 : p0) + __shfl_xor_sync(0xffffffffu, b3 ? p0 : p1, 8);
#pragma unroll
                    for (int m = 4; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
                    r[k] = v;
                }
                if ((lane & 7) == 0) {
                    const int q = (b4 ? 2 : 0) + (b3 ? 1 : 0);
#pragma unroll
                    for (int k = 0; k < 7; k++) red[warp][j0 + q][k] = r[k];
                }
            }
            // FP64 after each 64 sources, outside the 4-source loop (as a branch in that loop it
            // measured as issued on every iteration)
#pragma unroll
            for (int k = 0; k < 3; k++) { accd[k] += (double)acc[k]; acc[k] = 0.f; }
        }
        __syncthreads();
        const int si = (int)__float_as_int(tile[threadIdx.x].g.w);
        if (si >= 0) {
            // the 4 warps' FP32 sums of this source, added in FP32 (4 terms), then FP64
            double v[7];
#pragma unroll
            for (int k = 0; k < 7; k++)
                v[k] = (double)((red[0][threadIdx.x][k] + red[1][threadIdx.x][k]) +
                                (red[2][threadIdx.x][k] + red[3][threadIdx.x][k]));
#pragma unroll
            for (int k = 0; k < 3; k++) {
                atomicAdd(&xbar[3 * (int64_t)si + k], v[k]);
                atomicAdd(&gbar[3 * (int64_t)si + k], v[3 + k]);
            }
            if (K != K_SING) atomicAdd(&sbar[si], v[6]);
        }
    }
    if (valid) {
#pragma unroll
        for (int k = 0; k < 3; k++) atomicAdd(&xbar[3 * idx + k], accd[k] + (double)acc[k]);
    }
}

// Source splits of the mixed adjoint launch.  The adjoint kernels add their target and source
// sums with atomics (no split partials), so the count is free: the one that minimises the
// launch's length in block slots, ceil(blocks / resident slots) x (tiles per block + 1), where
// the + 1 is a block's fixed cost.  The 127-register mixed kernel holds 4 blocks per SM; at
// 32,000 particles the forward's rule (8 splits: 2,000 blocks, 3.3 waves of 608) leaves the last
// wave 29 % full, and this rule's 12 splits (3,000 blocks, 4.9 waves) measured 3.4 % faster.
// The FP64 adjoint keeps the forward's rule: under this one it measured 6 % slower.
template <typename Kern>
static int adj_splits(Kern kern, int64_t tblocks, int64_t tiles, int num_sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, UJ_THREADS, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int64_t slots = (int64_t)per_sm * num_sms;
    int64_t max_split = tiles / 4 > 1 ? tiles / 4 : 1;         // at least 4 tiles per split
    if (max_split > 65535) max_split = 65535;                   // gridDim.y
    int64_t best = 1, best_cost = INT64_MAX;
    for (int64_t s = 1; s <= max_split; s++) {
        const int64_t per = (tiles + s - 1) / s;
        const int64_t used = (tiles + per - 1) / per;              // no empty splits
        const int64_t cost = ((tblocks * used + slots - 1) / slots) * (per + 1);
        if (cost < best_cost) { best_cost = cost; best = used; }
    }
    return (int)best;
}

template <int K>
static cudaError_t launch_adj_k(const AdjArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                                int64_t* launches)
{
    const int64_t ns_pad = (a.n + UJ_TILE - 1) / UJ_TILE * UJ_TILE;
    const int64_t nt_pad = (a.n + UJ_THREADS - 1) / UJ_THREADS * UJ_THREADS;
    const int64_t tiles = ns_pad / UJ_TILE;
    const int nsplit = a.precision ? adj_splits(uj_adjoint_mixed_kernel<K>, nt_pad / UJ_THREADS, tiles, num_sms)
                                   : uj_num_splits(a.n, a.n, num_sms);
    const int64_t per_split = ((tiles + nsplit - 1) / nsplit) * UJ_TILE;
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(a.n, a.x, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)(nt_pad / UJ_THREADS), (unsigned)nsplit);
    if (a.precision) {
        SrcAdjMixed* src = (SrcAdjMixed*)w.src_pack;
        pack_src_adj_mixed<K><<<(unsigned)((ns_pad + 255) / 256), 256, 0, st>>>(a.n, ns_pad, a.x, a.gam, a.sig, tgt,
                                                                                src);
        uj_adjoint_mixed_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.n, tgt, a.Ubar, a.Jbar, ns_pad, src, per_split,
                                                                a.xbar, a.gbar, a.sbar);
    } else {
        SrcF64* src = (SrcF64*)w.src_pack;
        pack_src_adj<K><<<(unsigned)((ns_pad + 255) / 256), 256, 0, st>>>(a.n, ns_pad, a.x, a.gam, a.sig, src);
        uj_adjoint_f64_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.n, tgt, a.Ubar, a.Jbar, a.n, ns_pad, src, per_split,
                                                              a.xbar, a.gbar, a.sbar);
    }
    *launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_uj_adjoint(const AdjArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                              int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_adj_k<K_SING>(a, w, num_sms, st, launches);
    case K_GAUS: return launch_adj_k<K_GAUS>(a, w, num_sms, st, launches);
    case K_GAUSERF: return launch_adj_k<K_GAUSERF>(a, w, num_sms, st, launches);
    case K_WNKLMNS: return launch_adj_k<K_WNKLMNS>(a, w, num_sms, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
