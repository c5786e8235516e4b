// dynamic.cu -- the test-filter differences of the dynamic SFS procedure,
// evaluated directly.
//
// The pseudo-three-level dynamic procedure (src/FLOWVPM_subfilterscale.jl:
// 447-673) evaluates UJ and Estr once with every core size scaled by alpha
// (0.999 for the recommended two-level model) and once at sigma, and divides
// differences of the two: M = S(J_alpha) - S(J) and SFS_alpha - SFS.  Those
// differences are ~1e-3 of the terms, so when each term carries FP32 rounding
// (~1e-7 for J, ~1e-6 for SFS) the differences carry 1e-4 .. 1e-2, and the
// clipped ratio C turns that noise into extra dissipation.  Here the
// differences are evaluated as such, per pair:
//
//   dJ_t = J_t(alpha sigma) - J_t(sigma) = sum_s [j(dx, Gamma_s, alpha sigma_s) - j(dx, Gamma_s, sigma_s)]
//
// from the pair term of src/FLOWVPM_fmm.jl:112-160, whose sigma dependence
// sits in g(rho) and g'(rho)/sigma (rho = r/sigma): with h = rho (1/alpha - 1),
//   dg  = g(rho/alpha) - g(rho)                  = int_rho^{rho+h} g'(t) dt
//   dg1 = g'(rho/alpha)/alpha - g'(rho)          = (1/rho) int_rho^{rho+h} (t g''(t) + g'(t)) dt
// both by two-point Gauss-Legendre (error ~h^5, negligible at h ~ 1e-3 rho;
// wider filters take more panels),
// so each difference keeps FP32 relative accuracy.  Pairs beyond the kernel's
// reach (s = rho^2 above dyn_skip_s) are skipped warp-wide; Winckelmans has
// no such reach.  The SFS difference splits, exactly, as
//   SFS(alpha sigma; J + dJ) - SFS(sigma; J)
//     = sum_s [zeta~(r, alpha sigma_s) - zeta~(r, sigma_s)] (J_t - J_s)^T Gamma_s   (weight difference)
//     + Estr(alpha sigma; dJ)                                                     (an ordinary Estr)
// with zeta~(r, sigma) = zeta(r/sigma)/sigma^3; the first is the Estr kernel in
// its weight-difference mode (estr.cu), the second the Estr kernel itself.
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
        const float e = F_C2 * exp2f(t * t * -0.72134752044448170f);   // sqrt(2/pi) e^{-t^2/2}
        d1 = t * t * e;
        d2 = t * (2.0f - t * t) * e;
    } else if constexpr (K == K_GAUS) {
        const float t3 = t * t * t;
        const float e = exp2f(t3 * -1.4426950408889634f);              // e^{-t^3}
        d1 = 3.0f * t * t * e;
        d2 = t * (6.0f - 9.0f * t3) * e;
    } else if constexpr (K == K_WNKLMNS) {
        const float q = fmaf(t, t, 1.0f);
        const float iq = __frcp_rn(q);
        const float iq35 = iq * iq * iq * rsqrtf(q);                   // q^-3.5
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

// (dg, dg1) of one pair at rho for the filter factor alpha (ha = 1/alpha - 1):
// m two-point Gauss-Legendre panels on [rho, rho/alpha] (m from ha, warp-uniform;
// one panel for alpha = 0.999, eight for alpha = 0.667)
template <int K>
__device__ __forceinline__ void filter_diff(float rho, float ha, int m, float& dg, float& dg1)
{
    const float h = rho * ha / (float)m;
    const float o = 0.28867513459481287f * h;    // h / (2 sqrt 3)
    float s1 = 0.0f, s2 = 0.0f;
    for (int k = 0; k < m; k++) {
        const float c = fmaf((float)k + 0.5f, h, rho);
        float a1, a2, b1, b2;
        g_d1_d2_f32<K>(c - o, a1, a2);
        g_d1_d2_f32<K>(c + o, b1, b2);
        s1 += a1 + b1;
        s2 += fmaf(c - o, a2, a1) + fmaf(c + o, b2, b1);
    }
    dg = 0.5f * h * s1;
    dg1 = 0.5f * h * s2 / rho;
}

// Gauss-Legendre panels for the filter factor: the two-point rule's error per
// panel ~ (h/m)^5, so m grows with ha = 1/alpha - 1
inline int filter_panels(double ha) { return ha <= 0.0625 ? 1 : (int)std::ceil(ha * 16.0); }

constexpr int DYN_THREADS = 128;
constexpr int DYN_TILE = 128;

// dJ of every target (Morton order) from every source of the pack (same
// order), accumulated into dJ[idx*9 + k].  Pair math as above; dx as a
// double-float (x_hi, x_lo); FP32 sums over 64-source blocks, FP64 beyond.
template <int K>
__global__ void __launch_bounds__(DYN_THREADS)
uj_filter_diff_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad, const SrcMixed* __restrict__ src,
                      float ha, int panels, double* __restrict__ dJ)
{
    __shared__ SrcMixed tile[DYN_TILE];
    __shared__ float4 off[DYN_THREADS / 32][DYN_TILE];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * DYN_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 3.0e4, ty = 3.0e4, tz = 3.0e4;
    int32_t idx = 0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const float3 th = make_float3((float)tx, (float)ty, (float)tz);
    const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y), (float)(tz - (double)th.z));
    const double ox = __shfl_sync(0xffffffffu, tx, 0);
    const double oy = __shfl_sync(0xffffffffu, ty, 0);
    const double oz = __shfl_sync(0xffffffffu, tz, 0);
    const float3 to = make_float3((float)(tx - ox), (float)(ty - oy), (float)(tz - oz));
    const float skip = dyn_skip_s<K>();

    double acc[12];
#pragma unroll
    for (int k = 0; k < 12; k++) acc[k] = 0.0;
    for (int64_t base = 0; base < ns_pad; base += DYN_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < DYN_TILE / 32; q++) {
            const int j = lane + 32 * q;
            const float4 a = tile[j].a, b = tile[j].b;
            // FP32 offset from the warp origin (for the skip test only) and 1/sigma^2
            off[warp][j] = make_float4((float)(((double)a.x + (double)b.x) - ox), (float)(((double)a.y + (double)b.y) - oy),
                                       (float)(((double)a.z + (double)b.z) - oz), b.w * b.w);
        }
        __syncwarp();
#pragma unroll 1
        for (int sb = 0; sb < DYN_TILE; sb += 64) {
            float f[12];
#pragma unroll
            for (int k = 0; k < 12; k++) f[k] = 0.0f;
#pragma unroll 1
            for (int j0 = sb; j0 < sb + 64; j0 += 4) {
                bool far = true;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float4 h = off[warp][j0 + q];
                    const float dx = to.x - h.x, dy = to.y - h.y, dz = to.z - h.z;
                    far = far && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * h.w > skip;
                }
                if (__all_sync(0xffffffffu, far || !valid)) continue;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const SrcMixed& s = tile[j0 + q];
                    const float ex = (th.x - s.a.x) + (tl.x - s.b.x);
                    const float ey = (th.y - s.a.y) + (tl.y - s.b.y);
                    const float ez = (th.z - s.a.z) + (tl.z - s.b.z);
                    const float r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                    if (!(r2 > 0.0f)) continue;
                    const float isig = s.b.w;
                    const float rinv = rsqrtf(r2);
                    const float rho = r2 * rinv * isig;
                    float dg, dg1;
                    filter_diff<K>(rho, ha, panels, dg, dg1);
                    // Gamma * (-1/(4 pi)) from the pack (Winckelmans packs it over sigma^3)
                    float gx = s.gam.x, gy = s.gam.y, gz = s.gam.z;
                    if constexpr (!singular_tail<K>()) {
                        const float sig3 = 1.0f / (isig * isig * isig);
                        gx *= sig3; gy *= sig3; gz *= sig3;
                    }
                    const float ri2 = rinv * rinv, ri3 = ri2 * rinv;
                    // c = -(dx x Gamma)/(4 pi r^3); dU = dg c; a = daux c with
                    // daux = dg1 / (sigma r) - 3 dg / r^2; daux2 = -dg / (4 pi r^3)
                    const float cx = ri3 * (ey * gz - ez * gy), cy = ri3 * (ez * gx - ex * gz), cz = ri3 * (ex * gy - ey * gx);
                    const float daux = fmaf(dg1 * isig, rinv, -3.0f * dg * ri2);
                    const float dax2 = dg * ri3;   // times -Gamma/(4 pi): the packed gam
                    const float a1 = daux * cx, a2 = daux * cy, a3 = daux * cz;
                    f[0] = fmaf(dg, cx, f[0]); f[1] = fmaf(dg, cy, f[1]); f[2] = fmaf(dg, cz, f[2]);
                    f[3] = fmaf(a1, ex, f[3]);
                    f[4] = fmaf(a2, ex, fmaf(-dax2, gz, f[4]));
                    f[5] = fmaf(a3, ex, fmaf(dax2, gy, f[5]));
                    f[6] = fmaf(a1, ey, fmaf(dax2, gz, f[6]));
                    f[7] = fmaf(a2, ey, f[7]);
                    f[8] = fmaf(a3, ey, fmaf(-dax2, gx, f[8]));
                    f[9] = fmaf(a1, ez, fmaf(-dax2, gy, f[9]));
                    f[10] = fmaf(a2, ez, fmaf(dax2, gx, f[10]));
                    f[11] = fmaf(a3, ez, f[11]);
                }
            }
#pragma unroll
            for (int k = 0; k < 12; k++) acc[k] += (double)f[k];
        }
    }
    if (!valid) return;
#pragma unroll
    for (int k = 0; k < 9; k++) dJ[9 * (int64_t)idx + k] += acc[3 + k];
}

template <int K>
__global__ void pack_src_dyn(int64_t ns, int64_t ns_pad, const double* __restrict__ xs, const double* __restrict__ gs,
                             const double* __restrict__ sgs, SrcMixed* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ns_pad) return;
    SrcMixed p;
    if (i < ns) {
        const double px = xs[3 * i], py = xs[3 * i + 1], pz = xs[3 * i + 2];
        const float xh = (float)px, yh = (float)py, zh = (float)pz;
        const double sig = (K == K_SING) ? 1.0 : sgs[i];
        const double k = singular_tail<K>() ? -C4 : -C4 / (sig * sig * sig);
        p.a = make_float4(xh, yh, zh, (float)(sig * sig));
        p.b = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), (float)(1.0 / sig));
        p.gam = make_float4((float)(k * gs[3 * i]), (float)(k * gs[3 * i + 1]), (float)(k * gs[3 * i + 2]), 0.f);
    } else {   // padding: far away, no strength
        p.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
        p.b = make_float4(0.f, 0.f, 0.f, 1.f);
        p.gam = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    out[i] = p;
}

size_t dyn_src_pack_bytes(int64_t ns) { return (size_t)((ns + DYN_TILE - 1) / DYN_TILE * DYN_TILE) * sizeof(SrcMixed); }

template <int K>
static cudaError_t launch_uj_filter_diff_k(int64_t n, const double* x, const double* gam, const double* sig,
                                           double alpha, double* dJ, const Workspace& w, cudaStream_t st,
                                           int64_t* launches)
{
    const int64_t ns_pad = (n + DYN_TILE - 1) / DYN_TILE * DYN_TILE;
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(n, x, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    SrcMixed* src = (SrcMixed*)w.src_pack;
    pack_src_dyn<K><<<(unsigned)((ns_pad + 255) / 256), 256, 0, st>>>(n, ns_pad, x, gam, sig, src);
    const unsigned grid = (unsigned)((n + DYN_THREADS - 1) / DYN_THREADS);
    const double ha = 1.0 / alpha - 1.0;
    uj_filter_diff_kernel<K><<<grid, DYN_THREADS, 0, st>>>(n, tgt, ns_pad, src, (float)ha, filter_panels(ha), dJ);
    *launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_uj_filter_diff(int64_t n, const double* x, const double* gam, const double* sig, double alpha,
                                  double* dJ, int kernel, const Workspace& w, cudaStream_t st, int64_t* launches)
{
    if (n <= 0) return cudaSuccess;
    switch (kernel) {
    case K_SING: return cudaSuccess;   // g = 1: no sigma dependence
    case K_GAUS: return launch_uj_filter_diff_k<K_GAUS>(n, x, gam, sig, alpha, dJ, w, st, launches);
    case K_GAUSERF: return launch_uj_filter_diff_k<K_GAUSERF>(n, x, gam, sig, alpha, dJ, w, st, launches);
    case K_WNKLMNS: return launch_uj_filter_diff_k<K_WNKLMNS>(n, x, gam, sig, alpha, dJ, w, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
