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
#include "dyn_math.cuh"
#include "internal.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

#include <cmath>

namespace vpm {

constexpr int DYN_THREADS = 128;
constexpr int DYN_TILE = 128;

// dJ of every target (Morton order) from every source of the pack (same
// order), accumulated into dJ[idx*9 + k].  Pair math as above; dx as a
// double-float (x_hi, x_lo); FP32 sums over 64-source blocks, FP64 beyond.
template <int K, int M>
__global__ void __launch_bounds__(DYN_THREADS)
uj_filter_diff_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad, const SrcMixed* __restrict__ src,
                      float hm, int panels, double* __restrict__ dJ)
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

    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] = 0.0;
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
            float f[9];
#pragma unroll
            for (int k = 0; k < 9; k++) f[k] = 0.0f;
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
                float ex[4], ey[4], ez[4], r2[4];
                bool on[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const SrcMixed& s = tile[j0 + q];
                    ex[q] = (th.x - s.a.x) + (tl.x - s.b.x);
                    ey[q] = (th.y - s.a.y) + (tl.y - s.b.y);
                    ez[q] = (th.z - s.a.z) + (tl.z - s.b.z);
                    r2[q] = fmaf(ex[q], ex[q], fmaf(ey[q], ey[q], ez[q] * ez[q]));
                    on[q] = r2[q] > 0.0f;
                    r2[q] = on[q] ? r2[q] : 1.0f;
                }
#pragma unroll
                for (int q = 0; q < 4; q++)
                    filter_diff_pair<K, M>(ex[q], ey[q], ez[q], r2[q], tile[j0 + q].b.w, tile[j0 + q].gam, hm,
                                           panels, on[q], f);
            }
#pragma unroll
            for (int k = 0; k < 9; k++) acc[k] += (double)f[k];
        }
    }
    if (!valid) return;
#pragma unroll
    for (int k = 0; k < 9; k++) dJ[9 * (int64_t)idx + k] += acc[k];
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
    const int m = filter_panels(ha);
    if (m == 1)
        uj_filter_diff_kernel<K, 1><<<grid, DYN_THREADS, 0, st>>>(n, tgt, ns_pad, src, (float)ha, 1, dJ);
    else
        uj_filter_diff_kernel<K, 0><<<grid, DYN_THREADS, 0, st>>>(n, tgt, ns_pad, src, (float)(ha / m), m, dJ);
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
