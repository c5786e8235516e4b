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
#include "estr_tiles.cuh"
#include "internal.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

#include <cmath>

namespace vpm {

constexpr int DYN_THREADS = 128;
constexpr int DYN_TILE = 128;                 // padding of the source pack
constexpr int DYN_WARPS = DYN_THREADS / 32;
constexpr int DYN_WT = EST_TILE;              // sources per tile of a warp's stream
constexpr int DYN_FLUSH_TILES = 2;            // evaluated tiles between FP64 adds (64 sources)

__device__ __forceinline__ void dyn_stage(SrcMixed* d, const SrcMixed* g)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(d);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(&g->a) : "memory");
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa + 16u), "l"(&g->b) : "memory");
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa + 32u), "l"(&g->gam) : "memory");
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void dyn_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// dJ of every target (Morton order) from every source of the pack (same
// order), accumulated into dJ[idx*9 + k].  Pair math as above; dx as a
// double-float (x_hi, x_lo).  Each warp streams the sources on its own, 32 per
// tile, double-buffered with cp.async, over the tiles whose pack box is within
// dyn_skip_s of its targets (TileWalk); a loaded tile is skipped when each of its
// sources is out of reach of the warp's box of targets, a 4-source group when each
// of its pairs is (FP32 offsets from the warp's first target, df_offset).  FP32
// sums over DYN_FLUSH_TILES evaluated tiles, FP64 beyond.
template <int K, int M>
__global__ void __launch_bounds__(DYN_THREADS)
uj_filter_diff_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad, const SrcMixed* __restrict__ src,
                      const float4* __restrict__ box, float hm, int panels, double* __restrict__ dJ)
{
    __shared__ SrcMixed stage[DYN_WARPS][2][DYN_WT];
    __shared__ float4 offs[DYN_WARPS][2][DYN_WT];
    __shared__ float4 wbox[DYN_WARPS][4];   // target offsets low, high; FP32 positions low, high
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * DYN_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    int32_t idx = 0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const float3 th = make_float3((float)tx, (float)ty, (float)tz);
    const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y), (float)(tz - (double)th.z));
    const float3 oh = make_float3(__shfl_sync(0xffffffffu, th.x, 0), __shfl_sync(0xffffffffu, th.y, 0),
                                  __shfl_sync(0xffffffffu, th.z, 0));
    const float3 ol = make_float3(__shfl_sync(0xffffffffu, tl.x, 0), __shfl_sync(0xffffffffu, tl.y, 0),
                                  __shfl_sync(0xffffffffu, tl.z, 0));
    const float3 to = make_float3(df_offset(th.x, tl.x, oh.x, ol.x), df_offset(th.y, tl.y, oh.y, ol.y),
                                  df_offset(th.z, tl.z, oh.z, ol.z));
    {
        float v[12];
        const float p[6] = {to.x, to.y, to.z, th.x, th.y, th.z};
#pragma unroll
        for (int k = 0; k < 6; k++) {   // minima of (offset, position) and of their negatives
            v[k] = valid ? p[k] : 3.0e38f;
            v[6 + k] = valid ? -p[k] : 3.0e38f;
        }
#pragma unroll
        for (int m = 16; m > 0; m >>= 1)
#pragma unroll
            for (int k = 0; k < 12; k++) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], m));
        if (lane == 0) {
            wbox[warp][0] = make_float4(v[0], v[1], v[2], 0.f);
            wbox[warp][1] = make_float4(-v[6], -v[7], -v[8], 0.f);
            wbox[warp][2] = make_float4(v[3], v[4], v[5], 0.f);
            wbox[warp][3] = make_float4(-v[9], -v[10], -v[11], 0.f);
        }
        __syncwarp();
    }
    const float skip = dyn_skip_s<K>();
    double acc[9];
    float f[9];
#pragma unroll
    for (int k = 0; k < 9; k++) { acc[k] = 0.0; f[k] = 0.0f; }
    const int ntiles = (int)(ns_pad / DYN_WT);
    const SrcMixed* wsrc = src + lane;
    TileWalk walk;
    walk.init(ntiles);
    int cur = walk.next_s(box, wbox[warp][2], wbox[warp][3], lane, skip);
    if (cur >= 0) dyn_stage(&stage[warp][0][lane], wsrc + (int64_t)cur * DYN_WT);
    int in_flush = 0, buf = 0;
    while (cur >= 0) {
        const int nxt = walk.next_s(box, wbox[warp][2], wbox[warp][3], lane, skip);
        if (nxt >= 0) {
            dyn_stage(&stage[warp][buf ^ 1][lane], wsrc + (int64_t)nxt * DYN_WT);
            dyn_wait<1>();
        } else {
            dyn_wait<0>();
        }
        __syncwarp();
        bool beyond;
        {   // this lane's source: FP32 offset and 1/sigma^2, and whether it is out of reach of the warp's box
            const float4 a = stage[warp][buf][lane].a, b = stage[warp][buf][lane].b;
            const float px = df_offset(a.x, b.x, oh.x, ol.x), py = df_offset(a.y, b.y, oh.y, ol.y),
                        pz = df_offset(a.z, b.z, oh.z, ol.z);
            const float isig2 = b.w * b.w;
            offs[warp][buf][lane] = make_float4(px, py, pz, isig2);
            const float4 lo = wbox[warp][0], hi = wbox[warp][1];
            const float ex = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.0f);
            const float ey = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.0f);
            const float ez = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.0f);
            beyond = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) * isig2 > skip;
        }
        __syncwarp();
        if (!__all_sync(0xffffffffu, beyond)) {
#pragma unroll 1
            for (int j0 = 0; j0 < DYN_WT; j0 += 4) {
                bool far = true;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float4 h = offs[warp][buf][j0 + q];
                    const float dx = to.x - h.x, dy = to.y - h.y, dz = to.z - h.z;
                    far = far && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * h.w > skip;
                }
                if (__all_sync(0xffffffffu, far || !valid)) continue;
                float ex[4], ey[4], ez[4], r2[4];
                bool on[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const SrcMixed& sq = stage[warp][buf][j0 + q];
                    ex[q] = (th.x - sq.a.x) + (tl.x - sq.b.x);
                    ey[q] = (th.y - sq.a.y) + (tl.y - sq.b.y);
                    ez[q] = (th.z - sq.a.z) + (tl.z - sq.b.z);
                    r2[q] = fmaf(ex[q], ex[q], fmaf(ey[q], ey[q], ez[q] * ez[q]));
                    on[q] = valid && r2[q] > 0.0f;
                    r2[q] = on[q] ? r2[q] : 1.0f;
                }
#pragma unroll
                for (int q = 0; q < 4; q++)
                    filter_diff_pair<K, M>(ex[q], ey[q], ez[q], r2[q], stage[warp][buf][j0 + q].b.w,
                                           stage[warp][buf][j0 + q].gam, hm, panels, on[q], f);
            }
            if (++in_flush == DYN_FLUSH_TILES) {   // evaluated tiles only
                in_flush = 0;
#pragma unroll
                for (int k = 0; k < 9; k++) { acc[k] += (double)f[k]; f[k] = 0.0f; }
            }
        }
        __syncwarp();   // every lane is done with `buf` before it is refilled
        cur = nxt;
        buf ^= 1;
    }
    if (!valid) return;
#pragma unroll
    for (int k = 0; k < 9; k++) dJ[9 * (int64_t)idx + k] += acc[k] + (double)f[k];
}

template <int K>
__global__ void pack_src_dyn(int64_t ns, int64_t ns_pad, const double* __restrict__ xs, const double* __restrict__ gs,
                             const double* __restrict__ sgs, SrcMixed* __restrict__ out, float4* __restrict__ box)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ns_pad) return;   // whole warps: ns_pad is a multiple of 32
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
    estr_tile_box(i, ns, p.a.x, p.a.y, p.a.z, p.b.w * p.b.w, box);
}

// the records, then two float4 per 32-source tile (estr_tile_box)
size_t dyn_src_pack_bytes(int64_t ns)
{
    const size_t n = (size_t)((ns + DYN_TILE - 1) / DYN_TILE * DYN_TILE);
    return n * sizeof(SrcMixed) + n / DYN_WT * 2 * sizeof(float4);
}

template <int K>
static cudaError_t launch_uj_filter_diff_k(int64_t n, const double* x, const double* gam, const double* sig,
                                           double alpha, double* dJ, const Workspace& w, cudaStream_t st,
                                           int64_t* launches)
{
    const int64_t ns_pad = (n + DYN_TILE - 1) / DYN_TILE * DYN_TILE;
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(n, x, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    if (w.src_pack_bytes < dyn_src_pack_bytes(n)) return cudaErrorInvalidValue;
    SrcMixed* src = (SrcMixed*)w.src_pack;
    float4* box = (float4*)(src + ns_pad);
    pack_src_dyn<K><<<(unsigned)((ns_pad + 255) / 256), 256, 0, st>>>(n, ns_pad, x, gam, sig, src, box);
    const unsigned grid = (unsigned)((n + DYN_THREADS - 1) / DYN_THREADS);
    const double ha = 1.0 / alpha - 1.0;
    const int m = filter_panels(ha);
    if (m == 1)
        uj_filter_diff_kernel<K, 1><<<grid, DYN_THREADS, 0, st>>>(n, tgt, ns_pad, src, box, (float)ha, 1, dJ);
    else
        uj_filter_diff_kernel<K, 0><<<grid, DYN_THREADS, 0, st>>>(n, tgt, ns_pad, src, box, (float)(ha / m), m, dJ);
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
