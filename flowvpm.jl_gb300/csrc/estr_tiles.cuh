// estr_tiles.cuh -- per-tile boxes of a source pack and the walk over the tiles within
// reach of a warp's targets, shared by the mixed Estr (estr.cu), its adjoint
// (estr_adjoint.cu) and the filter differences (dynamic.cu).  Their Gaussian terms fall
// below FP32 resolution past a reach (zeta_skip_s, dyn_skip_s), so whole 32-source tiles
// out of a warp's reach need not be loaded.
#pragma once
#include "internal.h"
#include "vpm_math.cuh"

namespace vpm {

constexpr int EST_TILE = 32;   // particles per tile (one per lane of a warp)

// The box of every 32-source tile of a pack of ns_pad sources (ns real ones): for tile i,
// box[2 i] = (min x, min y, min z, min 1/sigma^2) and box[2 i + 1] = (max x, max y, max z, 0)
// over its real sources, in FP32 (the high parts); a tile of padding has an empty box.
// Called by whole warps, one tile per warp (ns_pad is a multiple of 32).
__device__ __forceinline__ void estr_tile_box(int64_t o, int64_t ns, float xh, float yh, float zh, float isig2,
                                              float4* __restrict__ box)
{
    const bool real = o < ns;
    float lo[4] = {real ? xh : 3.0e38f, real ? yh : 3.0e38f, real ? zh : 3.0e38f, real ? isig2 : 3.0e38f};
    float hi[3] = {real ? xh : -3.0e38f, real ? yh : -3.0e38f, real ? zh : -3.0e38f};
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
#pragma unroll
        for (int k = 0; k < 4; k++) lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], m));
#pragma unroll
        for (int k = 0; k < 3; k++) hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], m));
    }
    if ((o & (EST_TILE - 1)) == 0) {
        box[2 * (o / EST_TILE)] = make_float4(lo[0], lo[1], lo[2], lo[3]);
        box[2 * (o / EST_TILE) + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    }
}

// The tiles of a warp's source range that can be within reach of its targets, in order:
// lane l tests tile 32 c + l of chunk c against the targets' FP32 box (lo, hi) with the
// tile's box from the pack (estr_tile_box), a ballot gives the chunk's tiles in reach, and
// next() pops them.  A tile is out of reach when its box is farther than zeta_skip_s
// sigma^2 from the target box at the tile's largest sigma (every pair then has
// zeta/zeta(0) < 1e-13); the FP32 boxes shift that bound by a few ulp of the
// coordinates, where the weights are already far below the FP32 resolution of the sums.
// With wfix > 0 the test takes 1/sigma^2 = wfix instead of the tile's (the adjoint's second
// pass, whose tiles hold targets and whose sigma is the lanes' sources').  next_s takes the
// reach skip_s explicitly (the filter differences' dyn_skip_s); skip_s <= 0 or >= 1e37 (a
// kernel without a reach) takes every tile.  All 32 lanes call it, with the same values.
struct TileWalk {
    int n, c;
    unsigned mask;
    __device__ __forceinline__ void init(int ntiles) { n = ntiles; c = -1; mask = 0u; }
    template <int K>
    __device__ __forceinline__ int next(const float4* __restrict__ box, const float4 lo, const float4 hi, int lane,
                                        float wfix = 0.0f)
    {
        return next_s(box, lo, hi, lane, zeta_skip_s<K>(), wfix);
    }
    __device__ __forceinline__ int next_s(const float4* __restrict__ box, const float4 lo, const float4 hi, int lane,
                                          float skip_s, float wfix = 0.0f)
    {
        while (mask == 0u) {
            if ((c + 1) * 32 >= n) return -1;
            ++c;
            const int i = c * 32 + lane;
            bool in = i < n;
            if (skip_s > 0.0f && skip_s < 1.0e37f && in) {
                const float4 bl = box[2 * i], bh = box[2 * i + 1];
                const float ex = fmaxf(fmaxf(lo.x - bh.x, bl.x - hi.x), 0.0f);
                const float ey = fmaxf(fmaxf(lo.y - bh.y, bl.y - hi.y), 0.0f);
                const float ez = fmaxf(fmaxf(lo.z - bh.z, bl.z - hi.z), 0.0f);
                in = !(fmaf(ex, ex, fmaf(ey, ey, ez * ez)) * (wfix > 0.0f ? wfix : bl.w) > skip_s);
            }
            mask = __ballot_sync(0xffffffffu, in);
        }
        const int b = __ffs(mask) - 1;
        mask &= mask - 1u;
        return c * 32 + b;
    }
};

}  // namespace vpm
