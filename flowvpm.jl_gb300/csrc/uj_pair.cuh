// uj_pair.cuh -- the mixed (FP32-comp) UJ pair machinery shared by the all-pairs
// kernel (uj.cu) and the near-field warp-group kernel (leaflist.cu).
#pragma once
#include "internal.h"
#include "vpm_math.cuh"

namespace vpm {

// true for kernels equal to their singular form beyond some rho
template <int K>
__host__ __device__ constexpr bool singular_tail() { return K != K_WNKLMNS; }

// ----------------------------------------------------------- pair: mixed
// Accumulates U += G c, W += G gam, J' += Q c_i dx_j with c = dx x gam.  The
// trace of J' vanishes (c . dx = 0), so J'_33 is not accumulated; the caller
// sets it to -(J'_11 + J'_22).
__device__ __forceinline__ void accum_pair(float dx, float dy, float dz, float G, float Q, const float4& g,
                                           float (&u)[3], float (&jq)[8], float (&w)[3])
{
    const float cx = fmaf(dy, g.z, -dz * g.y);
    const float cy = fmaf(dz, g.x, -dx * g.z);
    const float cz = fmaf(dx, g.y, -dy * g.x);
    u[0] = fmaf(G, cx, u[0]);
    u[1] = fmaf(G, cy, u[1]);
    u[2] = fmaf(G, cz, u[2]);
    w[0] = fmaf(G, g.x, w[0]);
    w[1] = fmaf(G, g.y, w[1]);
    w[2] = fmaf(G, g.z, w[2]);
    const float bx = Q * cx, by = Q * cy, bz = Q * cz;
    jq[0] = fmaf(bx, dx, jq[0]);
    jq[1] = fmaf(by, dx, jq[1]);
    jq[2] = fmaf(bz, dx, jq[2]);
    jq[3] = fmaf(bx, dy, jq[3]);
    jq[4] = fmaf(by, dy, jq[4]);
    jq[5] = fmaf(bz, dy, jq[5]);
    jq[6] = fmaf(bx, dz, jq[6]);
    jq[7] = fmaf(by, dz, jq[7]);
}

// Four sources j0..j0+3 of the tile against this lane's target.
//   to      : target offset from the warp origin (FP32)
//   th, tl  : target double-float position
//   r2n     : (2 b)^2, b = the warp's extent around its origin
//   mybit   : with MASK, this lane's bit in each source's target mask (the bits
//             of gam.w): a source whose mask lacks it contributes nothing (every
//             lane still votes and computes)
//   VOTE    : false skips the far vote and takes the near form for every group
//             (the near-field lists, whose pairs are almost all within reach),
//             four pairs at a time with the form chosen warp-wide (near_GQ4)
//             and no singular branch; off[].w (1/sigma^2 for Winckelmans) is
//             still read
template <int K, bool MASK = false, bool VOTE = true>
__device__ __forceinline__ void pair4_mixed(const float3& to, const float3& th, const float3& tl, float r2n,
                                            const float4* __restrict__ off, const SrcMixed* __restrict__ tile,
                                            int j0, float (&u)[3], float (&jq)[8], float (&w)[3],
                                            unsigned mybit = 0u)
{
    float dx[4], dy[4], dz[4], r2[4], hw[4];
    bool far = VOTE;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if constexpr (VOTE || !singular_tail<K>()) {
            const float4 h = off[j0 + q];
            hw[q] = h.w;
            if constexpr (VOTE) {
                dx[q] = to.x - h.x;
                dy[q] = to.y - h.y;
                dz[q] = to.z - h.z;
                r2[q] = fmaf(dx[q], dx[q], fmaf(dy[q], dy[q], dz[q] * dz[q]));
                far = far && (r2[q] > (singular_tail<K>() ? h.w : r2n));
            }
        }
    }
    if (VOTE && __all_sync(0xffffffffu, far)) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float G, Q;
            if constexpr (singular_tail<K>()) {
                const float rs = frsqrt(r2[q]);
                const float rs2 = rs * rs;
                G = rs * rs2;
                Q = G * rs2;
            } else {
                near_GQ<K>(r2[q] * hw[q], hw[q], G, Q);
            }
            const float4 gq = tile[j0 + q].gam;
            if constexpr (MASK) {
                const bool on = (__float_as_uint(gq.w) & mybit) != 0u;
                G = on ? G : 0.0f;
                Q = on ? Q : 0.0f;
            }
            accum_pair(dx[q], dy[q], dz[q], G, Q, gq, u, jq, w);
        }
    } else if constexpr (VOTE) {
        // near groups of the all-pairs kernels: per pair (their register budget
        // does not hold four pairs' near-form intermediates)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float4 a = tile[j0 + q].a, b = tile[j0 + q].b;
            const float ex = (th.x - a.x) + (tl.x - b.x);
            const float ey = (th.y - a.y) + (tl.y - b.y);
            const float ez = (th.z - a.z) + (tl.z - b.z);
            const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
            float G, Q;
            if constexpr (singular_tail<K>()) {
                const float isig2 = b.w * b.w;
                near_GQ<K>(e2 * isig2, isig2, G, Q);
                const float isig3 = isig2 * b.w;
                G *= isig3;
                Q *= isig3;
            } else {
                near_GQ<K>(e2 * hw[q], hw[q], G, Q);
            }
            const bool nz = e2 > 0.0f;
            G = nz ? G : 0.0f;
            Q = nz ? Q : 0.0f;
            const float4 gq = tile[j0 + q].gam;
            if constexpr (MASK) {
                const bool on = (__float_as_uint(gq.w) & mybit) != 0u;
                G = on ? G : 0.0f;
                Q = on ? Q : 0.0f;
            }
            accum_pair(ex, ey, ez, G, Q, gq, u, jq, w);
        }
    } else {
        // every group (the near-field lists): the four pairs' forms chosen warp-wide
        float ex[4], ey[4], ez[4], e2[4], s4[4], i2[4], G[4], Q[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float4 a = tile[j0 + q].a, b = tile[j0 + q].b;
            ex[q] = (th.x - a.x) + (tl.x - b.x);
            ey[q] = (th.y - a.y) + (tl.y - b.y);
            ez[q] = (th.z - a.z) + (tl.z - b.z);
            e2[q] = fmaf(ex[q], ex[q], fmaf(ey[q], ey[q], ez[q] * ez[q]));
            i2[q] = singular_tail<K>() ? b.w * b.w : hw[q];
            s4[q] = e2[q] * i2[q];
        }
        near_GQ4<K, false>(s4, i2, G, Q);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float g = G[q], qq = Q[q];
            if constexpr (singular_tail<K>()) {
                const float isig3 = i2[q] * tile[j0 + q].b.w;
                g *= isig3;
                qq *= isig3;
            }
            const float4 gq = tile[j0 + q].gam;
            bool on = e2[q] > 0.0f;
            if constexpr (MASK) on = on && (__float_as_uint(gq.w) & mybit) != 0u;
            g = on ? g : 0.0f;
            qq = on ? qq : 0.0f;
            accum_pair(ex[q], ey[q], ez[q], g, qq, gq, u, jq, w);
        }
    }
}

}  // namespace vpm
