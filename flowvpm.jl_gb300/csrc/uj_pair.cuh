// uj_pair.cuh -- the UJ pair machinery (FP32-comp and FP64) shared by the all-pairs
// kernels (uj.cu) and the near-field warp-group kernels (leaflist.cu).
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

// Far form of four sources j0..j0+3 whose pairs with every target of the warp are
// known to be past the kernel's reach and past (2 b)^2: FP32 offsets, no test.
// off[].w is 1/sigma^2 for the kernels without a singular tail (Winckelmans).
template <int K>
__device__ __forceinline__ void pair4_far(const float3& to, const float4* __restrict__ off,
                                          const SrcMixed* __restrict__ tile, int j0, float (&u)[3],
                                          float (&jq)[8], float (&w)[3])
{
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float4 h = off[j0 + q];
        const float dx = to.x - h.x, dy = to.y - h.y, dz = to.z - h.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        float G, Q;
        if constexpr (singular_tail<K>()) {
            const float rs = frsqrt(r2);
            const float rs2 = rs * rs;
            G = rs * rs2;
            Q = G * rs2;
        } else {
            near_GQ<K>(r2 * h.w, h.w, G, Q);
        }
        accum_pair(dx, dy, dz, G, Q, tile[j0 + q].gam, u, jq, w);
    }
}

// pair4_far for two targets of the lane (offsets to0, to1), each source read once.
template <int K>
__device__ __forceinline__ void pair4_far2(const float3& to0, const float3& to1, const float4* __restrict__ off,
                                           const SrcMixed* __restrict__ tile, int j0, float (&u0)[3],
                                           float (&jq0)[8], float (&w0)[3], float (&u1)[3], float (&jq1)[8],
                                           float (&w1)[3])
{
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float4 h = off[j0 + q];
        const float4 g = tile[j0 + q].gam;
        {
            const float dx = to0.x - h.x, dy = to0.y - h.y, dz = to0.z - h.z;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            float G, Q;
            if constexpr (singular_tail<K>()) {
                const float rs = frsqrt(r2);
                const float rs2 = rs * rs;
                G = rs * rs2;
                Q = G * rs2;
            } else {
                near_GQ<K>(r2 * h.w, h.w, G, Q);
            }
            accum_pair(dx, dy, dz, G, Q, g, u0, jq0, w0);
        }
        {
            const float dx = to1.x - h.x, dy = to1.y - h.y, dz = to1.z - h.z;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            float G, Q;
            if constexpr (singular_tail<K>()) {
                const float rs = frsqrt(r2);
                const float rs2 = rs * rs;
                G = rs * rs2;
                Q = G * rs2;
            } else {
                near_GQ<K>(r2 * h.w, h.w, G, Q);
            }
            accum_pair(dx, dy, dz, G, Q, g, u1, jq1, w1);
        }
    }
}

// Full form of four sources j0..j0+3, per pair, with the displacement from the
// double-float positions (th + tl) - (a + b); r == 0 contributes nothing.
// off[].w as in pair4_far.
template <int K>
__device__ __forceinline__ void pair4_near(const float3& th, const float3& tl, const float4* __restrict__ off,
                                           const SrcMixed* __restrict__ tile, int j0, float (&u)[3],
                                           float (&jq)[8], float (&w)[3])
{
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
            const float hw = off[j0 + q].w;
            near_GQ<K>(e2 * hw, hw, G, Q);
        }
        const bool nz = e2 > 0.0f;
        G = nz ? G : 0.0f;
        Q = nz ? Q : 0.0f;
        accum_pair(ex, ey, ez, G, Q, tile[j0 + q].gam, u, jq, w);
    }
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
//   SCALED  : (with VOTE = false) the tile holds 1/sigma^2 in a.w and gam carries
//             the 1/sigma^3 of the near form (leaf_pack_lane), for every kernel
template <int K, bool MASK = false, bool VOTE = true, bool SCALED = false>
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
            i2[q] = SCALED ? a.w : singular_tail<K>() ? b.w * b.w : hw[q];
            s4[q] = e2[q] * i2[q];
        }
        near_GQ4<K, false>(s4, i2, G, Q);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float g = G[q], qq = Q[q];
            if constexpr (singular_tail<K>() && !SCALED) {
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

// ----------------------------------------------------------- pair: FP64
// The FP64 pair in the accumulated form of the mixed kernels: with c = dx x Gamma,
//     u += G c,   w += G Gamma,   jq[3 i + j] += Q c_j dx_i,
// G = g / r^3 and Q = -aux / (3 r^3) = (G - g' rho' r^-2 / 3) / r^2 (aux, g' = dg/drho and
// rho' = 1/sigma as in src/FLOWVPM_fmm.jl:122-146); the target's U = -u/(4 pi), and
// J = 3 jq/(4 pi) plus the Kronecker terms of src/FLOWVPM_fmm.jl:148-159 from -w/(4 pi)
// (uj_f64_finish).  Algebraically the reference's terms, regrouped so that the strength
// factor -1/(4 pi) and the products shared by the nine J entries are taken once.
// Gaussian-erf pairs past rho = 9 take g = 1, g' = 0 (the reference's cut) from the
// pack's threshold 81 sigma^2 without forming rho.  Pairs with r^2 == 0 are skipped.
template <int K>
__device__ __forceinline__ void pair_f64_acc(double tx, double ty, double tz, const SrcF64& s, double (&u)[3],
                                             double (&w)[3], double (&jq)[9])
{
    const double dx = tx - s.xy.x, dy = ty - s.xy.y, dz = tz - s.z_isig.x;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 == 0.0) return;
    const double rinv = rsqrt(r2);
    const double rinv2 = rinv * rinv;
    double G, Q;
    if (K == K_SING || (K == K_GAUSERF && r2 > s.gz_sig.y)) {
        G = rinv * rinv2;
        Q = G * rinv2;
    } else {
        const double isig = s.z_isig.y;
        double g, dg;
        g_dgdr_f64<K>(r2 * rinv * isig, g, dg);
        G = g * rinv * rinv2;
        Q = (G - dg * isig * rinv2 * (1.0 / 3.0)) * rinv2;
    }
    const double gx = s.gxy.x, gy = s.gxy.y, gz = s.gz_sig.x;
    const double cx = dy * gz - dz * gy, cy = dz * gx - dx * gz, cz = dx * gy - dy * gx;
    u[0] += G * cx; u[1] += G * cy; u[2] += G * cz;
    w[0] += G * gx; w[1] += G * gy; w[2] += G * gz;
    const double bx = Q * cx, by = Q * cy, bz = Q * cz;
    jq[0] += bx * dx; jq[1] += by * dx; jq[2] += bz * dx;
    jq[3] += bx * dy; jq[4] += by * dy; jq[5] += bz * dy;
    jq[6] += bx * dz; jq[7] += by * dz; jq[8] += bz * dz;
}

// U and J (the layout of pair_f64's acc) from the sums of pair_f64_acc.
__device__ __forceinline__ void uj_f64_finish(const double (&u)[3], const double (&w)[3], const double (&jq)[9],
                                              double (&acc)[12])
{
    constexpr double k = -C4;
#pragma unroll
    for (int m = 0; m < 3; m++) acc[m] = k * u[m];
#pragma unroll
    for (int m = 0; m < 9; m++) acc[3 + m] = (-3.0 * k) * jq[m];
    const double wx = k * w[0], wy = k * w[1], wz = k * w[2];
    acc[4] -= wz;
    acc[5] += wy;
    acc[6] += wz;
    acc[8] -= wx;
    acc[9] -= wy;
    acc[10] += wx;
}

}  // namespace vpm
