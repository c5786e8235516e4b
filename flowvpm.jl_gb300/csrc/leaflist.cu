// leaflist.cu -- near-field P2P over octree leaf pairs: the direct leg of
// UJ_fmm (FastMultipole's direct_list, src/FLOWVPM_UJ.jl:90-100) and the Estr
// pass over the same list (Estr_fmm!, src/FLOWVPM_subfilterscale_models.jl:94-188).
//
// Particles are processed in the tree's Morton order (nearfield.cu), so every
// leaf is a contiguous range.  Leaves are small (leaf_size is a maximum; a
// uniform cloud at leaf_size 64 averages ~11 particles a leaf), so work is not
// cut per leaf: one warp takes 32 consecutive Morton positions -- a few
// neighbouring leaves -- and walks the union of their source lists as
// particle intervals, each with the mask of the warp's leaves that need it.
// Sources are staged 32 at a time in the warp's shared memory, the tiles
// running on across interval boundaries so that they are full, each source
// carrying its interval's mask; a lane whose leaf is not in a source's mask
// computes that pair with zero weight.  Pair math is
// that of the all-pairs kernels (uj_pair.cuh for FP32-comp, the reference
// formula for FP64); Estr uses the factored form of estr.cu with the self
// pair excluded by position.
#include "dyn_math.cuh"
#include "internal.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

namespace vpm {

constexpr int NF_WARPS = 4;                  // warp groups per block
constexpr int NF_THREADS = 32 * NF_WARPS;
constexpr int NF_BLK_TILES = 2;              // 32-source tiles summed in FP32 per block
constexpr int NF_ESTR_FLUSH = 8;             // nf_estr: tiles of compensated FP32 sums between FP64 adds
constexpr int NF_MID_BLKS = 4;               // blocks summed in FP32 before the FP64 add
#ifndef VPM_NF_MIN_BLOCKS
#define VPM_NF_MIN_BLOCKS 4                  // resident blocks per SM the UJ kernel is compiled for
#endif
#ifndef VPM_NF_LEAF
#define VPM_NF_LEAF 0                        // 1: near-field UJ and Estr per target leaf; 0: warp groups
#endif
#ifndef VPM_NF_DF
#define VPM_NF_DF 1                          // nf_uj_leaf: 1 = double-float displacement on every group
#endif
#ifndef VPM_NF_LANE
#define VPM_NF_LANE 0                        // 1: near-field FP32-comp UJ with a list walk per lane (nf_uj_lane)
#endif

__global__ void tgt_from_perm(int64_t n, const double* __restrict__ x, const int32_t* __restrict__ perm,
                              TgtPos* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t j = perm[i];
    TgtPos t;
    t.x = x[3 * j]; t.y = x[3 * j + 1]; t.z = x[3 * j + 2];
    t.idx = (int32_t)j; t.pad = 0;
    out[i] = t;
}

template <int K>
__global__ void leaf_pack_mixed(int64_t n, const double* __restrict__ x, const double* __restrict__ gs,
                                const double* __restrict__ sgs, const int32_t* __restrict__ perm,
                                SrcMixed* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t i = perm[o];
    const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
    const float xh = (float)px, yh = (float)py, zh = (float)pz;
    const double sig = (K == K_SING) ? 1.0 : sgs[i];
    const double k = singular_tail<K>() ? -C4 : -C4 / (sig * sig * sig);
    SrcMixed p;
    p.a = make_float4(xh, yh, zh, (float)(sig * sig));
    p.b = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), (float)(1.0 / sig));
    p.gam = make_float4((float)(k * gs[3 * i]), (float)(k * gs[3 * i + 1]), (float)(k * gs[3 * i + 2]), 0.f);
    out[o] = p;
}

// As leaf_pack_mixed, with gam = -Gamma/(4 pi sigma^3) for every kernel (nf_uj_leaf).
template <int K>
__global__ void leaf_pack_scaled(int64_t n, const double* __restrict__ x, const double* __restrict__ gs,
                                 const double* __restrict__ sgs, const int32_t* __restrict__ perm,
                                 SrcMixed* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t i = perm[o];
    const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
    const float xh = (float)px, yh = (float)py, zh = (float)pz;
    const double sig = (K == K_SING) ? 1.0 : sgs[i];
    const double k = -C4 / (sig * sig * sig);
    SrcMixed p;
    p.a = make_float4(xh, yh, zh, (float)(sig * sig));
    p.b = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), (float)(1.0 / sig));
    p.gam = make_float4((float)(k * gs[3 * i]), (float)(k * gs[3 * i + 1]), (float)(k * gs[3 * i + 2]), 0.f);
    out[o] = p;
}

template <int K>
__global__ void leaf_pack_f64(int64_t n, const double* __restrict__ x, const double* __restrict__ gs,
                              const double* __restrict__ sgs, const int32_t* __restrict__ perm,
                              SrcF64* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t i = perm[o];
    const double sig = (K == K_SING) ? 1.0 : sgs[i];
    SrcF64 p;
    p.xy = make_double2(x[3 * i], x[3 * i + 1]);
    p.z_isig = make_double2(x[3 * i + 2], 1.0 / sig);
    p.gxy = make_double2(gs[3 * i], gs[3 * i + 1]);
    // .y: for Gaussian-erf the r^2 past which g = 1, g' = 0 (pair_f64_acc), else sigma
    p.gz_sig = make_double2(gs[3 * i + 2], K == K_GAUSERF ? 81.0 * sig * sig : sig);
    out[o] = p;
}

// Estr source payloads in Morton order (v = J^T Gamma or J Gamma, zero for static sources;
// Js = NULL: v = 0, the zeta sum's payload).
template <int K>
__global__ void leaf_pack_estr(int64_t n, const double* __restrict__ x, const double* __restrict__ gs,
                               const double* __restrict__ sgs, const double* __restrict__ Js,
                               const uint8_t* __restrict__ static_s, bool transposed,
                               const int32_t* __restrict__ perm, int precision, void* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t i = perm[o];
    const bool off = static_s && static_s[i];
    const double gx = gs[3 * i], gy = gs[3 * i + 1], gz = gs[3 * i + 2];
    double vx = 0.0, vy = 0.0, vz = 0.0;
    if (Js) {
        const double* J = Js + 9 * i;
        if (transposed) {
            vx = J[0] * gx + J[1] * gy + J[2] * gz; vy = J[3] * gx + J[4] * gy + J[5] * gz; vz = J[6] * gx + J[7] * gy + J[8] * gz;
        } else {
            vx = J[0] * gx + J[3] * gy + J[6] * gz; vy = J[1] * gx + J[4] * gy + J[7] * gz; vz = J[2] * gx + J[5] * gy + J[8] * gz;
        }
    }
    const double isig = 1.0 / sgs[i];
    if (precision) {   // the position as a double-float, so that the kernel's staging is plain loads
        const double k = off ? 0.0 : zeta_norm(K) * isig * isig * isig;
        const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
        const float xh = (float)px, yh = (float)py, zh = (float)pz;
        SrcEstrDF p;
        p.a = make_float4(xh, yh, zh, (float)(isig * isig));
        p.b = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), 0.f);
        p.g = make_float4((float)(k * gx), (float)(k * gy), (float)(k * gz), 0.f);
        p.v = make_float4((float)(k * vx), (float)(k * vy), (float)(k * vz), 0.f);
        ((SrcEstrDF*)out)[o] = p;
    } else {
        const double m = off ? 0.0 : 1.0;
        SrcEstrF64 p;
        p.xy = make_double2(x[3 * i], x[3 * i + 1]);
        p.z_isig = make_double2(x[3 * i + 2], isig);
        p.gxy = make_double2(m * gx, m * gy);
        p.gz_vx = make_double2(m * gz, m * vx);
        p.vyz = make_double2(m * vy, m * vz);
        ((SrcEstrF64*)out)[o] = p;
    }
}

// Warp-group geometry shared by the kernels: this lane's target (FP64
// position, caller index) and its bit in the interval masks (its leaf relative
// to the group's first leaf; 0 for the padding lanes of the last group).
struct GroupTarget {
    double tx, ty, tz;
    int32_t idx;
    unsigned bit;
    bool valid;
};

__device__ __forceinline__ GroupTarget group_target(int64_t n, int64_t p0, int lane, const TgtPos* __restrict__ tgt,
                                                    const int32_t* __restrict__ leaf_of)
{
    GroupTarget g;
    const int64_t t = p0 + lane;
    g.valid = t < n;
    const TgtPos p = tgt[g.valid ? t : p0];
    g.tx = p.x; g.ty = p.y; g.tz = p.z; g.idx = p.idx;
    g.bit = g.valid ? 1u << (leaf_of[t] - leaf_of[p0]) : 0u;
    return g;
}

// Walks a group's intervals 32 sources at a time, across interval boundaries,
// so that tiles are full.  Lane i keeps interval wbase + i of a 32-interval
// window in registers; the walk itself is warp-uniform.
struct IntervalWalk {
    const int4* ivs;
    int e, e1, off, wbase;
    int4 win;

    __device__ __forceinline__ void init(const int4* v, int e0, int e_end, int lane)
    {
        ivs = v; e = e0; e1 = e_end; off = 0; wbase = e0;
        win = (e0 + lane < e_end) ? ivs[e0 + lane] : make_int4(0, 0, 0, 0);
    }
    // Next tile: this lane's source position (-1 for none) and target mask; returns the tile's size.
    __device__ __forceinline__ int next(int lane, int& my_p, unsigned& my_mask)
    {
        int filled = 0;
        my_p = -1;
        my_mask = 0u;
        while (filled < 32 && e < e1) {
            if (e - wbase >= 32) {
                wbase = e;
                win = (wbase + lane < e1) ? ivs[wbase + lane] : make_int4(0, 0, 0, 0);
            }
            const int k = e - wbase;
            const int p0 = __shfl_sync(0xffffffffu, win.x, k);
            const int p1 = __shfl_sync(0xffffffffu, win.y, k);
            const unsigned m = (unsigned)__shfl_sync(0xffffffffu, win.z, k);
            const int take = min(p1 - p0 - off, 32 - filled);
            if (lane >= filled && lane < filled + take) {
                my_p = p0 + off + (lane - filled);
                my_mask = m;
            }
            filled += take;
            off += take;
            if (off == p1 - p0) { e++; off = 0; }
        }
        return filled;
    }
};

// ------------------------------------------------------------- UJ, FP32-comp
// Sources from leaf_pack_lane: 1/sigma^2 in a.w and the near form's 1/sigma^3 in gam, so
// that a pair takes neither (pair4_mixed with SCALED).
template <int K>
__global__ void __launch_bounds__(NF_THREADS, VPM_NF_MIN_BLOCKS)
nf_uj_mixed(int64_t n, int64_t ngroups, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ leaf_of,
            const int32_t* __restrict__ grp_row, const int4* __restrict__ ivs, const SrcMixed* __restrict__ src,
            double* U, double* J)
{
    __shared__ SrcMixed tile[NF_WARPS][32];
    __shared__ float4 off[NF_WARPS][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t grp = (int64_t)blockIdx.x * NF_WARPS + warp;
    if (grp >= ngroups) return;
    const int64_t p0 = 32 * grp;
    const GroupTarget me = group_target(n, p0, lane, tgt, leaf_of);
    const TgtPos o = tgt[p0];
    const float3 th = make_float3((float)me.tx, (float)me.ty, (float)me.tz);
    const float3 tl = make_float3((float)(me.tx - (double)th.x), (float)(me.ty - (double)th.y),
                                  (float)(me.tz - (double)th.z));
    const float3 oh = make_float3((float)o.x, (float)o.y, (float)o.z);
    const float3 ol = make_float3((float)(o.x - (double)oh.x), (float)(o.y - (double)oh.y), (float)(o.z - (double)oh.z));
    const float3 to = make_float3((float)(me.tx - o.x), (float)(me.ty - o.y), (float)(me.tz - o.z));
    float b2 = fmaf(to.x, to.x, fmaf(to.y, to.y, to.z * to.z));
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, m));
    const float r2n = fmaxf(4.0f * b2, 1.0e-30f);

    // FP64 sums of this lane in shared memory ([0..2] U, [3..5] W, [6..13] J'), touched once per
    // NF_MID_BLKS blocks: the registers go to occupancy instead
    __shared__ double acc64[14][NF_THREADS];
#pragma unroll
    for (int k = 0; k < 14; k++) acc64[k][threadIdx.x] = 0.0;
    float mu[3] = {0.f, 0.f, 0.f}, mw[3] = {0.f, 0.f, 0.f}, mj[8];
    float u[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f}, jq[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { mj[k] = 0.f; jq[k] = 0.f; }
    int tiles = 0, blks = 0;
    IntervalWalk walk;
    walk.init(ivs, grp_row[grp], grp_row[grp + 1], lane);
    for (;;) {
        int sp;
        unsigned smask;
        const int cnt = walk.next(lane, sp, smask);
        if (cnt == 0) break;
        SrcMixed sj;
        if (sp >= 0) {
            sj = src[sp];
        } else {   // padding: far away, no strength, no target
            sj.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
            sj.b = make_float4(0.f, 0.f, 0.f, 1.f);
            sj.gam = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        sj.gam.w = __uint_as_float(smask);
        __syncwarp();
        tile[warp][lane] = sj;
        off[warp][lane] = make_float4((sj.a.x - oh.x) + (sj.b.x - ol.x), (sj.a.y - oh.y) + (sj.b.y - ol.y),
                                      (sj.a.z - oh.z) + (sj.b.z - ol.z), sj.a.w);
        __syncwarp();
        const int ng = (cnt + 3) >> 2;
        for (int q = 0; q < ng; q++)
            pair4_mixed<K, true, false, true>(to, th, tl, r2n, off[warp], tile[warp], 4 * q, u, jq, w, me.bit);
        if (++tiles == NF_BLK_TILES) {
            tiles = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) { mu[k] += u[k]; mw[k] += w[k]; u[k] = 0.f; w[k] = 0.f; }
#pragma unroll
            for (int k = 0; k < 8; k++) { mj[k] += jq[k]; jq[k] = 0.f; }
            if (++blks == NF_MID_BLKS) {
                blks = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    acc64[k][threadIdx.x] += (double)mu[k];
                    acc64[3 + k][threadIdx.x] += (double)mw[k];
                    mu[k] = 0.f; mw[k] = 0.f;
                }
#pragma unroll
                for (int k = 0; k < 8; k++) { acc64[6 + k][threadIdx.x] += (double)mj[k]; mj[k] = 0.f; }
            }
        }
    }
    double dU[3], dW[3], dJ[8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        dU[k] = acc64[k][threadIdx.x] + ((double)mu[k] + (double)u[k]);
        dW[k] = acc64[3 + k][threadIdx.x] + ((double)mw[k] + (double)w[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) dJ[k] = acc64[6 + k][threadIdx.x] + ((double)mj[k] + (double)jq[k]);
    if (!me.valid) return;
    double j9[9];
#pragma unroll
    for (int k = 0; k < 8; k++) j9[k] = -3.0 * dJ[k];
    j9[8] = 3.0 * (dJ[0] + dJ[4]);
    j9[1] -= dW[2]; j9[2] += dW[1]; j9[3] += dW[2]; j9[5] -= dW[0]; j9[6] -= dW[1]; j9[7] += dW[0];
#pragma unroll
    for (int k = 0; k < 3; k++) U[3 * (int64_t)me.idx + k] += dU[k];
#pragma unroll
    for (int k = 0; k < 9; k++) J[9 * (int64_t)me.idx + k] += j9[k];
}

// --------------------------------------------- UJ, FP32-comp, a walk per lane
// Sources of nf_uj_lane: the double-float position with 1/sigma^2 in a.w, and
// gam = -Gamma/(4 pi sigma^3) for every kernel (the near form's sigma^-3 taken once).
template <int K>
__global__ void leaf_pack_lane(int64_t n, const double* __restrict__ x, const double* __restrict__ gs,
                               const double* __restrict__ sgs, const int32_t* __restrict__ perm,
                               SrcMixed* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t i = perm[o];
    const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
    const float xh = (float)px, yh = (float)py, zh = (float)pz;
    const double sig = (K == K_SING) ? 1.0 : sgs[i];
    const double k = -C4 / (sig * sig * sig);
    SrcMixed p;
    p.a = make_float4(xh, yh, zh, (float)(1.0 / (sig * sig)));
    p.b = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), 0.f);
    p.gam = make_float4((float)(k * gs[3 * i]), (float)(k * gs[3 * i + 1]), (float)(k * gs[3 * i + 2]), 0.f);
    out[o] = p;
}

// Each lane walks the source list of its own target's leaf, straight from the CSR rows
// (col[row[L] .. row[L+1]) source leaves, each the particle range [lb, le) of the pack),
// four sources at a time, so that every pair a lane computes is one of its leaf's pairs:
// no lane computes a pair of another leaf with zero weight, as the warp-group kernel's do
// (a third of them on the jet cloud).  A warp runs until its longest list ends.  Lanes
// read their sources themselves (read-only loads; the lanes of one leaf read the same
// address together).  Pair math as the warp-group kernel's (double-float displacement,
// the form of four pairs chosen warp-wide); FP32 sums over 64 sources, then FP32 mid-level
// sums, then FP64 in shared memory.
template <int K>
__global__ void __launch_bounds__(NF_THREADS, VPM_NF_MIN_BLOCKS)
nf_uj_lane(int64_t n, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ leaf_of,
           const int32_t* __restrict__ lb, const int32_t* __restrict__ le, const int32_t* __restrict__ row,
           const int32_t* __restrict__ col, const SrcMixed* __restrict__ src, double* U, double* J)
{
    const int64_t t = (int64_t)blockIdx.x * NF_THREADS + threadIdx.x;
    const bool valid = t < n;
    const TgtPos me = tgt[valid ? t : n - 1];
    const float3 th = make_float3((float)me.x, (float)me.y, (float)me.z);
    const float3 tl = make_float3((float)(me.x - (double)th.x), (float)(me.y - (double)th.y),
                                  (float)(me.z - (double)th.z));
    // the walk: the current range [pc, pe), the next range [nb, ne) loaded ahead, col entry e of [.., e1)
    int e = 0, e1 = 0, pc = 0, pe = 0, nb = 0, ne = 0;
    if (valid) {
        const int L = leaf_of[t];
        e = row[L];
        e1 = row[L + 1];
        if (e < e1) { const int S = col[e]; nb = lb[S]; ne = le[S]; }
    }
    __shared__ double acc64[14][NF_THREADS];
#pragma unroll
    for (int k = 0; k < 14; k++) acc64[k][threadIdx.x] = 0.0;
    float mu[3] = {0.f, 0.f, 0.f}, mw[3] = {0.f, 0.f, 0.f}, mj[8];
    float u[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f}, jq[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { mj[k] = 0.f; jq[k] = 0.f; }
    int its = 0, blks = 0;
    for (;;) {
        int sp[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (pc == pe && e < e1) {   // the next range of the list (leaves are never empty)
                pc = nb; pe = ne; ++e;
                if (e < e1) { const int S = col[e]; nb = lb[S]; ne = le[S]; }
            }
            const bool has = pc < pe;
            sp[q] = has ? pc : -1;
            pc += has ? 1 : 0;
        }
        if (!__any_sync(0xffffffffu, sp[0] >= 0)) break;   // every lane's list has ended
        float ex[4], ey[4], ez[4], s4[4], i2[4], G[4], Q[4];
        bool on[4];
        float4 gq[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float4 a = make_float4(th.x, th.y, th.z, 1.f), b = make_float4(tl.x, tl.y, tl.z, 0.f);
            gq[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (sp[q] >= 0) {
                a = __ldg(&src[sp[q]].a);
                b = __ldg(&src[sp[q]].b);
                gq[q] = __ldg(&src[sp[q]].gam);
            }
            ex[q] = (th.x - a.x) + (tl.x - b.x);
            ey[q] = (th.y - a.y) + (tl.y - b.y);
            ez[q] = (th.z - a.z) + (tl.z - b.z);
            const float e2 = fmaf(ex[q], ex[q], fmaf(ey[q], ey[q], ez[q] * ez[q]));
            on[q] = e2 > 0.0f;   // no source, the self pair and coincident particles: nothing
            i2[q] = a.w;
            s4[q] = on[q] ? e2 * a.w : 1.0f;
        }
        near_GQ4<K, false>(s4, i2, G, Q);
#pragma unroll
        for (int q = 0; q < 4; q++)
            accum_pair(ex[q], ey[q], ez[q], on[q] ? G[q] : 0.0f, on[q] ? Q[q] : 0.0f, gq[q], u, jq, w);
        if (++its == 16) {   // 64 sources a lane
            its = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) { mu[k] += u[k]; mw[k] += w[k]; u[k] = 0.f; w[k] = 0.f; }
#pragma unroll
            for (int k = 0; k < 8; k++) { mj[k] += jq[k]; jq[k] = 0.f; }
            if (++blks == NF_MID_BLKS) {
                blks = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    acc64[k][threadIdx.x] += (double)mu[k];
                    acc64[3 + k][threadIdx.x] += (double)mw[k];
                    mu[k] = 0.f; mw[k] = 0.f;
                }
#pragma unroll
                for (int k = 0; k < 8; k++) { acc64[6 + k][threadIdx.x] += (double)mj[k]; mj[k] = 0.f; }
            }
        }
    }
    if (!valid) return;
    double dU[3], dW[3], dJ[8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        dU[k] = acc64[k][threadIdx.x] + ((double)mu[k] + (double)u[k]);
        dW[k] = acc64[3 + k][threadIdx.x] + ((double)mw[k] + (double)w[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) dJ[k] = acc64[6 + k][threadIdx.x] + ((double)mj[k] + (double)jq[k]);
    double j9[9];
#pragma unroll
    for (int k = 0; k < 8; k++) j9[k] = -3.0 * dJ[k];
    j9[8] = 3.0 * (dJ[0] + dJ[4]);
    j9[1] -= dW[2]; j9[2] += dW[1]; j9[3] += dW[2]; j9[5] -= dW[0]; j9[6] -= dW[1]; j9[7] += dW[0];
#pragma unroll
    for (int k = 0; k < 3; k++) U[3 * (int64_t)me.idx + k] += dU[k];
#pragma unroll
    for (int k = 0; k < 9; k++) J[9 * (int64_t)me.idx + k] += j9[k];
}

// ------------------------------------------------- UJ, FP32-comp, per leaf
// One warp per target leaf, taken in chunks of at most 32 targets.  A chunk of
// a targets runs in Ks = min(8, 32/a) stripes: lane (i, k) = (lane % a,
// lane / a) holds target i and evaluates stripe k's share of every tile of
// sources, so a chunk uses a Ks of the 32 lanes and all of them need every
// source (no target masks: the leaf's own source list is walked, straight from
// its CSR row).  A tile holds T = 4 Ks g <= 32 sources, stripe k taking the
// g groups of four at [k T/Ks, (k + 1) T/Ks).  At the end of a chunk the
// stripes' FP64 sums are added in stripe order.
//
// Displacements: FP32 offsets from the chunk's first target (the warp origin),
// dx = t_off - s_off, whose error is at most ~1.5 ulp of |dx| when
// |dx| > 2b (b: the chunk's extent around the origin).  A group of four in
// which any lane has a pair closer than 2b takes the double-float difference
// (x_t,hi - x_s,hi) + (x_t,lo - x_s,lo) instead (one vote).  Target and source
// offsets are formed by the same FP32 double-float operations, so the self
// pair has r^2 == 0 exactly on either path.  Sources carry
// gam = -Gamma/(4 pi sigma^3), so the pair form needs no sigma^3 factor.

// Source ranges of one target leaf, walked T at a time across leaf boundaries.
// Lane i keeps source leaf wbase + i of a 32-leaf window of the CSR row.
struct LeafWalk {
    const int32_t* col;
    const int32_t* lb;
    const int32_t* le;
    int e, e1, off, wbase;
    int2 win;

    __device__ __forceinline__ void load(int lane)
    {
        win = make_int2(0, 0);
        if (wbase + lane < e1) {
            const int c = col[wbase + lane];
            win = make_int2(lb[c], le[c]);
        }
    }
    __device__ __forceinline__ void init(const int32_t* c, const int32_t* b, const int32_t* en, int e0, int e_end,
                                         int lane)
    {
        col = c; lb = b; le = en; e = e0; e1 = e_end; off = 0; wbase = e0;
        load(lane);
    }
    // Next tile of at most T sources: this lane's source position (-1 for none) if lane < T;
    // returns the tile's size.
    __device__ __forceinline__ int next(int lane, int T, int& my_p)
    {
        int filled = 0;
        my_p = -1;
        while (filled < T && e < e1) {
            if (e - wbase >= 32) {
                wbase = e;
                load(lane);
            }
            const int k = e - wbase;
            const int p0 = __shfl_sync(0xffffffffu, win.x, k);
            const int p1 = __shfl_sync(0xffffffffu, win.y, k);
            const int take = min(p1 - p0 - off, T - filled);
            if (lane >= filled && lane < filled + take) my_p = p0 + off + (lane - filled);
            filled += take;
            off += take;
            if (off == p1 - p0) { e++; off = 0; }
        }
        return filled;
    }
};

// Four sources j0..j0+3 of the tile against this lane's target (see above); idle lanes
// take part in the votes only.
template <int K>
__device__ __forceinline__ void pair4_leaf(const float3& to, const float3& th, const float3& tl, float r2n,
                                           const float4* __restrict__ off, const SrcMixed* __restrict__ tile, int j0,
                                           bool idle, float (&u)[3], float (&jq)[8], float (&w)[3])
{
    float dx[4], dy[4], dz[4], r2[4], i2[4];
    bool far = !VPM_NF_DF;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float4 h = off[j0 + q];
        i2[q] = h.w;
        if (!VPM_NF_DF) {
            dx[q] = to.x - h.x;
            dy[q] = to.y - h.y;
            dz[q] = to.z - h.z;
            r2[q] = fmaf(dx[q], dx[q], fmaf(dy[q], dy[q], dz[q] * dz[q]));
            far = far && r2[q] > r2n;
        }
    }
    if (VPM_NF_DF || !__all_sync(0xffffffffu, far || idle)) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float4 a = tile[j0 + q].a, b = tile[j0 + q].b;
            dx[q] = (th.x - a.x) + (tl.x - b.x);
            dy[q] = (th.y - a.y) + (tl.y - b.y);
            dz[q] = (th.z - a.z) + (tl.z - b.z);
            r2[q] = fmaf(dx[q], dx[q], fmaf(dy[q], dy[q], dz[q] * dz[q]));
        }
    }
    float s4[4], G[4], Q[4];
#pragma unroll
    for (int q = 0; q < 4; q++) s4[q] = idle ? 1.0e4f : r2[q] * i2[q];
    near_GQ4<K, true>(s4, i2, G, Q);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const bool on = !idle && r2[q] > 0.0f;
        accum_pair(dx[q], dy[q], dz[q], on ? G[q] : 0.0f, on ? Q[q] : 0.0f, tile[j0 + q].gam, u, jq, w);
    }
}

template <int K>
__global__ void __launch_bounds__(NF_THREADS, VPM_NF_MIN_BLOCKS)
nf_uj_leaf(int64_t nleaves, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ lb,
           const int32_t* __restrict__ le, const int32_t* __restrict__ row, const int32_t* __restrict__ col,
           const SrcMixed* __restrict__ src, double* U, double* J)
{
    constexpr int NF_BLK_PAIRS = 64;    // pairs per lane summed in FP32 before the mid-level sum
    constexpr int NF_MID_PAIRS = 256;   // pairs per lane summed in the mid-level FP32 sum before FP64
    __shared__ SrcMixed tile[NF_WARPS][32];
    __shared__ float4 off[NF_WARPS][32];
    __shared__ double acc64[14][NF_THREADS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t leaf = (int64_t)blockIdx.x * NF_WARPS + warp;
    if (leaf >= nleaves) return;
    const int p_begin = lb[leaf], p_end = le[leaf];
    for (int c0 = p_begin; c0 < p_end; c0 += 32) {
        const int na = min(32, p_end - c0);
        const int ks = min(8, 32 / na);
        const int T = 4 * ks * max(1, 32 / (4 * ks));
        const int m = T / ks;                               // sources per stripe and tile
        const int ti = lane % na, stripe = lane / na;
        const bool idle = stripe >= ks;
        const TgtPos me = tgt[c0 + ti];
        const TgtPos o = tgt[c0];
        const float3 th = make_float3((float)me.x, (float)me.y, (float)me.z);
        const float3 tl = make_float3((float)(me.x - (double)th.x), (float)(me.y - (double)th.y),
                                      (float)(me.z - (double)th.z));
        const float3 oh = make_float3((float)o.x, (float)o.y, (float)o.z);
        const float3 ol = make_float3((float)(o.x - (double)oh.x), (float)(o.y - (double)oh.y),
                                      (float)(o.z - (double)oh.z));
        // the same FP32 double-float operations as the sources' offsets: the self pair has r^2 == 0
        const float3 to = make_float3(df_offset(th.x, tl.x, oh.x, ol.x), df_offset(th.y, tl.y, oh.y, ol.y),
                                      df_offset(th.z, tl.z, oh.z, ol.z));
        float b2 = fmaf(to.x, to.x, fmaf(to.y, to.y, to.z * to.z));
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, sh));
        const float r2n = fmaxf(4.0f * b2, 1.0e-30f);
#pragma unroll
        for (int k = 0; k < 14; k++) acc64[k][threadIdx.x] = 0.0;
        float mu[3] = {0.f, 0.f, 0.f}, mw[3] = {0.f, 0.f, 0.f}, mj[8];
        float u[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f}, jq[8];
#pragma unroll
        for (int k = 0; k < 8; k++) { mj[k] = 0.f; jq[k] = 0.f; }
        int blk = 0, mid = 0;
        LeafWalk walk;
        walk.init(col, lb, le, row[leaf], row[leaf + 1], lane);
        for (;;) {
            int sp;
            const int cnt = walk.next(lane, T, sp);
            if (cnt == 0) break;
            __syncwarp();
            if (lane < T) {
                SrcMixed sj;
                if (sp >= 0) {
                    sj = src[sp];
                } else {   // padding: far away, no strength
                    sj.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
                    sj.b = make_float4(0.f, 0.f, 0.f, 1.f);
                    sj.gam = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                tile[warp][lane] = sj;
                off[warp][lane] = make_float4(df_offset(sj.a.x, sj.b.x, oh.x, ol.x),
                                              df_offset(sj.a.y, sj.b.y, oh.y, ol.y),
                                              df_offset(sj.a.z, sj.b.z, oh.z, ol.z), sj.b.w * sj.b.w);
            }
            __syncwarp();
            // stripe k's groups; every lane runs the same trip count (warp-wide votes)
            const int j1 = (idle ? 0 : stripe) * m;
            for (int q = 0; q < m; q += 4)
                pair4_leaf<K>(to, th, tl, r2n, off[warp], tile[warp], j1 + q, idle, u, jq, w);
            blk += m;
            if (blk >= NF_BLK_PAIRS) {
                blk = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) { mu[k] += u[k]; mw[k] += w[k]; u[k] = 0.f; w[k] = 0.f; }
#pragma unroll
                for (int k = 0; k < 8; k++) { mj[k] += jq[k]; jq[k] = 0.f; }
                mid += NF_BLK_PAIRS;
                if (mid >= NF_MID_PAIRS) {
                    mid = 0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        acc64[k][threadIdx.x] += (double)mu[k];
                        acc64[3 + k][threadIdx.x] += (double)mw[k];
                        mu[k] = 0.f; mw[k] = 0.f;
                    }
#pragma unroll
                    for (int k = 0; k < 8; k++) { acc64[6 + k][threadIdx.x] += (double)mj[k]; mj[k] = 0.f; }
                }
            }
        }
        // this lane's totals, then the stripes of each target added in order
#pragma unroll
        for (int k = 0; k < 3; k++) {
            acc64[k][threadIdx.x] += (double)mu[k] + (double)u[k];
            acc64[3 + k][threadIdx.x] += (double)mw[k] + (double)w[k];
        }
#pragma unroll
        for (int k = 0; k < 8; k++) acc64[6 + k][threadIdx.x] += (double)mj[k] + (double)jq[k];
        __syncwarp();
        if (lane < na) {
            double dU[3], dW[3], dJ[8];
            const int base = threadIdx.x - lane;
#pragma unroll
            for (int k = 0; k < 3; k++) { dU[k] = 0.0; dW[k] = 0.0; }
#pragma unroll
            for (int k = 0; k < 8; k++) dJ[k] = 0.0;
            for (int st = 0; st < ks; st++) {
                const int l2 = base + lane + st * na;
#pragma unroll
                for (int k = 0; k < 3; k++) { dU[k] += acc64[k][l2]; dW[k] += acc64[3 + k][l2]; }
#pragma unroll
                for (int k = 0; k < 8; k++) dJ[k] += acc64[6 + k][l2];
            }
            double j9[9];
#pragma unroll
            for (int k = 0; k < 8; k++) j9[k] = -3.0 * dJ[k];
            j9[8] = 3.0 * (dJ[0] + dJ[4]);
            j9[1] -= dW[2]; j9[2] += dW[1]; j9[3] += dW[2]; j9[5] -= dW[0]; j9[6] -= dW[1]; j9[7] += dW[0];
            const int64_t idx = me.idx;
#pragma unroll
            for (int k = 0; k < 3; k++) U[3 * idx + k] += dU[k];
#pragma unroll
            for (int k = 0; k < 9; k++) J[9 * idx + k] += j9[k];
        }
        __syncwarp();   // acc64 is reset by the next chunk
    }
}

// ----------------------------------------------- Estr, FP32-comp, per leaf
// The layout of nf_uj_leaf (one warp per target leaf, chunks of <= 32 targets
// in Ks stripes, the leaf's own CSR row walked T sources at a time) for the
// Estr sums Zg = sum z g, Zv = sum z v of the factored form (estr.cu).  Target
// and source offsets from the chunk's first target are formed by the same
// FP32 double-float operations, so coincident particles (the self pair
// included) have r^2 == 0 exactly and are skipped (ZETA: kept).  Per lane the
// pairs of a tile are summed in FP32 and added with compensation (comp_add)
// once at least 8 have gathered, and to FP64 every 256.
template <int K>
__global__ void leaf_pack_estr_df(int64_t n, const double* __restrict__ x, const double* __restrict__ gs,
                                  const double* __restrict__ sgs, const double* __restrict__ Js,
                                  const uint8_t* __restrict__ static_s, bool transposed,
                                  const int32_t* __restrict__ perm, SrcEstrDF* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t i = perm[o];
    const bool st = static_s && static_s[i];
    const double gx = gs[3 * i], gy = gs[3 * i + 1], gz = gs[3 * i + 2];
    double vx = 0.0, vy = 0.0, vz = 0.0;
    if (Js) {
        const double* J = Js + 9 * i;
        if (transposed) {
            vx = J[0] * gx + J[1] * gy + J[2] * gz; vy = J[3] * gx + J[4] * gy + J[5] * gz; vz = J[6] * gx + J[7] * gy + J[8] * gz;
        } else {
            vx = J[0] * gx + J[3] * gy + J[6] * gz; vy = J[1] * gx + J[4] * gy + J[7] * gz; vz = J[2] * gx + J[5] * gy + J[8] * gz;
        }
    }
    const double isig = 1.0 / sgs[i];
    const double k = st ? 0.0 : zeta_norm(K) * isig * isig * isig;
    const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
    const float xh = (float)px, yh = (float)py, zh = (float)pz;
    SrcEstrDF p;
    p.a = make_float4(xh, yh, zh, (float)(isig * isig));
    p.b = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), 0.f);
    p.g = make_float4((float)(k * gx), (float)(k * gy), (float)(k * gz), 0.f);
    p.v = make_float4((float)(k * vx), (float)(k * vy), (float)(k * vz), 0.f);
    out[o] = p;
}

template <int K, bool DZ = false, bool ZETA = false>
__global__ void __launch_bounds__(NF_THREADS)
nf_estr_leaf(int64_t nleaves, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ lb,
             const int32_t* __restrict__ le, const int32_t* __restrict__ row, const int32_t* __restrict__ col,
             const SrcEstrDF* __restrict__ src, const double* __restrict__ Jt, const uint8_t* __restrict__ static_t,
             bool transposed, double* SFS, float3 fd = make_float3(0.f, 0.f, 0.f))
{
    static_assert(!(DZ && ZETA), "one mode at a time");
    __shared__ SrcEstrDF tile[NF_WARPS][32];
    __shared__ float4 off[NF_WARPS][32];
    __shared__ double acc64[6][NF_THREADS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t leaf = (int64_t)blockIdx.x * NF_WARPS + warp;
    if (leaf >= nleaves) return;
    const int p_begin = lb[leaf], p_end = le[leaf];
    for (int c0 = p_begin; c0 < p_end; c0 += 32) {
        const int na = min(32, p_end - c0);
        const int ks = min(8, 32 / na);
        const int T = 4 * ks * max(1, 32 / (4 * ks));
        const int m = T / ks;
        const int ti = lane % na, stripe = lane / na;
        const bool idle = stripe >= ks;
        const TgtPos me = tgt[c0 + ti];
        const TgtPos o = tgt[c0];
        const float3 oh = make_float3((float)o.x, (float)o.y, (float)o.z);
        const float3 ol = make_float3((float)(o.x - (double)oh.x), (float)(o.y - (double)oh.y),
                                      (float)(o.z - (double)oh.z));
        float3 to;
        {
            const float3 th = make_float3((float)me.x, (float)me.y, (float)me.z);
            const float3 tl = make_float3((float)(me.x - (double)th.x), (float)(me.y - (double)th.y),
                                          (float)(me.z - (double)th.z));
            to = make_float3(df_offset(th.x, tl.x, oh.x, ol.x), df_offset(th.y, tl.y, oh.y, ol.y),
                             df_offset(th.z, tl.z, oh.z, ol.z));
        }
#pragma unroll
        for (int k = 0; k < 6; k++) acc64[k][threadIdx.x] = 0.0;
        float sg[3] = {0.f, 0.f, 0.f}, cg[3] = {0.f, 0.f, 0.f}, sv[3] = {0.f, 0.f, 0.f}, cv[3] = {0.f, 0.f, 0.f};
        float fg[3] = {0.f, 0.f, 0.f}, fv[3] = {0.f, 0.f, 0.f};
        int part = 0, flush = 0;
        LeafWalk walk;
        walk.init(col, lb, le, row[leaf], row[leaf + 1], lane);
        for (;;) {
            int sp;
            const int cnt = walk.next(lane, T, sp);
            if (cnt == 0) break;
            __syncwarp();
            if (lane < T) {
                SrcEstrDF sj;
                if (sp >= 0) {
                    sj = src[sp];
                } else {   // padding: far away, no payload
                    sj.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
                    sj.b = sj.g = sj.v = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                tile[warp][lane] = sj;
                off[warp][lane] = make_float4(df_offset(sj.a.x, sj.b.x, oh.x, ol.x),
                                              df_offset(sj.a.y, sj.b.y, oh.y, ol.y),
                                              df_offset(sj.a.z, sj.b.z, oh.z, ol.z), sj.a.w);
            }
            __syncwarp();
            if (!idle) {
                const int j1 = stripe * m;
                for (int q = 0; q < m; q++) {
                    const float4 h = off[warp][j1 + q];
                    const float dx = to.x - h.x, dy = to.y - h.y, dz = to.z - h.z;
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float s2 = r2 * h.w;
                    float z = zhat_f32<K>(s2);
                    if constexpr (DZ) z *= zeta_ratio_m1<K>(s2, fd);
                    if constexpr (!ZETA) z = r2 == 0.0f ? 0.0f : z;
                    const float4 g = tile[warp][j1 + q].g;
                    fg[0] = fmaf(z, g.x, fg[0]); fg[1] = fmaf(z, g.y, fg[1]); fg[2] = fmaf(z, g.z, fg[2]);
                    if constexpr (!ZETA) {
                        const float4 v = tile[warp][j1 + q].v;
                        fv[0] = fmaf(z, v.x, fv[0]); fv[1] = fmaf(z, v.y, fv[1]); fv[2] = fmaf(z, v.z, fv[2]);
                    }
                }
                part += m;
                if (part >= 8) {
                    part = 0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        comp_add(sg[k], cg[k], fg[k]); fg[k] = 0.f;
                        if constexpr (!ZETA) { comp_add(sv[k], cv[k], fv[k]); fv[k] = 0.f; }
                    }
                }
                flush += m;
                if (flush >= 256) {
                    flush = 0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        acc64[k][threadIdx.x] += (double)sg[k] + (double)cg[k];
                        acc64[3 + k][threadIdx.x] += (double)sv[k] + (double)cv[k];
                        sg[k] = cg[k] = sv[k] = cv[k] = 0.f;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            acc64[k][threadIdx.x] += ((double)sg[k] + (double)cg[k]) + (double)fg[k];
            acc64[3 + k][threadIdx.x] += ((double)sv[k] + (double)cv[k]) + (double)fv[k];
        }
        __syncwarp();
        if (lane < na) {
            const int64_t idx = me.idx;
            const bool live = ZETA || !(static_t && static_t[idx]);
            if (live) {
                double zg[3] = {0.0, 0.0, 0.0}, zv[3] = {0.0, 0.0, 0.0};
                const int base = threadIdx.x - lane;
                for (int st = 0; st < ks; st++) {
                    const int l2 = base + lane + st * na;
#pragma unroll
                    for (int k = 0; k < 3; k++) { zg[k] += acc64[k][l2]; zv[k] += acc64[3 + k][l2]; }
                }
                if constexpr (ZETA) {
#pragma unroll
                    for (int k = 0; k < 3; k++) SFS[3 * idx + k] += zg[k];
                } else {
                    const double* Jp = Jt + 9 * idx;
                    double o3[3];
                    if (transposed) {
                        o3[0] = Jp[0] * zg[0] + Jp[1] * zg[1] + Jp[2] * zg[2] - zv[0];
                        o3[1] = Jp[3] * zg[0] + Jp[4] * zg[1] + Jp[5] * zg[2] - zv[1];
                        o3[2] = Jp[6] * zg[0] + Jp[7] * zg[1] + Jp[8] * zg[2] - zv[2];
                    } else {
                        o3[0] = Jp[0] * zg[0] + Jp[3] * zg[1] + Jp[6] * zg[2] - zv[0];
                        o3[1] = Jp[1] * zg[0] + Jp[4] * zg[1] + Jp[7] * zg[2] - zv[1];
                        o3[2] = Jp[2] * zg[0] + Jp[5] * zg[1] + Jp[8] * zg[2] - zv[2];
                    }
#pragma unroll
                    for (int k = 0; k < 3; k++) SFS[3 * idx + k] += o3[k];
                }
            }
        }
        __syncwarp();   // acc64 is reset by the next chunk
    }
}

// ------------------------------------------- dynamic procedure, FP32-comp
// dJ_t += the test-filter difference of every near pair's J term,
// j(dx, Gamma_s, alpha sigma_s) - j(dx, Gamma_s, sigma_s), evaluated as a
// difference (dynamic.cu) over the group's intervals, four pairs at a time
// without branches (masked pairs and pairs at r = 0 add zero); M as in
// filter_diff.  No far vote: near-list pairs are almost all within reach.
template <int K, int M>
__global__ void __launch_bounds__(NF_THREADS)
nf_filter_diff(int64_t n, int64_t ngroups, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ leaf_of,
               const int32_t* __restrict__ grp_row, const int4* __restrict__ ivs, const SrcMixed* __restrict__ src,
               float hm, int panels, double* dJ)
{
    __shared__ SrcMixed tile[NF_WARPS][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t grp = (int64_t)blockIdx.x * NF_WARPS + warp;
    if (grp >= ngroups) return;
    const int64_t p0 = 32 * grp;
    const GroupTarget me = group_target(n, p0, lane, tgt, leaf_of);
    const float3 th = make_float3((float)me.tx, (float)me.ty, (float)me.tz);
    const float3 tl = make_float3((float)(me.tx - (double)th.x), (float)(me.ty - (double)th.y),
                                  (float)(me.tz - (double)th.z));
    double acc[9];
    float f[9];
#pragma unroll
    for (int k = 0; k < 9; k++) { acc[k] = 0.0; f[k] = 0.f; }
    int tiles = 0;
    IntervalWalk walk;
    walk.init(ivs, grp_row[grp], grp_row[grp + 1], lane);
    for (;;) {
        int sp;
        unsigned smask;
        const int cnt = walk.next(lane, sp, smask);
        if (cnt == 0) break;
        SrcMixed sj;
        if (sp >= 0) {
            sj = src[sp];
        } else {   // padding: far away, no strength, no target
            sj.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
            sj.b = make_float4(0.f, 0.f, 0.f, 1.f);
            sj.gam = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        sj.gam.w = __uint_as_float(smask);
        __syncwarp();
        tile[warp][lane] = sj;
        __syncwarp();
        for (int j0 = 0; j0 < cnt; j0 += 4) {   // cnt <= 32: j0 + 3 stays in the tile
            float ex[4], ey[4], ez[4], r2[4];
            bool on[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const SrcMixed& s = tile[warp][j0 + q];
                ex[q] = (th.x - s.a.x) + (tl.x - s.b.x);
                ey[q] = (th.y - s.a.y) + (tl.y - s.b.y);
                ez[q] = (th.z - s.a.z) + (tl.z - s.b.z);
                r2[q] = fmaf(ex[q], ex[q], fmaf(ey[q], ey[q], ez[q] * ez[q]));
                on[q] = (__float_as_uint(s.gam.w) & me.bit) != 0u && r2[q] > 0.0f;
                r2[q] = on[q] ? r2[q] : 1.0f;
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                filter_diff_pair<K, M>(ex[q], ey[q], ez[q], r2[q], tile[warp][j0 + q].b.w, tile[warp][j0 + q].gam, hm,
                                       panels, on[q], f);
        }
        if (++tiles == NF_BLK_TILES) {
            tiles = 0;
#pragma unroll
            for (int k = 0; k < 9; k++) { acc[k] += (double)f[k]; f[k] = 0.f; }
        }
    }
    if (!me.valid) return;
#pragma unroll
    for (int k = 0; k < 9; k++) dJ[9 * (int64_t)me.idx + k] += acc[k] + (double)f[k];
}

// --------------------------------------------------------------------- UJ, FP64
// pair_f64_acc (uj_pair.cuh) over the group's intervals, for the targets of each source's mask.
template <int K>
__global__ void __launch_bounds__(NF_THREADS)
nf_uj_f64(int64_t n, int64_t ngroups, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ leaf_of,
          const int32_t* __restrict__ grp_row, const int4* __restrict__ ivs, const SrcF64* __restrict__ src,
          double* U, double* J)
{
    __shared__ SrcF64 tile[NF_WARPS][32];
    __shared__ unsigned tmask[NF_WARPS][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t grp = (int64_t)blockIdx.x * NF_WARPS + warp;
    if (grp >= ngroups) return;
    const GroupTarget me = group_target(n, 32 * grp, lane, tgt, leaf_of);
    double u[3] = {0.0, 0.0, 0.0}, w[3] = {0.0, 0.0, 0.0}, jq[9];
#pragma unroll
    for (int k = 0; k < 9; k++) jq[k] = 0.0;
    IntervalWalk walk;
    walk.init(ivs, grp_row[grp], grp_row[grp + 1], lane);
    for (;;) {
        int sp;
        unsigned smask;
        const int cnt = walk.next(lane, sp, smask);
        if (cnt == 0) break;
        __syncwarp();
        if (sp >= 0) tile[warp][lane] = src[sp];
        tmask[warp][lane] = smask;
        __syncwarp();
        for (int j = 0; j < cnt; j++)
            if (tmask[warp][j] & me.bit) pair_f64_acc<K>(me.tx, me.ty, me.tz, tile[warp][j], u, w, jq);
    }
    if (!me.valid) return;
    double acc[12];
    uj_f64_finish(u, w, jq, acc);
#pragma unroll
    for (int k = 0; k < 3; k++) U[3 * (int64_t)me.idx + k] += acc[k];
#pragma unroll
    for (int k = 0; k < 9; k++) J[9 * (int64_t)me.idx + k] += acc[3 + k];
}

// ------------------------------------------------------------------------- Estr
// SFS_t += J_t^T sum_s z_s g_s - sum_s z_s v_s  (z = zeta(r/sigma_s), g and v
// pre-scaled by ZNORM / sigma_s^3 in the pack), over the group's intervals,
// skipping the self pair (mixed: every pair at r = 0, as in estr.cu), for
// non-static targets.  With DZ (mixed only) each weight is the dynamic
// procedure's weight difference zeta~(r, alpha sigma_s) - zeta~(r, sigma_s),
// fd as in estr.cu.  With ZETA the kernel is zeta_fmm's near-field sum
// (src/FLOWVPM_viscous.jl:523-556): SFS_t += sum_s z_s g_s over every target,
// the self pair and static particles included (payload packed with Js = NULL).
template <int K, bool MIXED, bool DZ = false, bool ZETA = false>
__global__ void __launch_bounds__(NF_THREADS)
nf_estr(int64_t n, int64_t ngroups, const TgtPos* __restrict__ tgt, const int32_t* __restrict__ leaf_of,
        const int32_t* __restrict__ grp_row, const int4* __restrict__ ivs, const void* __restrict__ srcv,
        const double* __restrict__ Jt, const uint8_t* __restrict__ static_t, bool transposed, double* SFS,
        float3 fd = make_float3(0.f, 0.f, 0.f))
{
    static_assert(MIXED || !DZ, "weight differences are FP32-comp only");
    static_assert(!(DZ && ZETA), "one mode at a time");
    // mixed: per source (x_hi, 1/sigma^2), (x_lo), g, v;  FP64: the packed source
    __shared__ __align__(16) float4 mtile[MIXED ? NF_WARPS : 1][4][32];
    __shared__ SrcEstrF64 dtile[MIXED ? 1 : NF_WARPS][32];
    __shared__ int spos[NF_WARPS][32];                          // source position, -1 for padding
    __shared__ unsigned tmask[NF_WARPS][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t grp = (int64_t)blockIdx.x * NF_WARPS + warp;
    if (grp >= ngroups) return;
    const int64_t p0 = 32 * grp;
    const GroupTarget me = group_target(n, p0, lane, tgt, leaf_of);
    const bool live = me.valid && (ZETA || !(static_t && static_t[me.idx]));
    const unsigned bit = live ? me.bit : 0u;
    const int tpos = (int)(p0 + lane);
    const float3 th = make_float3((float)me.tx, (float)me.ty, (float)me.tz);
    const float3 tl = make_float3((float)(me.tx - (double)th.x), (float)(me.ty - (double)th.y),
                                  (float)(me.tz - (double)th.z));
    double zg[3] = {0.0, 0.0, 0.0}, zv[3] = {0.0, 0.0, 0.0};
    // mixed: compensated FP32 sums of 8-source partial sums (comp_add), FP64 every NF_ESTR_FLUSH tiles
    // (as the all-pairs mixed Estr; the FP64 pipe runs at 1/64 of the FP32 rate)
    float sg[3] = {0.f, 0.f, 0.f}, cg[3] = {0.f, 0.f, 0.f}, sv[3] = {0.f, 0.f, 0.f}, cv[3] = {0.f, 0.f, 0.f};
    int tiles = 0;
    IntervalWalk walk;
    walk.init(ivs, grp_row[grp], grp_row[grp + 1], lane);
    for (;;) {
        int sp;
        unsigned smask;
        const int cnt = walk.next(lane, sp, smask);
        if (cnt == 0) break;
        __syncwarp();
        if constexpr (MIXED) {
            if (sp >= 0) {
                const SrcEstrDF p = ((const SrcEstrDF*)srcv)[sp];
                mtile[warp][0][lane] = p.a;
                mtile[warp][1][lane] = p.b;
                mtile[warp][2][lane] = p.g;
                mtile[warp][3][lane] = p.v;
            } else {   // padding: far away, no payload (read by the unrolled sub-blocks with mask 0)
                mtile[warp][0][lane] = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
                mtile[warp][1][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
                mtile[warp][2][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
                mtile[warp][3][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        } else {
            if (sp >= 0) dtile[warp][lane] = ((const SrcEstrF64*)srcv)[sp];
        }
        spos[warp][lane] = sp;
        tmask[warp][lane] = smask;
        __syncwarp();
        if constexpr (MIXED) {
            for (int j0 = 0; j0 < cnt; j0 += 8) {   // cnt <= 32: j0 + 7 stays in the tile (padding has mask 0)
                float fg[3] = {0.f, 0.f, 0.f}, fv[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int j = j0; j < j0 + 8; j++) {
                    const float4 h = mtile[warp][0][j], l = mtile[warp][1][j];
                    const float dx = (th.x - h.x) + (tl.x - l.x);
                    const float dy = (th.y - h.y) + (tl.y - l.y);
                    const float dz = (th.z - h.z) + (tl.z - l.z);
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    float z = zhat_f32<K>(r2 * h.w);
                    if constexpr (DZ) z *= zeta_ratio_m1<K>(r2 * h.w, fd);
                    // pairs at r = 0 are skipped (ZETA: kept, the self pair included)
                    const bool on = (tmask[warp][j] & bit) != 0u && (ZETA || r2 != 0.0f);
                    z = on ? z : 0.0f;
                    const float4 g = mtile[warp][2][j];
                    fg[0] = fmaf(z, g.x, fg[0]); fg[1] = fmaf(z, g.y, fg[1]); fg[2] = fmaf(z, g.z, fg[2]);
                    if constexpr (!ZETA) {
                        const float4 v = mtile[warp][3][j];
                        fv[0] = fmaf(z, v.x, fv[0]); fv[1] = fmaf(z, v.y, fv[1]); fv[2] = fmaf(z, v.z, fv[2]);
                    }
                }
#pragma unroll
                for (int k = 0; k < 3; k++) { comp_add(sg[k], cg[k], fg[k]); comp_add(sv[k], cv[k], fv[k]); }
            }
            if (++tiles == NF_ESTR_FLUSH) {
                tiles = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    zg[k] += (double)sg[k] + (double)cg[k];
                    zv[k] += (double)sv[k] + (double)cv[k];
                    sg[k] = cg[k] = sv[k] = cv[k] = 0.f;
                }
            }
        } else {
            for (int j = 0; j < cnt; j++) {
                if (!(tmask[warp][j] & bit) || (!ZETA && spos[warp][j] == tpos)) continue;
                const SrcEstrF64& p = dtile[warp][j];
                const double dx = p.xy.x - me.tx, dy = p.xy.y - me.ty, dz = p.z_isig.x - me.tz;
                const double isig = p.z_isig.y;
                const double z = zeta_f64<K>(sqrt(dx * dx + dy * dy + dz * dz) * isig) * isig * isig * isig;
                zg[0] += z * p.gxy.x; zg[1] += z * p.gxy.y; zg[2] += z * p.gz_vx.x;
                zv[0] += z * p.gz_vx.y; zv[1] += z * p.vyz.x; zv[2] += z * p.vyz.y;
            }
        }
    }
    if constexpr (MIXED) {
#pragma unroll
        for (int k = 0; k < 3; k++) { zg[k] += (double)sg[k] + (double)cg[k]; zv[k] += (double)sv[k] + (double)cv[k]; }
    }
    if (!live) return;
    double o[3];
    if constexpr (ZETA) {
#pragma unroll
        for (int k = 0; k < 3; k++) SFS[3 * (int64_t)me.idx + k] += zg[k];
        return;
    }
    const double* Jp = Jt + 9 * (int64_t)me.idx;
    if (transposed) {
        o[0] = Jp[0] * zg[0] + Jp[1] * zg[1] + Jp[2] * zg[2] - zv[0];
        o[1] = Jp[3] * zg[0] + Jp[4] * zg[1] + Jp[5] * zg[2] - zv[1];
        o[2] = Jp[6] * zg[0] + Jp[7] * zg[1] + Jp[8] * zg[2] - zv[2];
    } else {
        o[0] = Jp[0] * zg[0] + Jp[3] * zg[1] + Jp[6] * zg[2] - zv[0];
        o[1] = Jp[1] * zg[0] + Jp[4] * zg[1] + Jp[7] * zg[2] - zv[1];
        o[2] = Jp[2] * zg[0] + Jp[5] * zg[1] + Jp[8] * zg[2] - zv[2];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) SFS[3 * (int64_t)me.idx + k] += o[k];
}

// ---------------------------------------------------------------------- launcher
size_t leaf_work_bytes(int64_t n)
{
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t src = sizeof(SrcEstrDF) > sizeof(SrcEstrF64) ? sizeof(SrcEstrDF) : sizeof(SrcEstrF64);
    return al(n * sizeof(TgtPos)) + al(n * src);
}

template <int K>
static cudaError_t launch_leaf_k(const LeafArgs& a, const NearLists& L, void* work, cudaStream_t st,
                                 int64_t* launches)
{
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const int64_t n = a.n;
    char* p = (char*)work;
    TgtPos* tgt = (TgtPos*)p;            p += al(n * sizeof(TgtPos));
    void* src = p;
    const unsigned g = (unsigned)((n + 255) / 256);
    const unsigned gb = (unsigned)((L.ngroups + NF_WARPS - 1) / NF_WARPS);
    const unsigned gl = (unsigned)((L.nleaves + NF_WARPS - 1) / NF_WARPS);
    tgt_from_perm<<<g, 256, 0, st>>>(n, a.x, L.perm, tgt);
    *launches += 1;
    if (a.uj && a.precision) {
#if VPM_NF_LANE
        leaf_pack_lane<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, L.perm, (SrcMixed*)src);
        nf_uj_lane<K><<<(unsigned)((n + NF_THREADS - 1) / NF_THREADS), NF_THREADS, 0, st>>>(
            n, tgt, L.leaf_of, L.leaf_begin, L.leaf_end, L.row, L.col, (const SrcMixed*)src, a.U, a.J);
#elif VPM_NF_LEAF
        leaf_pack_scaled<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, L.perm, (SrcMixed*)src);
        nf_uj_leaf<K><<<gl, NF_THREADS, 0, st>>>(L.nleaves, tgt, L.leaf_begin, L.leaf_end, L.row, L.col,
                                                 (const SrcMixed*)src, a.U, a.J);
#else
        leaf_pack_lane<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, L.perm, (SrcMixed*)src);
        nf_uj_mixed<K><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs,
                                                  (const SrcMixed*)src, a.U, a.J);
#endif
        *launches += 2;
    } else if (a.uj) {
        leaf_pack_f64<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, L.perm, (SrcF64*)src);
        nf_uj_f64<K><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs,
                                                (const SrcF64*)src, a.U, a.J);
        *launches += 2;
    }
    if (a.sfs) {
        if (VPM_NF_LEAF && a.precision) {
            leaf_pack_estr_df<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, a.J, a.static_flags, a.transposed, L.perm,
                                                     (SrcEstrDF*)src);
            nf_estr_leaf<K><<<gl, NF_THREADS, 0, st>>>(L.nleaves, tgt, L.leaf_begin, L.leaf_end, L.row, L.col,
                                                       (const SrcEstrDF*)src, a.J, a.static_flags, a.transposed,
                                                       a.SFS);
        } else {
            leaf_pack_estr<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, a.J, a.static_flags, a.transposed, L.perm,
                                                  a.precision, src);
            if (a.precision)
                nf_estr<K, true><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs, src, a.J,
                                                            a.static_flags, a.transposed, a.SFS);
            else
                nf_estr<K, false><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs, src,
                                                             a.J, a.static_flags, a.transposed, a.SFS);
        }
        *launches += 2;
    }
    return cudaGetLastError();
}

// The dynamic procedure's differences over the near lists, FP32-comp:
// dJ = the filter difference of J; dSFS = the weight-difference Estr at J plus
// the Estr of dJ at alpha sigma (sig_a); a.J is J, a.sfs and a.U unused.
template <int K>
static cudaError_t launch_leaf_dyn_k(const LeafArgs& a, const NearLists& L, double alpha, const double* sig_a,
                                     double* dJ, double* dSFS, void* work, cudaStream_t st, int64_t* launches)
{
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const int64_t n = a.n;
    char* p = (char*)work;
    TgtPos* tgt = (TgtPos*)p;            p += al(n * sizeof(TgtPos));
    void* src = p;
    const unsigned g = (unsigned)((n + 255) / 256);
    const unsigned gb = (unsigned)((L.ngroups + NF_WARPS - 1) / NF_WARPS);
    const double ha = 1.0 / alpha - 1.0;
    tgt_from_perm<<<g, 256, 0, st>>>(n, a.x, L.perm, tgt);
    *launches += 1;
    if constexpr (K != K_SING) {   // g = 1 has no sigma dependence: dJ = 0
        leaf_pack_mixed<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, L.perm, (SrcMixed*)src);
        const int m = filter_panels(ha);
        if (m == 1)
            nf_filter_diff<K, 1><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs,
                                                            (const SrcMixed*)src, (float)ha, 1, dJ);
        else
            nf_filter_diff<K, 0><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs,
                                                            (const SrcMixed*)src, (float)(ha / m), m, dJ);
        *launches += 2;
    }
    const float3 fd = make_float3((float)(1.0 / (alpha * alpha * alpha) - 1.0), (float)(1.0 / (alpha * alpha * alpha)),
                                  (float)(1.0 / (alpha * alpha) - 1.0));
#if VPM_NF_LEAF
    const unsigned gl = (unsigned)((L.nleaves + NF_WARPS - 1) / NF_WARPS);
    leaf_pack_estr_df<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, a.J, a.static_flags, a.transposed, L.perm,
                                             (SrcEstrDF*)src);
    nf_estr_leaf<K, true><<<gl, NF_THREADS, 0, st>>>(L.nleaves, tgt, L.leaf_begin, L.leaf_end, L.row, L.col,
                                                     (const SrcEstrDF*)src, a.J, a.static_flags, a.transposed, dSFS,
                                                     fd);
    leaf_pack_estr_df<K><<<g, 256, 0, st>>>(n, a.x, a.gam, sig_a, dJ, a.static_flags, a.transposed, L.perm,
                                             (SrcEstrDF*)src);
    nf_estr_leaf<K><<<gl, NF_THREADS, 0, st>>>(L.nleaves, tgt, L.leaf_begin, L.leaf_end, L.row, L.col,
                                               (const SrcEstrDF*)src, dJ, a.static_flags, a.transposed, dSFS);
#else
    leaf_pack_estr<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, a.J, a.static_flags, a.transposed, L.perm, 1, src);
    nf_estr<K, true, true><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs, src, a.J,
                                                      a.static_flags, a.transposed, dSFS, fd);
    leaf_pack_estr<K><<<g, 256, 0, st>>>(n, a.x, a.gam, sig_a, dJ, a.static_flags, a.transposed, L.perm, 1, src);
    nf_estr<K, true><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs, src, dJ,
                                                a.static_flags, a.transposed, dSFS);
#endif
    *launches += 4;
    return cudaGetLastError();
}

cudaError_t launch_leaf_dynamic(const LeafArgs& a, const NearLists& L, double alpha, const double* sig_a, double* dJ,
                                double* dSFS, void* work, cudaStream_t st, int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    if (!a.precision) return cudaErrorInvalidValue;   // FP32-comp only
    switch (a.kernel) {
    case K_SING: return launch_leaf_dyn_k<K_SING>(a, L, alpha, sig_a, dJ, dSFS, work, st, launches);
    case K_GAUS: return launch_leaf_dyn_k<K_GAUS>(a, L, alpha, sig_a, dJ, dSFS, work, st, launches);
    case K_GAUSERF: return launch_leaf_dyn_k<K_GAUSERF>(a, L, alpha, sig_a, dJ, dSFS, work, st, launches);
    case K_WNKLMNS: return launch_leaf_dyn_k<K_WNKLMNS>(a, L, alpha, sig_a, dJ, dSFS, work, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

// zeta_fmm's near-field sum: W += sum over the near lists of zeta(r/sigma_s)/sigma_s^3 Gamma_s
// (a.x, a.gam, a.sig; every particle a target, the self pair included).
template <int K>
static cudaError_t launch_leaf_zeta_k(const LeafArgs& a, const NearLists& L, double* W, void* work, cudaStream_t st,
                                      int64_t* launches)
{
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const int64_t n = a.n;
    char* p = (char*)work;
    TgtPos* tgt = (TgtPos*)p;            p += al(n * sizeof(TgtPos));
    void* src = p;
    const unsigned g = (unsigned)((n + 255) / 256);
    const unsigned gb = (unsigned)((L.ngroups + NF_WARPS - 1) / NF_WARPS);
    const unsigned gl = (unsigned)((L.nleaves + NF_WARPS - 1) / NF_WARPS);
    tgt_from_perm<<<g, 256, 0, st>>>(n, a.x, L.perm, tgt);
    if (VPM_NF_LEAF && a.precision) {
        leaf_pack_estr_df<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, nullptr, nullptr, true, L.perm, (SrcEstrDF*)src);
        nf_estr_leaf<K, false, true><<<gl, NF_THREADS, 0, st>>>(L.nleaves, tgt, L.leaf_begin, L.leaf_end, L.row,
                                                                L.col, (const SrcEstrDF*)src, nullptr, nullptr, true,
                                                                W);
    } else {
        leaf_pack_estr<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, nullptr, nullptr, true, L.perm, a.precision, src);
        if (a.precision)
            nf_estr<K, true, false, true><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs,
                                                                     src, nullptr, nullptr, true, W);
        else
            nf_estr<K, false, false, true><<<gb, NF_THREADS, 0, st>>>(n, L.ngroups, tgt, L.leaf_of, L.grp_row, L.ivs,
                                                                      src, nullptr, nullptr, true, W);
    }
    *launches += 3;
    return cudaGetLastError();
}

cudaError_t launch_leaf_zeta(const LeafArgs& a, const NearLists& L, double* W, void* work, cudaStream_t st,
                             int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_leaf_zeta_k<K_SING>(a, L, W, work, st, launches);
    case K_GAUS: return launch_leaf_zeta_k<K_GAUS>(a, L, W, work, st, launches);
    case K_GAUSERF: return launch_leaf_zeta_k<K_GAUSERF>(a, L, W, work, st, launches);
    case K_WNKLMNS: return launch_leaf_zeta_k<K_WNKLMNS>(a, L, W, work, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_leaflist(const LeafArgs& a, const NearLists& L, void* work, cudaStream_t st, int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_leaf_k<K_SING>(a, L, work, st, launches);
    case K_GAUS: return launch_leaf_k<K_GAUS>(a, L, work, st, launches);
    case K_GAUSERF: return launch_leaf_k<K_GAUSERF>(a, L, work, st, launches);
    case K_WNKLMNS: return launch_leaf_k<K_WNKLMNS>(a, L, work, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
