// uj.cu -- all-pairs U and J kernels (the P2P pair loop of
// src/FLOWVPM_fmm.jl:102-168, over all sources as UJ_direct does,
// src/FLOWVPM_UJ.jl:35).
//
// Layout: one target per thread, UJ_THREADS targets per block, targets in
// Morton order (order.cu) so each warp holds 32 neighbouring targets.  Sources
// are packed once per call (in the same Morton order when they are the
// targets).  The FP64 kernel streams them through shared memory in block-wide
// tiles of UJ_TILE; in the mixed kernel every warp streams them on its own in
// tiles of 32, double-buffered with cp.async, so warps never wait for one
// another.  gridDim.y splits the sources when there are too few target blocks
// to fill the GPU; each split then writes FP64 partial sums to scratch and
// uj_reduce adds them, in split order, to the outputs.
//
// Mixed (FP32-comp) kernel.  Positions are double-floats (hi + lo in FP32).
//  * Far pairs: each warp takes its first target as origin and, once per tile,
//    converts every source to an FP32 offset from it; dx = o_t - o_s then costs
//    3 FP32 subtractions with an error of a few ulp of |dx| + the warp's extent
//    b.  A source is "far" for a lane when r^2 > max(s_far sigma^2, (2b)^2):
//    the kernel is then in its singular form (G = r^-3, Q = r^-5, no sigma) and
//    the offset error is below 1.5 ulp of |dx|.
//  * When any lane of the warp has a near pair among 4 sources (one vote), the
//    warp evaluates those 4 pairs with dx = (x_t,hi - x_s,hi) + (x_t,lo - x_s,lo)
//    and the full regular form of the kernel (vpm_math.cuh).
// Sums run in FP32 over blocks of UJ_BLOCK sources, then in an FP32 mid-level
// sum over UJ_FLUSH_TILES tiles, then in FP64.
#include "internal.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

namespace vpm {

static_assert(UJ_TILE == UJ_THREADS, "one source loaded per thread per tile");
static_assert(UJ_TILE % UJ_BLOCK == 0, "FP32 blocks must tile the shared tile");
static_assert(UJ_BLOCK % 4 == 0, "far/near votes cover groups of 4 sources");
static_assert(UJ_TILE % 32 == 0, "per-warp conversion covers the tile in whole passes");

static inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

size_t uj_src_pack_bytes(int64_t ns, int precision)
{
    const int64_t n = round_up(ns, UJ_TILE);
    return (size_t)n * (precision ? sizeof(SrcMixed) : sizeof(SrcF64));
}

int uj_num_splits(int64_t nt, int64_t ns, int num_sms)
{
    const int64_t tblocks = (nt + UJ_THREADS - 1) / UJ_THREADS;
    const int64_t tiles = (ns + UJ_TILE - 1) / UJ_TILE;
    // aim for about two waves of ~6 resident blocks per SM
    const int64_t want = 12LL * num_sms;
    int64_t nsplit = (want + tblocks - 1) / tblocks;
    int64_t max_split = tiles / 4;          // keep at least 4 tiles per split
    if (max_split < 1) max_split = 1;
    if (nsplit > max_split) nsplit = max_split;
    if (nsplit < 1) nsplit = 1;
    const int64_t per = (tiles + nsplit - 1) / nsplit;   // no empty splits
    nsplit = (tiles + per - 1) / per;
    return (int)nsplit;
}

size_t uj_partial_bytes(int64_t nt, int nsplit)
{
    return nsplit > 1 ? (size_t)nsplit * 12 * (size_t)round_up(nt, UJ_THREADS) * sizeof(double) : 0;
}


// ------------------------------------------------------------------ packing
// When `order` is given (sources = targets), source i of the pack is particle
// order[i].idx, i.e. the sources follow the targets' Morton order: a warp's
// near sources then sit in few 4-source groups, so fewer groups take the near
// path.  The order of a sum's terms does not otherwise matter.
template <int K>
__global__ void pack_src_mixed(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
                               const double* __restrict__ gs, const double* __restrict__ sgs,
                               const TgtPos* __restrict__ order, SrcMixed* __restrict__ out)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= ns_pad) return;
    SrcMixed p;
    if (o < ns) {
        const int64_t i = order ? (int64_t)order[o].idx : o;
        const double x = xs[3 * i], y = xs[3 * i + 1], z = xs[3 * i + 2];
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        const double sig = (K == K_SING) ? 1.0 : sgs[i];
        const double k = singular_tail<K>() ? -C4 : -C4 / (sig * sig * sig);
        p.a = make_float4(xh, yh, zh, (float)(sig * sig));
        p.b = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh),
                          (float)(1.0 / sig));
        p.gam = make_float4((float)(k * gs[3 * i]), (float)(k * gs[3 * i + 1]), (float)(k * gs[3 * i + 2]), 0.f);
    } else {  // padding: no strength, at the origin, unit core
        p.a = make_float4(0.f, 0.f, 0.f, 1.f);
        p.b = make_float4(0.f, 0.f, 0.f, 1.f);
        p.gam = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    out[o] = p;
}

template <int K>
__global__ void pack_src_f64(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
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
        // .y: for Gaussian-erf the r^2 past which g = 1, g' = 0 (rho > 9), else sigma
        p.gz_sig = make_double2(gs[3 * i + 2], K == K_GAUSERF ? 81.0 * sig * sig : sig);
    } else {
        p.xy = make_double2(0.0, 0.0);
        p.z_isig = make_double2(0.0, 1.0);
        p.gxy = make_double2(0.0, 0.0);
        p.gz_sig = make_double2(0.0, 1.0);
    }
    out[i] = p;
}

// ------------------------------------------------------------ pair: FP64
// The reference formula of src/FLOWVPM_fmm.jl:112-160 with 1/sigma taken from
// the payload and r^-1 from rsqrt.  Pairs with r^2 == 0 are skipped (:118).
template <int K>
__device__ __forceinline__ void pair_f64(double tx, double ty, double tz, const SrcF64& s,
                                         double (&acc)[12])
{
    const double dx = tx - s.xy.x, dy = ty - s.xy.y, dz = tz - s.z_isig.x;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 != 0.0) {
        const double rinv = rsqrt(r2);
        const double r = r2 * rinv;
        const double isig = s.z_isig.y;
        double g, dg;
        g_dgdr_f64<K>(r * isig, g, dg);
        const double r3inv = rinv * rinv * rinv;
        const double gx = s.gxy.x, gy = s.gxy.y, gz = s.gz_sig.x;
        const double k = -C4 * r3inv;
        const double crss1 = k * (dy * gz - dz * gy);
        const double crss2 = k * (dz * gx - dx * gz);
        const double crss3 = k * (dx * gy - dy * gx);
        acc[0] += g * crss1;
        acc[1] += g * crss2;
        acc[2] += g * crss3;
        const double aux = dg * isig * rinv - 3.0 * g * rinv * rinv;
        const double aux2 = -C4 * g * r3inv;
        const double a1 = aux * crss1, a2 = aux * crss2, a3 = aux * crss3;
        acc[3] += a1 * dx;
        acc[4] += a2 * dx - aux2 * gz;
        acc[5] += a3 * dx + aux2 * gy;
        acc[6] += a1 * dy + aux2 * gz;
        acc[7] += a2 * dy;
        acc[8] += a3 * dy - aux2 * gx;
        acc[9] += a1 * dz - aux2 * gy;
        acc[10] += a2 * dz + aux2 * gx;
        acc[11] += a3 * dz;
    }
}

#ifndef VPM_UJ_F64_ACC
// 1: the FP64 pair in the accumulated form (pair_f64_acc, uj_pair.cuh), measured 1.44x
// faster than 0, the reference's per-pair form (pair_f64: 62 FP64 instructions a pair),
// on 2^15 x 2^20 Gaussian-erf pairs
#define VPM_UJ_F64_ACC 1
#endif

// --------------------------------------------------------------- epilogue
__device__ __forceinline__ void write_uj(int64_t t, int32_t idx, const double (&acc)[12], double* U,
                                         int64_t ldU, double* J, int64_t ldJ, double* partial, int64_t nt_pad)
{
    if (partial) {
        double* p = partial + (int64_t)blockIdx.y * 12 * nt_pad + t;
#pragma unroll
        for (int k = 0; k < 12; k++) p[k * nt_pad] = acc[k];
    } else {
        const int64_t i = idx;
#pragma unroll
        for (int k = 0; k < 3; k++) U[i * ldU + k] += acc[k];
#pragma unroll
        for (int k = 0; k < 9; k++) J[i * ldJ + k] += acc[3 + k];
    }
}

__global__ void uj_reduce(int64_t nt, int nsplit, const double* __restrict__ partial, int64_t nt_pad,
                          const TgtPos* __restrict__ tgt, double* U, int64_t ldU, double* J, int64_t ldJ)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int64_t i = tgt[t].idx;
    for (int k = 0; k < 12; k++) {
        double s = 0.0;
        for (int sp = 0; sp < nsplit; sp++) s += partial[((int64_t)sp * 12 + k) * nt_pad + t];
        if (k < 3) U[i * ldU + k] += s;
        else J[i * ldJ + (k - 3)] += s;
    }
}

// ------------------------------------------------------------ main kernels
template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
uj_f64_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad, const SrcF64* __restrict__ src,
              int64_t per_split, double* U, int64_t ldU, double* J, int64_t ldJ,
              double* partial, int64_t nt_pad)
{
    __shared__ SrcF64 tile[UJ_TILE];
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 1.0e3, ty = 1.0e3, tz = 1.0e3;
    int32_t idx = 0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    double acc[12];
#if VPM_UJ_F64_ACC
    double u[3] = {0.0, 0.0, 0.0}, w[3] = {0.0, 0.0, 0.0}, jq[9];
#pragma unroll
    for (int k = 0; k < 9; k++) jq[k] = 0.0;
#else
#pragma unroll
    for (int k = 0; k < 12; k++) acc[k] = 0.0;
#endif
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < UJ_TILE; j++) {
#if VPM_UJ_F64_ACC
            pair_f64_acc<K>(tx, ty, tz, tile[j], u, w, jq);
#else
            pair_f64<K>(tx, ty, tz, tile[j], acc);
#endif
        }
    }
#if VPM_UJ_F64_ACC
    uj_f64_finish(u, w, jq, acc);
#endif
    if (valid) write_uj(t, idx, acc, U, ldU, J, ldJ, partial, nt_pad);
}

// 16-byte asynchronous global->shared copy (LDGSTS), L2-cached.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

#ifndef VPM_UJ_BULK
// 1: one lane fills its warp's 1,536-byte source tile with a bulk copy (cp.async.bulk)
// completed on an mbarrier, instead of 3 cp.async a lane (uj_mixed_kernel only).  Measured
// at N = 2^20: the same U, J to every digit, but 3.4 % slower for Gaussian-erf (1394-1402 ms
// a launch against 1352-1354) and 3.1 % for Winckelmans (1546-1548 against 1499-1502); not
// profiled: each lane saves 2 copy instructions a tile and polls the barrier once instead.
#define VPM_UJ_BULK 0
#endif
#if VPM_UJ_BULK
constexpr int UJ_BULK_SPIN = 1 << 14;       // try_wait rounds before a wait gives up
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* m)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(m)) : "memory");
}
// bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) completing on m
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* m)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(m)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(m)) : "memory");
}
// true once the phase of m with this parity has completed; false after UJ_BULK_SPIN rounds
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity)
{
    for (int i = 0; i < UJ_BULK_SPIN; i++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done) : "r"(smem_addr(m)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}
#endif

constexpr int WT = 32;                      // sources per warp tile (one per lane)
constexpr int BLOCK_TILES = UJ_BLOCK / WT;  // warp tiles per FP32 block
// FP32 blocks per FP32 mid-level sum: 16 x 64 sources between FP64 adds (4 measured 1.2 %
// slower -- the FP64 pipe runs at 1/64 rate -- with the same U, J error against the oracle)
constexpr int MID_BLOCKS = 16;
// Resident blocks per SM the register budget targets, per kernel: at N = 2^20 with the
// per-tile far flags, Gaussian-erf ran 1360 ms a launch at 5 (96 registers), 1400 at 6
// (80) and 1408 at 7 (72, a few spills); Winckelmans, whose far form is its full form,
// 1522 at 5 and 1503 at 6.  -DVPM_UJ_MIN_BLOCKS=n sets one budget for every kernel.
template <int K>
__host__ __device__ constexpr int uj_min_blocks()
{
#ifdef VPM_UJ_MIN_BLOCKS
    return VPM_UJ_MIN_BLOCKS;
#else
    return K == K_WNKLMNS ? 6 : 5;
#endif
}
#ifndef VPM_UJ_UNROLL
#define VPM_UJ_UNROLL 2                     // 4-source groups unrolled per iteration of a tile
#endif
constexpr int UJ_UNROLL = VPM_UJ_UNROLL;
#ifndef VPM_UJ_F32X2
#define VPM_UJ_F32X2 0                      // 1: the packed-FP32 mixed kernel (uj_mixed_x2_kernel)
#endif
#ifndef VPM_UJ_SMEM_ACC
// 1: the FP64 sums (touched once per 1,024 sources) live in shared memory, which frees the
// registers for 7 resident blocks per SM instead of 5 -- measured 3.6 % faster at N = 2^20
#define VPM_UJ_SMEM_ACC 1
#endif
#ifndef VPM_UJ_TPL
// targets per lane of the mixed kernel: 1 (uj_mixed_kernel) or 2 (uj_mixed2_kernel)
#define VPM_UJ_TPL 1
#endif
#ifndef VPM_UJ_TILE_FLAGS
// 1: far/near decided once per tile from the warp's target box: the loading lane flags its
// source far when the box is out of the source's reach, one ballot gives the tile's flags,
// a tile of far sources runs the far form with no test, other tiles choose per 4-source
// group.  0: every pair tested, one vote per 4-source group (pair4_mixed).
#define VPM_UJ_TILE_FLAGS 1
#endif

// Each warp streams the sources on its own: 32 per tile, double-buffered with
// cp.async, so warps never wait for each other (no block-wide barrier).
template <int K>
__global__ void __launch_bounds__(UJ_THREADS, uj_min_blocks<K>())
uj_mixed_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad,
                const SrcMixed* __restrict__ src, int64_t per_split, double* U, int64_t ldU,
                double* J, int64_t ldJ, double* partial, int64_t nt_pad)
{
    __shared__ SrcMixed stage[UJ_WARPS][2][WT];
    __shared__ float4 offs[UJ_WARPS][2][WT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 3.0e4, ty = 3.0e4, tz = 3.0e4;
    int32_t idx = 0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const float3 th = make_float3((float)tx, (float)ty, (float)tz);
    const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y), (float)(tz - (double)th.z));
    // warp origin: lane 0's target (valid whenever any lane of the warp is)
    const double ox = __shfl_sync(0xffffffffu, tx, 0);
    const double oy = __shfl_sync(0xffffffffu, ty, 0);
    const double oz = __shfl_sync(0xffffffffu, tz, 0);
    const float3 oh = make_float3(__shfl_sync(0xffffffffu, th.x, 0), __shfl_sync(0xffffffffu, th.y, 0),
                                  __shfl_sync(0xffffffffu, th.z, 0));
    const float3 ol = make_float3(__shfl_sync(0xffffffffu, tl.x, 0), __shfl_sync(0xffffffffu, tl.y, 0),
                                  __shfl_sync(0xffffffffu, tl.z, 0));
    const float3 to = valid ? make_float3((float)(tx - ox), (float)(ty - oy), (float)(tz - oz))
                            : make_float3(3.0e4f, 3.0e4f, 3.0e4f);
    // (2 b)^2 with b the largest |offset| of the warp's valid targets
    float b2 = valid ? fmaf(to.x, to.x, fmaf(to.y, to.y, to.z * to.z)) : 0.0f;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, m));
    const float r2n = fmaxf(4.0f * b2, 1.0e-30f);
    const float sfar = s_far<K>();
#if VPM_UJ_TILE_FLAGS
    // the box of the warp's valid targets (offsets; empty when it has none), read by the
    // loading lanes
    __shared__ float4 wbox[UJ_WARPS][2];
    {
        float lo[3] = {valid ? to.x : 3.0e38f, valid ? to.y : 3.0e38f, valid ? to.z : 3.0e38f};
        float hi[3] = {valid ? to.x : -3.0e38f, valid ? to.y : -3.0e38f, valid ? to.z : -3.0e38f};
#pragma unroll
        for (int m = 16; m > 0; m >>= 1)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], m));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], m));
            }
        if (lane == 0) {
            wbox[warp][0] = make_float4(lo[0], lo[1], lo[2], 0.f);
            wbox[warp][1] = make_float4(hi[0], hi[1], hi[2], 0.f);
        }
        __syncwarp();
    }
#endif

#if VPM_UJ_SMEM_ACC
    // FP64 sums of this thread: [0..2] U, [3..5] W, [6..13] J' (touched once per mid-level flush)
    __shared__ double acc64[14][UJ_THREADS];
#pragma unroll
    for (int k = 0; k < 14; k++) acc64[k][threadIdx.x] = 0.0;
#define ACC_DU(k) acc64[k][threadIdx.x]
#define ACC_DW(k) acc64[3 + (k)][threadIdx.x]
#define ACC_DJ(k) acc64[6 + (k)][threadIdx.x]
#else
    double dU[3] = {0.0, 0.0, 0.0}, dW[3] = {0.0, 0.0, 0.0};
    double dJ[8];
#pragma unroll
    for (int k = 0; k < 8; k++) dJ[k] = 0.0;
#define ACC_DU(k) dU[k]
#define ACC_DW(k) dW[k]
#define ACC_DJ(k) dJ[k]
#endif
    float mu[3] = {0.f, 0.f, 0.f}, mw[3] = {0.f, 0.f, 0.f}, mj[8];
    float u[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f}, jq[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { mj[k] = 0.f; jq[k] = 0.f; }

    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    const int ntiles = (int)((s1 - s0) / WT);
#if VPM_UJ_BULK
    // one mbarrier per buffer of the warp; tile it lands in buffer it & 1 on that barrier's
    // phase it >> 1
    __shared__ __align__(8) uint64_t tbar[UJ_WARPS][2];
    if (lane == 0) {
        mbar_init(&tbar[warp][0]);
        mbar_init(&tbar[warp][1]);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();
    bool bulk_ok = true;
    int it_fail = 0;
    if (ntiles > 0 && lane == 0)
        bulk_g2s(&stage[warp][0][0], src + s0, WT * sizeof(SrcMixed), &tbar[warp][0]);
#else
    const SrcMixed* wsrc = src + s0 + lane;
    if (ntiles > 0) {
        SrcMixed* d = &stage[warp][0][lane];
        cp_async16(&d->a, &wsrc->a);
        cp_async16(&d->b, &wsrc->b);
        cp_async16(&d->gam, &wsrc->gam);
        cp_async_commit();
    }
#endif
    int in_block = 0, in_mid = 0;
    for (int it = 0; it < ntiles; it++) {
        const int buf = it & 1;
#if VPM_UJ_BULK
        if (it + 1 < ntiles && lane == 0) {
            // the lanes' reads of this buffer (ordered by the loop's last __syncwarp) before
            // the async proxy overwrites it
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            bulk_g2s(&stage[warp][buf ^ 1][0], src + s0 + (int64_t)(it + 1) * WT, WT * sizeof(SrcMixed),
                     &tbar[warp][buf ^ 1]);
        }
        if (!__all_sync(0xffffffffu, mbar_wait(&tbar[warp][buf], (uint32_t)(it >> 1) & 1u))) {
            bulk_ok = false;
            it_fail = it;
            break;
        }
#else
        if (it + 1 < ntiles) {
            const SrcMixed* g = wsrc + (int64_t)(it + 1) * WT;
            SrcMixed* d = &stage[warp][buf ^ 1][lane];
            cp_async16(&d->a, &g->a);
            cp_async16(&d->b, &g->b);
            cp_async16(&d->gam, &g->gam);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
#endif
        __syncwarp();
#if VPM_UJ_TILE_FLAGS
        bool far_src;
        {   // this lane's source: FP32 offset from the warp origin, and whether every pair
            // with the warp's targets is past max(reach, (2 b)^2)
            const float4 a = stage[warp][buf][lane].a, b = stage[warp][buf][lane].b;
            const float px = (a.x - oh.x) + (b.x - ol.x), py = (a.y - oh.y) + (b.y - ol.y),
                        pz = (a.z - oh.z) + (b.z - ol.z);
            offs[warp][buf][lane] = make_float4(px, py, pz, b.w * b.w);
            const float4 lo = wbox[warp][0], hi = wbox[warp][1];
            const float ex = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.0f);
            const float ey = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.0f);
            const float ez = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.0f);
            const float thr = singular_tail<K>() ? fmaxf(sfar * a.w, r2n) : r2n;
            far_src = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > thr;
        }
        const unsigned farbits = __ballot_sync(0xffffffffu, far_src);
        __syncwarp();
        if (farbits == 0xffffffffu) {
#pragma unroll (UJ_UNROLL)
            for (int j = 0; j < WT; j += 4) pair4_far<K>(to, offs[warp][buf], stage[warp][buf], j, u, jq, w);
        } else {
#pragma unroll 1
            for (int j = 0; j < WT; j += 4) {
                if (((farbits >> j) & 0xFu) == 0xFu)
                    pair4_far<K>(to, offs[warp][buf], stage[warp][buf], j, u, jq, w);
                else
                    pair4_near<K>(th, tl, offs[warp][buf], stage[warp][buf], j, u, jq, w);
            }
        }
#else
        {   // this lane's source: FP32 offset from the warp origin and its far threshold
            const float4 a = stage[warp][buf][lane].a, b = stage[warp][buf][lane].b;
            const float thr = singular_tail<K>() ? fmaxf(sfar * a.w, r2n) : b.w * b.w;
            offs[warp][buf][lane] = make_float4((a.x - oh.x) + (b.x - ol.x), (a.y - oh.y) + (b.y - ol.y),
                                                (a.z - oh.z) + (b.z - ol.z), thr);
        }
        __syncwarp();
#pragma unroll (UJ_UNROLL)
        for (int j = 0; j < WT; j += 4)
            pair4_mixed<K>(to, th, tl, r2n, offs[warp][buf], stage[warp][buf], j, u, jq, w);
#endif
        if (++in_block == BLOCK_TILES) {
#pragma unroll
            for (int k = 0; k < 3; k++) { mu[k] += u[k]; mw[k] += w[k]; u[k] = 0.f; w[k] = 0.f; }
#pragma unroll
            for (int k = 0; k < 8; k++) { mj[k] += jq[k]; jq[k] = 0.f; }
            in_block = 0;
            if (++in_mid == MID_BLOCKS) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    ACC_DU(k) += (double)mu[k]; ACC_DW(k) += (double)mw[k]; mu[k] = 0.f; mw[k] = 0.f;
                }
#pragma unroll
                for (int k = 0; k < 8; k++) { ACC_DJ(k) += (double)mj[k]; mj[k] = 0.f; }
                in_mid = 0;
            }
        }
        __syncwarp();   // every lane is done with `buf` before it is refilled
    }
    // remaining partial block and mid-level sums
    double fU[3], fW[3], fJ[8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        fU[k] = ACC_DU(k) + ((double)mu[k] + (double)u[k]);
        fW[k] = ACC_DW(k) + ((double)mw[k] + (double)w[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) fJ[k] = ACC_DJ(k) + ((double)mj[k] + (double)jq[k]);
#undef ACC_DU
#undef ACC_DW
#undef ACC_DJ
#if VPM_UJ_BULK
    if (!bulk_ok) {
        // a tile that did not arrive: wait (bounded) for this warp's copies still in flight,
        // then mark the warp's sums as failed
        mbar_wait(&tbar[warp][it_fail & 1], (uint32_t)(it_fail >> 1) & 1u);
        if (it_fail + 1 < ntiles) mbar_wait(&tbar[warp][(it_fail + 1) & 1], (uint32_t)((it_fail + 1) >> 1) & 1u);
        const double qnan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
        for (int k = 0; k < 3; k++) { fU[k] = qnan; fW[k] = qnan; }
#pragma unroll
        for (int k = 0; k < 8; k++) fJ[k] = qnan;
    }
#endif
    if (!valid) return;
    // J = -3 J' (J'_33 = -J'_11 - J'_22) plus the Kronecker term of
    // src/FLOWVPM_fmm.jl:148-159 (W = sum aux2 Gamma)
    double j9[9];
#pragma unroll
    for (int k = 0; k < 8; k++) j9[k] = -3.0 * fJ[k];
    j9[8] = 3.0 * (fJ[0] + fJ[4]);
    j9[1] -= fW[2];
    j9[2] += fW[1];
    j9[3] += fW[2];
    j9[5] -= fW[0];
    j9[6] -= fW[1];
    j9[7] += fW[0];
    double acc[12] = {fU[0], fU[1], fU[2], j9[0], j9[1], j9[2], j9[3], j9[4], j9[5], j9[6], j9[7], j9[8]};
    write_uj(t, idx, acc, U, ldU, J, ldJ, partial, nt_pad);
}
// --------------------------------------------- mixed kernel, two targets a lane
// uj_mixed_kernel with two targets per lane: a warp takes 64 Morton-consecutive
// targets (lane l: base + l and base + 32 + l), so that each source's shared-memory
// reads, its tile's far flag and the tile's loads and conversions serve two pairs.
// Blocks of 128 threads take 256 targets; the register budget is 3 resident blocks
// per SM (every sum of both targets in registers, FP64 sums in shared memory).
template <int K>
__global__ void __launch_bounds__(UJ_THREADS, 3)
uj_mixed2_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad,
                 const SrcMixed* __restrict__ src, int64_t per_split, double* U, int64_t ldU,
                 double* J, int64_t ldJ, double* partial, int64_t nt_pad)
{
    __shared__ SrcMixed stage[UJ_WARPS][2][WT];
    __shared__ float4 offs[UJ_WARPS][2][WT];
    __shared__ float4 wbox[UJ_WARPS][2];
    __shared__ double acc64[14][2 * UJ_THREADS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * (2 * UJ_THREADS) + 64 * warp;
    const int64_t tt[2] = {base + lane, base + 32 + lane};
    bool valid[2];
    double tx[2], ty[2], tz[2];
    int32_t idx[2];
    float3 th[2], tl[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        valid[k] = tt[k] < nt;
        tx[k] = ty[k] = tz[k] = 3.0e4;
        idx[k] = 0;
        if (valid[k]) {
            const TgtPos p = tgt[tt[k]];
            tx[k] = p.x; ty[k] = p.y; tz[k] = p.z; idx[k] = p.idx;
        }
        th[k] = make_float3((float)tx[k], (float)ty[k], (float)tz[k]);
        tl[k] = make_float3((float)(tx[k] - (double)th[k].x), (float)(ty[k] - (double)th[k].y),
                            (float)(tz[k] - (double)th[k].z));
    }
    // warp origin: lane 0's first target (valid whenever any target of the warp is)
    const double ox = __shfl_sync(0xffffffffu, tx[0], 0);
    const double oy = __shfl_sync(0xffffffffu, ty[0], 0);
    const double oz = __shfl_sync(0xffffffffu, tz[0], 0);
    const float3 oh = make_float3(__shfl_sync(0xffffffffu, th[0].x, 0), __shfl_sync(0xffffffffu, th[0].y, 0),
                                  __shfl_sync(0xffffffffu, th[0].z, 0));
    const float3 ol = make_float3(__shfl_sync(0xffffffffu, tl[0].x, 0), __shfl_sync(0xffffffffu, tl[0].y, 0),
                                  __shfl_sync(0xffffffffu, tl[0].z, 0));
    float3 to[2];
    float b2 = 0.0f;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        to[k] = valid[k] ? make_float3((float)(tx[k] - ox), (float)(ty[k] - oy), (float)(tz[k] - oz))
                         : make_float3(3.0e4f, 3.0e4f, 3.0e4f);
        if (valid[k]) b2 = fmaxf(b2, fmaf(to[k].x, to[k].x, fmaf(to[k].y, to[k].y, to[k].z * to[k].z)));
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, m));
    const float r2n = fmaxf(4.0f * b2, 1.0e-30f);
    const float sfar = s_far<K>();
    {   // the box of the warp's valid targets (offsets)
        float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
#pragma unroll
        for (int k = 0; k < 2; k++)
            if (valid[k]) {
                lo[0] = fminf(lo[0], to[k].x); lo[1] = fminf(lo[1], to[k].y); lo[2] = fminf(lo[2], to[k].z);
                hi[0] = fmaxf(hi[0], to[k].x); hi[1] = fmaxf(hi[1], to[k].y); hi[2] = fmaxf(hi[2], to[k].z);
            }
#pragma unroll
        for (int m = 16; m > 0; m >>= 1)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], m));
                hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], m));
            }
        if (lane == 0) {
            wbox[warp][0] = make_float4(lo[0], lo[1], lo[2], 0.f);
            wbox[warp][1] = make_float4(hi[0], hi[1], hi[2], 0.f);
        }
    }
#pragma unroll
    for (int k = 0; k < 14; k++) { acc64[k][threadIdx.x] = 0.0; acc64[k][UJ_THREADS + threadIdx.x] = 0.0; }
    __syncwarp();
    float mu0[3] = {0.f, 0.f, 0.f}, mw0[3] = {0.f, 0.f, 0.f}, mj0[8];
    float mu1[3] = {0.f, 0.f, 0.f}, mw1[3] = {0.f, 0.f, 0.f}, mj1[8];
    float u0[3] = {0.f, 0.f, 0.f}, w0[3] = {0.f, 0.f, 0.f}, jq0[8];
    float u1[3] = {0.f, 0.f, 0.f}, w1[3] = {0.f, 0.f, 0.f}, jq1[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { mj0[k] = 0.f; jq0[k] = 0.f; mj1[k] = 0.f; jq1[k] = 0.f; }

    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    const int ntiles = (int)((s1 - s0) / WT);
    const SrcMixed* wsrc = src + s0 + lane;
    if (ntiles > 0) {
        SrcMixed* d = &stage[warp][0][lane];
        cp_async16(&d->a, &wsrc->a);
        cp_async16(&d->b, &wsrc->b);
        cp_async16(&d->gam, &wsrc->gam);
        cp_async_commit();
    }
    int in_block = 0, in_mid = 0;
    for (int it = 0; it < ntiles; it++) {
        const int buf = it & 1;
        if (it + 1 < ntiles) {
            const SrcMixed* g = wsrc + (int64_t)(it + 1) * WT;
            SrcMixed* d = &stage[warp][buf ^ 1][lane];
            cp_async16(&d->a, &g->a);
            cp_async16(&d->b, &g->b);
            cp_async16(&d->gam, &g->gam);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        bool far_src;
        {
            const float4 a = stage[warp][buf][lane].a, b = stage[warp][buf][lane].b;
            const float px = (a.x - oh.x) + (b.x - ol.x), py = (a.y - oh.y) + (b.y - ol.y),
                        pz = (a.z - oh.z) + (b.z - ol.z);
            offs[warp][buf][lane] = make_float4(px, py, pz, b.w * b.w);
            const float4 lo = wbox[warp][0], hi = wbox[warp][1];
            const float ex = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.0f);
            const float ey = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.0f);
            const float ez = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.0f);
            const float thr = singular_tail<K>() ? fmaxf(sfar * a.w, r2n) : r2n;
            far_src = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > thr;
        }
        const unsigned farbits = __ballot_sync(0xffffffffu, far_src);
        __syncwarp();
        if (farbits == 0xffffffffu) {
#pragma unroll (UJ_UNROLL)
            for (int j = 0; j < WT; j += 4)
                pair4_far2<K>(to[0], to[1], offs[warp][buf], stage[warp][buf], j, u0, jq0, w0, u1, jq1, w1);
        } else {
#pragma unroll 1
            for (int j = 0; j < WT; j += 4) {
                if (((farbits >> j) & 0xFu) == 0xFu) {
                    pair4_far2<K>(to[0], to[1], offs[warp][buf], stage[warp][buf], j, u0, jq0, w0, u1, jq1, w1);
                } else {
                    pair4_near<K>(th[0], tl[0], offs[warp][buf], stage[warp][buf], j, u0, jq0, w0);
                    pair4_near<K>(th[1], tl[1], offs[warp][buf], stage[warp][buf], j, u1, jq1, w1);
                }
            }
        }
        if (++in_block == BLOCK_TILES) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                mu0[k] += u0[k]; mw0[k] += w0[k]; u0[k] = 0.f; w0[k] = 0.f;
                mu1[k] += u1[k]; mw1[k] += w1[k]; u1[k] = 0.f; w1[k] = 0.f;
            }
#pragma unroll
            for (int k = 0; k < 8; k++) { mj0[k] += jq0[k]; jq0[k] = 0.f; mj1[k] += jq1[k]; jq1[k] = 0.f; }
            in_block = 0;
            if (++in_mid == MID_BLOCKS) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    acc64[k][threadIdx.x] += (double)mu0[k];
                    acc64[3 + k][threadIdx.x] += (double)mw0[k];
                    acc64[k][UJ_THREADS + threadIdx.x] += (double)mu1[k];
                    acc64[3 + k][UJ_THREADS + threadIdx.x] += (double)mw1[k];
                    mu0[k] = mw0[k] = mu1[k] = mw1[k] = 0.f;
                }
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    acc64[6 + k][threadIdx.x] += (double)mj0[k];
                    acc64[6 + k][UJ_THREADS + threadIdx.x] += (double)mj1[k];
                    mj0[k] = mj1[k] = 0.f;
                }
                in_mid = 0;
            }
        }
        __syncwarp();   // every lane is done with `buf` before it is refilled
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (!valid[k]) continue;
        const int c = k * UJ_THREADS + threadIdx.x;
        double fU[3], fW[3], fJ[8];
#pragma unroll
        for (int m = 0; m < 3; m++) {
            fU[m] = acc64[m][c] + ((double)(k ? mu1[m] : mu0[m]) + (double)(k ? u1[m] : u0[m]));
            fW[m] = acc64[3 + m][c] + ((double)(k ? mw1[m] : mw0[m]) + (double)(k ? w1[m] : w0[m]));
        }
#pragma unroll
        for (int m = 0; m < 8; m++)
            fJ[m] = acc64[6 + m][c] + ((double)(k ? mj1[m] : mj0[m]) + (double)(k ? jq1[m] : jq0[m]));
        double j9[9];
#pragma unroll
        for (int m = 0; m < 8; m++) j9[m] = -3.0 * fJ[m];
        j9[8] = 3.0 * (fJ[0] + fJ[4]);
        j9[1] -= fW[2]; j9[2] += fW[1]; j9[3] += fW[2]; j9[5] -= fW[0]; j9[6] -= fW[1]; j9[7] += fW[0];
        double acc[12] = {fU[0], fU[1], fU[2], j9[0], j9[1], j9[2], j9[3], j9[4], j9[5], j9[6], j9[7], j9[8]};
        write_uj(tt[k], idx[k], acc, U, ldU, J, ldJ, partial, nt_pad);
    }
}

// ------------------------------------------------- packed-FP32 mixed kernel
// The mixed kernel with the pair math in Blackwell's packed FP32 instructions
// (fma / mul / sub .rn.f32x2: two FP32 operations per lane and instruction),
// each instruction taking one pair of sources.  The per-warp tile is staged as
// before; the loading lanes then write it to a packed structure-of-arrays
// layout per source pair (2p, 2p+1): offsets (x, y), (z, far threshold) and
// strengths (gx, gy), (gz, -gx), (-gy, -gz), so that one 16-byte shared load
// gives two packed operands.  Far groups (one vote per four sources, as
// before) run entirely packed; near groups compute their displacements and
// kernel forms per source and pack them for the same accumulation.  Sums are
// kept per pair half (even / odd source) in FP32 blocks, then added in the
// mid-level FP32 sums and in FP64 as in uj_mixed_kernel.
typedef unsigned long long u64;
__device__ __forceinline__ u64 pk2(float lo, float hi)
{
    u64 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(u64 r, float& lo, float& hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
__device__ __forceinline__ u64 ffma2(u64 a, u64 b, u64 c)
{
    u64 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ u64 fmul2(u64 a, u64 b)
{
    u64 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 fsub2(u64 a, u64 b)
{
    u64 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// Packed source pair: px = (x0, x1, y0, y1), pz = (z0, z1, thr0, thr1),
// ga = (gx0, gx1, gy0, gy1), gb = (gz0, gz1, -gx0, -gx1), gc = (-gy0, -gy1, -gz0, -gz1).
struct __align__(16) PairX2 { float4 px, pz, ga, gb, gc; };

// Accumulate two pairs (packed halves) of one lane: U += G c, W += G gam, J' += Q c_i dx_j.
__device__ __forceinline__ void accum_x2(u64 dX, u64 dY, u64 dZ, u64 G, u64 Q, const PairX2& s, u64 (&u)[3],
                                         u64 (&w)[3], u64 (&jq)[8])
{
    const u64 GX = pk2(s.ga.x, s.ga.y), GY = pk2(s.ga.z, s.ga.w), GZ = pk2(s.gb.x, s.gb.y);
    const u64 NGX = pk2(s.gb.z, s.gb.w), NGY = pk2(s.gc.x, s.gc.y), NGZ = pk2(s.gc.z, s.gc.w);
    const u64 CX = ffma2(dY, GZ, fmul2(dZ, NGY));
    const u64 CY = ffma2(dZ, GX, fmul2(dX, NGZ));
    const u64 CZ = ffma2(dX, GY, fmul2(dY, NGX));
    u[0] = ffma2(G, CX, u[0]);
    u[1] = ffma2(G, CY, u[1]);
    u[2] = ffma2(G, CZ, u[2]);
    w[0] = ffma2(G, GX, w[0]);
    w[1] = ffma2(G, GY, w[1]);
    w[2] = ffma2(G, GZ, w[2]);
    const u64 BX = fmul2(Q, CX), BY = fmul2(Q, CY), BZ = fmul2(Q, CZ);
    jq[0] = ffma2(BX, dX, jq[0]);
    jq[1] = ffma2(BY, dX, jq[1]);
    jq[2] = ffma2(BZ, dX, jq[2]);
    jq[3] = ffma2(BX, dY, jq[3]);
    jq[4] = ffma2(BY, dY, jq[4]);
    jq[5] = ffma2(BZ, dY, jq[5]);
    jq[6] = ffma2(BX, dZ, jq[6]);
    jq[7] = ffma2(BY, dZ, jq[7]);
}

// Four sources (two packed pairs p0, p0 + 1) against this lane's target.
template <int K>
__device__ __forceinline__ void pair4_x2(u64 TX, u64 TY, u64 TZ, const float3& th, const float3& tl,
                                         const PairX2* __restrict__ pr, const SrcMixed* __restrict__ tile, int p0,
                                         u64 (&u)[3], u64 (&w)[3], u64 (&jq)[8])
{
    u64 dX[2], dY[2], dZ[2], R2[2];
    bool far = true;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float4 px = pr[p0 + h].px, pz = pr[p0 + h].pz;
        dX[h] = fsub2(TX, pk2(px.x, px.y));
        dY[h] = fsub2(TY, pk2(px.z, px.w));
        dZ[h] = fsub2(TZ, pk2(pz.x, pz.y));
        R2[h] = ffma2(dX[h], dX[h], ffma2(dY[h], dY[h], fmul2(dZ[h], dZ[h])));
        float r0, r1;
        upk2(R2[h], r0, r1);
        far = far && r0 > pz.z && r1 > pz.w;
    }
    if (__all_sync(0xffffffffu, far)) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float r0, r1;
            upk2(R2[h], r0, r1);
            u64 G, Q;
            if constexpr (singular_tail<K>()) {
                const u64 RS = pk2(frsqrt(r0), frsqrt(r1));
                const u64 RSS = fmul2(RS, RS);
                G = fmul2(RS, RSS);
                Q = fmul2(G, RSS);
            } else {   // Winckelmans: the regular form at every distance
                const float4 pz = pr[p0 + h].pz;
                float g0, q0, g1, q1;
                near_GQ<K>(r0 * pz.z, pz.z, g0, q0);
                near_GQ<K>(r1 * pz.w, pz.w, g1, q1);
                G = pk2(g0, g1);
                Q = pk2(q0, q1);
            }
            accum_x2(dX[h], dY[h], dZ[h], G, Q, pr[p0 + h], u, w, jq);
        }
    } else {
        // near group: double-float displacement and the full form, per source
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float ex[2], ey[2], ez[2], gg[2], qq[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int j = 2 * (p0 + h) + e;
                const float4 a = tile[j].a, b = tile[j].b;
                ex[e] = (th.x - a.x) + (tl.x - b.x);
                ey[e] = (th.y - a.y) + (tl.y - b.y);
                ez[e] = (th.z - a.z) + (tl.z - b.z);
                const float e2 = fmaf(ex[e], ex[e], fmaf(ey[e], ey[e], ez[e] * ez[e]));
                float G, Q;
                if constexpr (singular_tail<K>()) {
                    const float isig2 = b.w * b.w;
                    near_GQ<K>(e2 * isig2, isig2, G, Q);
                    const float isig3 = isig2 * b.w;
                    G *= isig3;
                    Q *= isig3;
                } else {
                    const float i2 = e ? pr[p0 + h].pz.w : pr[p0 + h].pz.z;
                    near_GQ<K>(e2 * i2, i2, G, Q);
                }
                const bool nz = e2 > 0.0f;
                gg[e] = nz ? G : 0.0f;
                qq[e] = nz ? Q : 0.0f;
            }
            accum_x2(pk2(ex[0], ex[1]), pk2(ey[0], ey[1]), pk2(ez[0], ez[1]), pk2(gg[0], gg[1]), pk2(qq[0], qq[1]),
                     pr[p0 + h], u, w, jq);
        }
    }
}

#ifndef VPM_UJ_X2_MIN_BLOCKS
#define VPM_UJ_X2_MIN_BLOCKS 5
#endif

template <int K>
__global__ void __launch_bounds__(UJ_THREADS, VPM_UJ_X2_MIN_BLOCKS)
uj_mixed_x2_kernel(int64_t nt, const TgtPos* __restrict__ tgt, int64_t ns_pad,
                   const SrcMixed* __restrict__ src, int64_t per_split, double* U, int64_t ldU,
                   double* J, int64_t ldJ, double* partial, int64_t nt_pad)
{
    __shared__ SrcMixed stage[UJ_WARPS][2][WT];
    __shared__ PairX2 prs[UJ_WARPS][2][WT / 2];
    __shared__ double acc64[14][UJ_THREADS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
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
    const float3 oh = make_float3(__shfl_sync(0xffffffffu, th.x, 0), __shfl_sync(0xffffffffu, th.y, 0),
                                  __shfl_sync(0xffffffffu, th.z, 0));
    const float3 ol = make_float3(__shfl_sync(0xffffffffu, tl.x, 0), __shfl_sync(0xffffffffu, tl.y, 0),
                                  __shfl_sync(0xffffffffu, tl.z, 0));
    const float3 to = valid ? make_float3((float)(tx - ox), (float)(ty - oy), (float)(tz - oz))
                            : make_float3(3.0e4f, 3.0e4f, 3.0e4f);
    float b2 = valid ? fmaf(to.x, to.x, fmaf(to.y, to.y, to.z * to.z)) : 0.0f;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, m));
    const float r2n = fmaxf(4.0f * b2, 1.0e-30f);
    const float sfar = s_far<K>();
    const u64 TX = pk2(to.x, to.x), TY = pk2(to.y, to.y), TZ = pk2(to.z, to.z);

#pragma unroll
    for (int k = 0; k < 14; k++) acc64[k][threadIdx.x] = 0.0;
    float mu[3] = {0.f, 0.f, 0.f}, mw[3] = {0.f, 0.f, 0.f}, mj[8];
#pragma unroll
    for (int k = 0; k < 8; k++) mj[k] = 0.f;
    u64 u[3], w[3], jq[8];
    const u64 Z0 = pk2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; k++) { u[k] = Z0; w[k] = Z0; }
#pragma unroll
    for (int k = 0; k < 8; k++) jq[k] = Z0;

    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    const int ntiles = (int)((s1 - s0) / WT);
    const SrcMixed* wsrc = src + s0 + lane;
    if (ntiles > 0) {
        SrcMixed* d = &stage[warp][0][lane];
        cp_async16(&d->a, &wsrc->a);
        cp_async16(&d->b, &wsrc->b);
        cp_async16(&d->gam, &wsrc->gam);
        cp_async_commit();
    }
    int in_block = 0, in_mid = 0;
    for (int it = 0; it < ntiles; it++) {
        const int buf = it & 1;
        if (it + 1 < ntiles) {
            const SrcMixed* g = wsrc + (int64_t)(it + 1) * WT;
            SrcMixed* d = &stage[warp][buf ^ 1][lane];
            cp_async16(&d->a, &g->a);
            cp_async16(&d->b, &g->b);
            cp_async16(&d->gam, &g->gam);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        {   // this lane's source into its half of the packed pair record
            const float4 a = stage[warp][buf][lane].a, b = stage[warp][buf][lane].b, g = stage[warp][buf][lane].gam;
            const float thr = singular_tail<K>() ? fmaxf(sfar * a.w, r2n) : b.w * b.w;
            const float px = (a.x - oh.x) + (b.x - ol.x), py = (a.y - oh.y) + (b.y - ol.y),
                        pz = (a.z - oh.z) + (b.z - ol.z);
            float* r = reinterpret_cast<float*>(&prs[warp][buf][lane >> 1]);
            const int e = lane & 1;
            r[0 + e] = px;  r[2 + e] = py;       // px
            r[4 + e] = pz;  r[6 + e] = thr;      // pz
            r[8 + e] = g.x; r[10 + e] = g.y;     // ga
            r[12 + e] = g.z; r[14 + e] = -g.x;   // gb
            r[16 + e] = -g.y; r[18 + e] = -g.z;  // gc
        }
        __syncwarp();
#pragma unroll (UJ_UNROLL)
        for (int p = 0; p < WT / 2; p += 2)
            pair4_x2<K>(TX, TY, TZ, th, tl, prs[warp][buf], stage[warp][buf], p, u, w, jq);
        if (++in_block == BLOCK_TILES) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                float a0, a1, b0, b1;
                upk2(u[k], a0, a1);
                upk2(w[k], b0, b1);
                mu[k] += a0 + a1;
                mw[k] += b0 + b1;
                u[k] = Z0;
                w[k] = Z0;
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float a0, a1;
                upk2(jq[k], a0, a1);
                mj[k] += a0 + a1;
                jq[k] = Z0;
            }
            in_block = 0;
            if (++in_mid == MID_BLOCKS) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    acc64[k][threadIdx.x] += (double)mu[k];
                    acc64[3 + k][threadIdx.x] += (double)mw[k];
                    mu[k] = 0.f;
                    mw[k] = 0.f;
                }
#pragma unroll
                for (int k = 0; k < 8; k++) { acc64[6 + k][threadIdx.x] += (double)mj[k]; mj[k] = 0.f; }
                in_mid = 0;
            }
        }
        __syncwarp();   // every lane is done with `buf` before it is refilled
    }
    double fU[3], fW[3], fJ[8];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float a0, a1, b0, b1;
        upk2(u[k], a0, a1);
        upk2(w[k], b0, b1);
        fU[k] = acc64[k][threadIdx.x] + ((double)mu[k] + ((double)a0 + (double)a1));
        fW[k] = acc64[3 + k][threadIdx.x] + ((double)mw[k] + ((double)b0 + (double)b1));
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        float a0, a1;
        upk2(jq[k], a0, a1);
        fJ[k] = acc64[6 + k][threadIdx.x] + ((double)mj[k] + ((double)a0 + (double)a1));
    }
    if (!valid) return;
    double j9[9];
#pragma unroll
    for (int k = 0; k < 8; k++) j9[k] = -3.0 * fJ[k];
    j9[8] = 3.0 * (fJ[0] + fJ[4]);
    j9[1] -= fW[2];
    j9[2] += fW[1];
    j9[3] += fW[2];
    j9[5] -= fW[0];
    j9[6] -= fW[1];
    j9[7] += fW[0];
    double acc[12] = {fU[0], fU[1], fU[2], j9[0], j9[1], j9[2], j9[3], j9[4], j9[5], j9[6], j9[7], j9[8]};
    write_uj(t, idx, acc, U, ldU, J, ldJ, partial, nt_pad);
}

// --------------------------------------------------------------- launcher
template <int K>
static cudaError_t launch_uj_k(const UJArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                               int64_t* launches)
{
    const int64_t ns_pad = round_up(a.ns, UJ_TILE);
    const int64_t nt_pad = round_up(a.nt, UJ_THREADS);
    const int nsplit = uj_num_splits(a.nt, a.ns, num_sms);
    const int64_t tiles = ns_pad / UJ_TILE;
    const int64_t per_split = ((tiles + nsplit - 1) / nsplit) * UJ_TILE;
    double* partial = nsplit > 1 ? w.partial : nullptr;
    const dim3 grid((unsigned)(nt_pad / UJ_THREADS), (unsigned)nsplit);
    const int pb = 256;
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(a.nt, a.xt, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    if (a.precision == 0) {
        SrcF64* src = (SrcF64*)w.src_pack;
        pack_src_f64<K><<<(unsigned)((ns_pad + pb - 1) / pb), pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs, src);
        uj_f64_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, ns_pad, src, per_split, a.U, a.ldU,
                                                       a.J, a.ldJ, partial, nt_pad);
    } else {
        SrcMixed* src = (SrcMixed*)w.src_pack;
        pack_src_mixed<K><<<(unsigned)((ns_pad + pb - 1) / pb), pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs,
                                                                             a.self ? tgt : nullptr, src);
#if VPM_UJ_F32X2
        uj_mixed_x2_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, ns_pad, src, per_split, a.U, a.ldU,
                                                            a.J, a.ldJ, partial, nt_pad);
#elif VPM_UJ_TPL == 2
        const dim3 grid2((unsigned)((a.nt + 2 * UJ_THREADS - 1) / (2 * UJ_THREADS)), (unsigned)nsplit);
        uj_mixed2_kernel<K><<<grid2, UJ_THREADS, 0, st>>>(a.nt, tgt, ns_pad, src, per_split, a.U, a.ldU,
                                                           a.J, a.ldJ, partial, nt_pad);
#else
        uj_mixed_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, ns_pad, src, per_split, a.U, a.ldU,
                                                         a.J, a.ldJ, partial, nt_pad);
#endif
    }
    *launches += 2;
    if (partial) {
        uj_reduce<<<(unsigned)((a.nt + pb - 1) / pb), pb, 0, st>>>(a.nt, nsplit, partial, nt_pad, tgt, a.U,
                                                                 a.ldU, a.J, a.ldJ);
        *launches += 1;
    }
    return cudaGetLastError();
}

cudaError_t launch_uj(const UJArgs& a, const Workspace& w, int num_sms, cudaStream_t st, int64_t* launches)
{
    if (a.nt <= 0 || a.ns <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_uj_k<K_SING>(a, w, num_sms, st, launches);
    case K_GAUS: return launch_uj_k<K_GAUS>(a, w, num_sms, st, launches);
    case K_GAUSERF: return launch_uj_k<K_GAUSERF>(a, w, num_sms, st, launches);
    case K_WNKLMNS: return launch_uj_k<K_WNKLMNS>(a, w, num_sms, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
