// estr.cu -- SFS vortex-stretching pass Estr (src/FLOWVPM_subfilterscale_models.jl:16-92).
//
// The reference adds, for every non-static target t and non-static source s,
//     SFS_t += zeta(r/sigma_s)/sigma_s^3 * (J_t - J_s)^T Gamma_s      (transposed)
// This is evaluated in the exactly equivalent factored form
//     SFS_t += J_t^T Zg_t - Zv_t,   Zg_t = sum_s z_ts Gamma_s,  Zv_t = sum_s z_ts v_s,
// with z_ts = zeta(r/sigma_s)/sigma_s^3 and v_s = J_s^T Gamma_s (J_s Gamma_s for
// the classic scheme), so a source carries 10 numbers instead of 16 and a pair
// costs about 25 flop.  The self pair, which the reference includes but which
// contributes exactly zero there, is excluded by index (in the factored form
// its two terms would only cancel to rounding).  Static sources are packed with
// zero strength; static targets are left untouched.  Targets run in Morton
// order (order.cu) like the UJ kernels.  The FP64 kernel keeps the reference's
// zeta formula; the mixed kernel uses FP32 pair math on per-warp FP32 offsets
// (see uj.cu) and FP64 accumulation of FP32 blocks, and skips every pair at
// r = 0 (the self pair, and coincident particles, whose J are equal so that
// their reference term is zero; in the factored form their two terms would
// only cancel to FP32 rounding, at the largest weight zeta(0)).
#include "dyn_math.cuh"
#include "estr_tiles.cuh"
#include "internal.h"
#include "vpm_math.cuh"

namespace vpm {

static inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// Sources summed in plain FP32 before a compensated add.  J_t^T Zg - Zv is a
// difference of two sums far larger than itself (by |J| / |J_t - J_s| and by
// the cancellation of neighbours on either side of a target), so their FP32
// rounding is what limits the mixed Estr; sums of 8 added with compensation
// bring it from ~1e-5 to ~2e-6 of max |SFS| on a smooth field.
constexpr int ESTR_SUB = 8;

static_assert(UJ_BLOCK % ESTR_SUB == 0, "whole sub-blocks");

constexpr int EWT = EST_TILE;   // sources per tile of the mixed kernel's streams (one per lane)

size_t estr_src_pack_bytes(int64_t ns, int precision)
{
    const int64_t n = round_up(ns, UJ_TILE);
    // FP32-comp: the records, then two float4 per 32-source tile (estr_tile_boxes)
    return precision ? (size_t)n * sizeof(SrcEstrDF) + (size_t)(n / EWT) * 2 * sizeof(float4)
                     : (size_t)n * sizeof(SrcEstrF64);
}

// v = J^T Gamma (transposed) or J Gamma (classic); J column-major 3x3.
__device__ __forceinline__ void stretch_vec(const double* J, double gx, double gy, double gz,
                                            bool transposed, double& vx, double& vy, double& vz)
{
    if (transposed) {
        vx = J[0] * gx + J[1] * gy + J[2] * gz;
        vy = J[3] * gx + J[4] * gy + J[5] * gz;
        vz = J[6] * gx + J[7] * gy + J[8] * gz;
    } else {
        vx = J[0] * gx + J[3] * gy + J[6] * gz;
        vy = J[1] * gx + J[4] * gy + J[7] * gz;
        vz = J[2] * gx + J[5] * gy + J[8] * gz;
    }
}

template <int K>
__global__ void pack_estr_mixed(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
                                const double* __restrict__ gs, const double* __restrict__ sgs,
                                const double* __restrict__ Js, int64_t ldJs,
                                const uint8_t* __restrict__ static_s, bool transposed,
                                const TgtPos* __restrict__ order, SrcEstrDF* __restrict__ out,
                                float4* __restrict__ box)
{
    // with `order` (sources = targets) the pack follows the targets' Morton order
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= ns_pad) return;   // whole warps: ns_pad is a multiple of 32
    SrcEstrDF p;
    if (o < ns) {
        const int64_t i = order ? (int64_t)order[o].idx : o;
        const double isig = 1.0 / sgs[i];
        const double isig2 = isig * isig;
        const double x = xs[3 * i], y = xs[3 * i + 1], z = xs[3 * i + 2];
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        p.a = make_float4(xh, yh, zh, (float)isig2);
        p.b = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
        const bool off = static_s && static_s[i];
        const double k = off ? 0.0 : zeta_norm(K) * isig2 * isig;
        const double gx = gs[3 * i], gy = gs[3 * i + 1], gz = gs[3 * i + 2];
        double vx = 0.0, vy = 0.0, vz = 0.0;   // the zeta field (Js null) needs no v
        if (Js) stretch_vec(Js + i * ldJs, gx, gy, gz, transposed, vx, vy, vz);
        p.g = make_float4((float)(k * gx), (float)(k * gy), (float)(k * gz), 0.f);
        p.v = make_float4((float)(k * vx), (float)(k * vy), (float)(k * vz), 0.f);
    } else {   // padding: far away, no strength
        p.a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
        p.b = make_float4(0.f, 0.f, 0.f, 0.f);
        p.g = p.v = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    out[o] = p;
    estr_tile_box(o, ns, p.a.x, p.a.y, p.a.z, p.a.w, box);
}

template <int K>
__global__ void pack_estr_f64(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
                              const double* __restrict__ gs, const double* __restrict__ sgs,
                              const double* __restrict__ Js, int64_t ldJs,
                              const uint8_t* __restrict__ static_s, bool transposed,
                              SrcEstrF64* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ns_pad) return;
    SrcEstrF64 p;
    if (i < ns) {
        const bool off = static_s && static_s[i];
        const double gx = off ? 0.0 : gs[3 * i], gy = off ? 0.0 : gs[3 * i + 1], gz = off ? 0.0 : gs[3 * i + 2];
        double vx = 0.0, vy = 0.0, vz = 0.0;
        if (Js) stretch_vec(Js + i * ldJs, gx, gy, gz, transposed, vx, vy, vz);
        p.xy = make_double2(xs[3 * i], xs[3 * i + 1]);
        p.z_isig = make_double2(xs[3 * i + 2], 1.0 / sgs[i]);
        p.gxy = make_double2(gx, gy);
        p.gz_vx = make_double2(gz, vx);
        p.vyz = make_double2(vy, vz);
    } else {
        p.xy = make_double2(0.0, 0.0);
        p.z_isig = make_double2(0.0, 1.0);
        p.gxy = p.gz_vx = p.vyz = make_double2(0.0, 0.0);
    }
    out[i] = p;
}

// SFS contribution J_t^T Zg - Zv  (or J_t Zg - Zv), FP64.
__device__ __forceinline__ void estr_combine(const double* Jt, const double (&zg)[3], const double (&zv)[3],
                                             bool transposed, double (&out)[3])
{
    double sx, sy, sz;
    stretch_vec(Jt, zg[0], zg[1], zg[2], transposed, sx, sy, sz);
    out[0] = sx - zv[0];
    out[1] = sy - zv[1];
    out[2] = sz - zv[2];
}

__device__ __forceinline__ void write_estr(int64_t t, int64_t idx, const double (&o)[3], double* SFS, int64_t ldS,
                                           double* partial, int64_t nt_pad)
{
    if (partial) {
        double* p = partial + (int64_t)blockIdx.y * 3 * nt_pad + t;
        p[0] = o[0]; p[nt_pad] = o[1]; p[2 * nt_pad] = o[2];
    } else {
        SFS[idx * ldS] += o[0]; SFS[idx * ldS + 1] += o[1]; SFS[idx * ldS + 2] += o[2];
    }
}

__global__ void estr_reduce(int64_t nt, int nsplit, const double* __restrict__ partial, int64_t nt_pad,
                            const TgtPos* __restrict__ tgt, const uint8_t* __restrict__ static_t,
                            double* SFS, int64_t ldS)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int64_t i = tgt[t].idx;
    if (static_t && static_t[i]) return;
    for (int k = 0; k < 3; k++) {
        double s = 0.0;
        for (int sp = 0; sp < nsplit; sp++) s += partial[((int64_t)sp * 3 + k) * nt_pad + t];
        SFS[i * ldS + k] += s;
    }
}

// With ZETA the kernels evaluate zeta_direct instead (src/FLOWVPM_viscous.jl:467-488):
// W_t += sum_s zeta(r/sigma_s)/sigma_s^3 Gamma_s over every source and target, the
// self pair included, written to the SFS output.
template <int K, bool ZETA>
__global__ void __launch_bounds__(UJ_THREADS)
estr_f64_kernel(int64_t nt, const TgtPos* __restrict__ tgt, const double* __restrict__ Jt, int64_t ldJt,
                const uint8_t* __restrict__ static_t, int64_t ns_pad, const SrcEstrF64* __restrict__ src,
                int64_t per_split, bool self, bool transposed, double* SFS, int64_t ldS,
                double* partial, int64_t nt_pad)
{
    __shared__ SrcEstrF64 tile[UJ_TILE];
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    double tx = 1.0e3, ty = 1.0e3, tz = 1.0e3;
    int64_t idx = -1;
    if (t < nt) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const bool valid = t < nt && (ZETA || !(static_t && static_t[idx]));
    const int64_t self_idx = (self && !ZETA) ? idx : -1;
    double zg[3] = {0.0, 0.0, 0.0}, zv[3] = {0.0, 0.0, 0.0};
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < UJ_TILE; j++) {
            const SrcEstrF64& p = tile[j];
            if (base + j == self_idx) continue;
            const double dx = p.xy.x - tx, dy = p.xy.y - ty, dz = p.z_isig.x - tz;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            const double isig = p.z_isig.y;
            const double z = zeta_f64<K>(r * isig) * isig * isig * isig;
            zg[0] += z * p.gxy.x; zg[1] += z * p.gxy.y; zg[2] += z * p.gz_vx.x;
            if constexpr (!ZETA) { zv[0] += z * p.gz_vx.y; zv[1] += z * p.vyz.x; zv[2] += z * p.vyz.y; }
        }
    }
    if (!valid) return;
    double o[3];
    if constexpr (ZETA) { o[0] = zg[0]; o[1] = zg[1]; o[2] = zg[2]; }
    else estr_combine(Jt + idx * ldJt, zg, zv, transposed, o);
    write_estr(t, idx, o, SFS, ldS, partial, nt_pad);
}

// 16-byte asynchronous global->shared copy (LDGSTS), L2-cached.
__device__ __forceinline__ void ecp_async16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void ecp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void ecp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int ESTR_FLUSH_TILES = 8;      // evaluated warp tiles between FP64 adds (256 sources)

// The mixed Estr.  Each warp streams the sources on its own, 32 per tile,
// double-buffered with cp.async (no block-wide barrier); the loading lane
// converts its source to an FP32 offset from the warp's first target with
// FP32 double-float arithmetic (df_offset: rounded once), and each target's
// own offset is formed by the same operations, so that the self pair and
// coincident particles have
// r^2 == 0 exactly (they are skipped: their terms would only cancel to FP32
// rounding, at the largest weight).  For the Gaussian kernels the terms past
// zeta_skip_s (zeta/zeta(0) < 1e-13: below the FP32 resolution of the sums) are
// skipped at three levels: a tile whose pack box is out of reach of the warp's
// targets is not loaded (TileWalk); a loaded tile is skipped when every one of its
// sources is out of reach of the warp's target box; an 8-source sub-block when
// every pair of the warp is.  Sums: 8-source FP32 partials added with
// compensation (comp_add), FP64 every ESTR_FLUSH_TILES evaluated tiles.
// With DZ (the weight difference of the dynamic procedure's test filter,
// dynamic.cu) each weight zeta~(r, sigma_s) is replaced by
// zeta~(r, alpha sigma_s) - zeta~(r, sigma_s) = zeta~(r, sigma_s) (ratio - 1),
// ratio - 1 from zeta_ratio_m1 with the factors fd = (alpha^-3 - 1, alpha^-3, alpha^-2 - 1).
template <int K, bool ZETA, bool DZ = false>
__global__ void __launch_bounds__(UJ_THREADS)
estr_mixed_kernel(int64_t nt, const TgtPos* __restrict__ tgt, const double* __restrict__ Jt, int64_t ldJt,
                  const uint8_t* __restrict__ static_t, int64_t ns_pad, const SrcEstrDF* __restrict__ src,
                  const float4* __restrict__ box, int64_t per_split, bool self, bool transposed, double* SFS,
                  int64_t ldS, double* partial, int64_t nt_pad, float3 fd = make_float3(0.f, 0.f, 0.f))
{
    __shared__ SrcEstrDF stage[UJ_WARPS][2][EWT];
    __shared__ float4 offs[UJ_WARPS][2][EWT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    int64_t idx = -1;
    if (t < nt) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const bool valid = t < nt && (ZETA || !(static_t && static_t[idx]));
    // warp origin: lane 0's target as a double-float
    const double ox = __shfl_sync(0xffffffffu, tx, 0), oy = __shfl_sync(0xffffffffu, ty, 0),
                 oz = __shfl_sync(0xffffffffu, tz, 0);
    const float3 oh = make_float3((float)ox, (float)oy, (float)oz);
    const float3 ol = make_float3((float)(ox - (double)oh.x), (float)(oy - (double)oh.y), (float)(oz - (double)oh.z));
    // the target's offset by the same FP32 double-float operations as the sources' (below);
    // padding lanes sit at the origin
    float3 to = make_float3(0.f, 0.f, 0.f);
    if (t < nt) {
        const float3 th = make_float3((float)tx, (float)ty, (float)tz);
        const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y),
                                      (float)(tz - (double)th.z));
        to = make_float3(df_offset(th.x, tl.x, oh.x, ol.x), df_offset(th.y, tl.y, oh.y, ol.y),
                         df_offset(th.z, tl.z, oh.z, ol.z));
    }
    // the warp's target boxes: offsets (for the per-source test of a tile) and FP32
    // positions of its targets (for the tile boxes of the pack); [0], [1] = offsets low,
    // high; [2], [3] = positions low, high (empty without a target)
    __shared__ float4 wbox[UJ_WARPS][4];
    {
        float v[12] = {to.x, to.y, to.z, -to.x, -to.y, -to.z};
        const bool real = t < nt;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float h = (float)(k == 0 ? tx : k == 1 ? ty : tz);
            v[6 + k] = real ? h : 3.0e38f;
            v[9 + k] = real ? -h : 3.0e38f;
        }
#pragma unroll
        for (int m = 16; m > 0; m >>= 1)
#pragma unroll
            for (int k = 0; k < 12; k++) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], m));
        if (lane == 0) {
            wbox[warp][0] = make_float4(v[0], v[1], v[2], 0.f);
            wbox[warp][1] = make_float4(-v[3], -v[4], -v[5], 0.f);
            wbox[warp][2] = make_float4(v[6], v[7], v[8], 0.f);
            wbox[warp][3] = make_float4(-v[9], -v[10], -v[11], 0.f);
        }
        __syncwarp();
    }
    double zg[3] = {0.0, 0.0, 0.0}, zv[3] = {0.0, 0.0, 0.0};
    float sg[3] = {0.f, 0.f, 0.f}, cg[3] = {0.f, 0.f, 0.f}, sv[3] = {0.f, 0.f, 0.f}, cv[3] = {0.f, 0.f, 0.f};
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    const int ntiles = (int)((s1 - s0) / EWT);
    const SrcEstrDF* wsrc = src + s0 + lane;
    // the split's tiles within reach of the warp's targets, 32 tiles per ballot
    TileWalk walk;
    walk.init(ntiles);
    int cur = walk.next<K>(box + 2 * (s0 / EWT), wbox[warp][2], wbox[warp][3], lane);
    if (cur >= 0) {
        SrcEstrDF* d = &stage[warp][0][lane];
        const SrcEstrDF* gp = wsrc + (int64_t)cur * EWT;
        ecp_async16(&d->a, &gp->a); ecp_async16(&d->b, &gp->b);
        ecp_async16(&d->g, &gp->g); ecp_async16(&d->v, &gp->v);
        ecp_commit();
    }
    int in_flush = 0, buf = 0;
    while (cur >= 0) {
        const int nxt = walk.next<K>(box + 2 * (s0 / EWT), wbox[warp][2], wbox[warp][3], lane);
        if (nxt >= 0) {
            const SrcEstrDF* gp = wsrc + (int64_t)nxt * EWT;
            SrcEstrDF* d = &stage[warp][buf ^ 1][lane];
            ecp_async16(&d->a, &gp->a); ecp_async16(&d->b, &gp->b);
            ecp_async16(&d->g, &gp->g); ecp_async16(&d->v, &gp->v);
            ecp_commit();
            ecp_wait<1>();
        } else {
            ecp_wait<0>();
        }
        __syncwarp();
        bool beyond;
        {   // this lane's source: FP32 offset, and whether it is out of reach of the whole target box
            const float4 a = stage[warp][buf][lane].a, b = stage[warp][buf][lane].b;
            const float px = df_offset(a.x, b.x, oh.x, ol.x), py = df_offset(a.y, b.y, oh.y, ol.y),
                        pz = df_offset(a.z, b.z, oh.z, ol.z);
            offs[warp][buf][lane] = make_float4(px, py, pz, a.w);
            const float4 lo = wbox[warp][0], hi = wbox[warp][1];
            const float ex = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.0f);
            const float ey = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.0f);
            const float ez = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.0f);
            beyond = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) * a.w > zeta_skip_s<K>();
        }
        __syncwarp();
        if (!(zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, beyond))) {
#pragma unroll 1
            for (int sub = 0; sub < EWT; sub += ESTR_SUB) {
                float sv8[ESTR_SUB], r28[ESTR_SUB];
                bool far = true;
#pragma unroll
                for (int jj = 0; jj < ESTR_SUB; jj++) {
                    const float4 h = offs[warp][buf][sub + jj];
                    const float dx = to.x - h.x, dy = to.y - h.y, dz = to.z - h.z;
                    r28[jj] = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    sv8[jj] = r28[jj] * h.w;
                    far = far && sv8[jj] > zeta_skip_s<K>();
                }
                if (zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, far)) continue;
                float fg[3] = {0.f, 0.f, 0.f}, fv[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int jj = 0; jj < ESTR_SUB; jj++) {
                    const int j = sub + jj;
                    float z = zhat_f32<K>(sv8[jj]);
                    if constexpr (DZ) z *= zeta_ratio_m1<K>(sv8[jj], fd);
                    if constexpr (!ZETA) z = (r28[jj] == 0.0f) ? 0.0f : z;
                    const float4 g = stage[warp][buf][j].g;
                    fg[0] = fmaf(z, g.x, fg[0]);
                    fg[1] = fmaf(z, g.y, fg[1]);
                    fg[2] = fmaf(z, g.z, fg[2]);
                    if constexpr (!ZETA) {
                        const float4 v = stage[warp][buf][j].v;
                        fv[0] = fmaf(z, v.x, fv[0]);
                        fv[1] = fmaf(z, v.y, fv[1]);
                        fv[2] = fmaf(z, v.z, fv[2]);
                    }
                }
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    comp_add(sg[k], cg[k], fg[k]);
                    if constexpr (!ZETA) comp_add(sv[k], cv[k], fv[k]);
                }
            }
            // skipped tiles add nothing, so only the tiles taken count towards a flush
            if (++in_flush == ESTR_FLUSH_TILES) {
                in_flush = 0;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    zg[k] += (double)sg[k] + (double)cg[k];
                    sg[k] = cg[k] = 0.f;
                    if constexpr (!ZETA) {
                        zv[k] += (double)sv[k] + (double)cv[k];
                        sv[k] = cv[k] = 0.f;
                    }
                }
            }
        }
        __syncwarp();   // every lane is done with `buf` before it is refilled
        cur = nxt;
        buf ^= 1;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        zg[k] += (double)sg[k] + (double)cg[k];
        if constexpr (!ZETA) zv[k] += (double)sv[k] + (double)cv[k];
    }
    if (!valid) return;
    double o[3];
    if constexpr (ZETA) { o[0] = zg[0]; o[1] = zg[1]; o[2] = zg[2]; }
    else estr_combine(Jt + idx * ldJt, zg, zv, transposed, o);
    write_estr(t, idx, o, SFS, ldS, partial, nt_pad);
}

template <int K>
static cudaError_t launch_estr_k(const EstrArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
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
    const unsigned pgrid = (unsigned)((ns_pad + pb - 1) / pb);
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(a.nt, a.xt, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    const uint8_t* static_s = a.zeta ? nullptr : a.static_s;
    const uint8_t* static_t = a.zeta ? nullptr : a.static_t;
    if (a.dz_alpha > 0.0 && a.precision == 0) return cudaErrorInvalidValue;   // FP32-comp only
    if (a.precision == 0) {
        SrcEstrF64* src = (SrcEstrF64*)w.src_pack;
        pack_estr_f64<K><<<pgrid, pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs, a.zeta ? nullptr : a.Js, a.ldJs,
                                                static_s, a.transposed, src);
        if (a.zeta)
            estr_f64_kernel<K, true><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad, src,
                                                                  per_split, a.self, a.transposed, a.SFS, a.ldS,
                                                                  partial, nt_pad);
        else
            estr_f64_kernel<K, false><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad, src,
                                                                   per_split, a.self, a.transposed, a.SFS, a.ldS,
                                                                   partial, nt_pad);
    } else {
        SrcEstrDF* src = (SrcEstrDF*)w.src_pack;
        float4* box = (float4*)(src + ns_pad);   // the tile boxes follow the records
        pack_estr_mixed<K><<<pgrid, pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs, a.zeta ? nullptr : a.Js, a.ldJs,
                                                  static_s, a.transposed, a.self ? tgt : nullptr, src, box);
        if (a.zeta)
            estr_mixed_kernel<K, true><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad, src,
                                                                    box, per_split, a.self, a.transposed, a.SFS,
                                                                    a.ldS, partial, nt_pad);
        else if (a.dz_alpha > 0.0) {
            const double al = a.dz_alpha;
            const float3 fd = make_float3((float)(1.0 / (al * al * al) - 1.0), (float)(1.0 / (al * al * al)),
                                          (float)(1.0 / (al * al) - 1.0));
            estr_mixed_kernel<K, false, true><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad,
                                                                           src, box, per_split, a.self, a.transposed,
                                                                           a.SFS, a.ldS, partial, nt_pad, fd);
        } else
            estr_mixed_kernel<K, false><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad, src,
                                                                     box, per_split, a.self, a.transposed, a.SFS,
                                                                     a.ldS, partial, nt_pad);
    }
    *launches += 2;
    if (partial) {
        estr_reduce<<<(unsigned)((a.nt + pb - 1) / pb), pb, 0, st>>>(a.nt, nsplit, partial, nt_pad, tgt,
                                                                   static_t, a.SFS, a.ldS);
        *launches += 1;
    }
    return cudaGetLastError();
}

cudaError_t launch_estr(const EstrArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                        int64_t* launches)
{
    if (a.nt <= 0 || a.ns <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_estr_k<K_SING>(a, w, num_sms, st, launches);
    case K_GAUS: return launch_estr_k<K_GAUS>(a, w, num_sms, st, launches);
    case K_GAUSERF: return launch_estr_k<K_GAUSERF>(a, w, num_sms, st, launches);
    case K_WNKLMNS: return launch_estr_k<K_WNKLMNS>(a, w, num_sms, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
