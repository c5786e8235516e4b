// estr_adjoint.cu -- reverse mode of the SFS stretching pass Estr
// (src/FLOWVPM_subfilterscale_models.jl:16-92), which the reference's rrule
// leaves unimplemented ("SFS pullback not implemented yet!",
// src/FLOWVPM_rrules.jl:153-157).
//
// Forward, over non-static targets t and non-static sources s != t:
//     SFS_t = sum_s z_ts S_ts,   z_ts = zeta(r/sigma_s)/sigma_s^3,
//     S_ts = (J_t - J_s)^T Gamma_s  (transposed)  or  (J_t - J_s) Gamma_s  (classic).
// With Sbar_t = dL/dSFS_t and M = J as a 3x3 matrix (M[a][b] = J[a + 3b]):
//     w_ts = Sbar_t . S_ts = Gamma_s . a_t - v_s . Sbar_t,
//     a_t = M_t Sbar_t, v_s = M_s^T Gamma_s   (transposed; classic: a_t = M_t^T Sbar_t,
//                                              v_s = M_s Gamma_s, the forward's payload)
// and, with kappa = (zeta'(rho)/rho)/zeta(rho) (-1 Gaussian-erf, -3 rho Gaussian,
// -7/(1 + rho^2) Winckelmans, 0 singular):
//     dL/dx_t    += sum_s w z_ts kappa / sigma_s^2 dx_ts          (dx_ts = x_t - x_s)
//     dL/dJ_t    += Zg_t Sbar_t^T  (classic: Sbar_t Zg_t^T),  Zg_t = sum_s z_ts Gamma_s
//     dL/dx_s    -= sum_t w z_ts kappa / sigma_s^2 dx_ts
//     dL/dsigma_s += -sum_t w z_ts (rho^2 kappa + 3) / sigma_s
//     dL/dGamma_s += A_s - M_s B_s  (classic: A_s - M_s^T B_s)
//     dL/dJ_s    -= Gamma_s B_s^T  (classic: B_s Gamma_s^T)
// with A_s = sum_t z_ts a_t and B_s = sum_t z_ts Sbar_t.
//
// Two passes, each over all pairs with one particle per thread and no atomics,
// so the results are deterministic: pass 1 with the targets in the lanes
// (Zg_t and the x_t sum), pass 2 with the sources in the lanes (the ten
// source-side sums; z_ts depends on sigma_s only, so every 1/sigma_s factor is a
// lane constant applied once at the end).  Particles run in Morton order
// (order.cu) in both roles; sums go to FP64 partial arrays per source split,
// and an epilogue kernel per pass adds the splits in order and forms the
// outputs.  FP64 follows the formulas above pair by pair, coincident pairs
// (r = 0, s != t) included as in the forward; FP32-comp takes the forward mixed
// Estr's arithmetic (per-warp streaming, FP32 offsets from a per-warp
// double-float origin, tile and sub-block skips past the kernel's reach,
// compensated 8-pair sub-sums, FP64 across tiles) and skips pairs at r = 0, as
// that forward does.
#include "estr_tiles.cuh"
#include "internal.h"
#include "vpm_math.cuh"

namespace vpm {

static inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

namespace {

constexpr int EA_SUB = 8;           // pairs summed in plain FP32 before a compensated add
constexpr int NACC1 = 6;            // pass 1 sums: Zg[3], X[3]
constexpr int NACC2 = 10;           // pass 2 sums: A[3], B[3], X[3], Sg

// Pass-1 payload (a source): FP64 position, 1/sigma (FP64) or 1/sigma^2
// (mixed), Gamma and v; in the mixed pack Gamma and v carry ZNORM/sigma^3.
struct __align__(16) EA1F64 { double x, y, z, isig, gx, gy, gz, vx, vy, vz; };
struct __align__(16) EA1Mx { float4 a, b, g, v; };        // a = (x_hi, isig2), b = (x_lo, 0)
// Pass-2 payload (a target): FP64 position, a_t and Sbar_t.
struct __align__(16) EA2F64 { double x, y, z, pad, ax, ay, az, sx, sy, sz; };
struct __align__(16) EA2Mx { float4 h, l, a, sb; };       // h = (x_hi, 0), l = (x_lo, 0)

// M v (ab = false) or M^T v (ab = true) for J column-major 3x3 (M[a][b] = J[a + 3b]).
__device__ __forceinline__ void mat_vec(const double* J, double x0, double x1, double x2, bool transpose, double (&o)[3])
{
    if (transpose) {
        o[0] = J[0] * x0 + J[1] * x1 + J[2] * x2;
        o[1] = J[3] * x0 + J[4] * x1 + J[5] * x2;
        o[2] = J[6] * x0 + J[7] * x1 + J[8] * x2;
    } else {
        o[0] = J[0] * x0 + J[3] * x1 + J[6] * x2;
        o[1] = J[1] * x0 + J[4] * x1 + J[7] * x2;
        o[2] = J[2] * x0 + J[5] * x1 + J[8] * x2;
    }
}

// kappa(rho) = (zeta'(rho)/rho)/zeta(rho) as a function of s = rho^2
template <int K>
__device__ __forceinline__ double kappa_f64(double s)
{
    if constexpr (K == K_GAUSERF) return -1.0;
    else if constexpr (K == K_GAUS) return -3.0 * sqrt(s);
    else if constexpr (K == K_WNKLMNS) return -7.0 / (1.0 + s);
    else return 0.0;
}
template <int K>
__device__ __forceinline__ float kappa_f32(float s)
{
    if constexpr (K == K_GAUSERF) return -1.0f;
    else if constexpr (K == K_GAUS) return -3.0f * sqrtf(s);
    else if constexpr (K == K_WNKLMNS) return -7.0f * frcp(1.0f + s);
    else return 0.0f;
}

// ------------------------------------------------------------------- packing
// Sources (pass 1) and targets (pass 2) in the targets' Morton order; static
// particles carry zero Gamma, v, a and Sbar (they take no part in Estr).
template <int K>
__global__ void ea_pack(int64_t n, int64_t n_pad, const TgtPos* __restrict__ order, const double* __restrict__ x,
                        const double* __restrict__ gam, const double* __restrict__ sig, const double* __restrict__ J,
                        const uint8_t* __restrict__ st, const double* __restrict__ Sbar, bool transposed, bool mixed,
                        void* __restrict__ p1, void* __restrict__ p2, float4* __restrict__ box)
{
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n_pad) return;
    double px = 0.0, py = 0.0, pz = 0.0, isig = 1.0, G[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0};
    double a[3] = {0.0, 0.0, 0.0}, sb[3] = {0.0, 0.0, 0.0};
    if (o < n) {
        const int64_t i = order[o].idx;
        px = x[3 * i]; py = x[3 * i + 1]; pz = x[3 * i + 2];
        isig = 1.0 / sig[i];
        if (!(st && st[i])) {
            for (int k = 0; k < 3; k++) { G[k] = gam[3 * i + k]; sb[k] = Sbar[3 * i + k]; }
            mat_vec(J + 9 * i, G[0], G[1], G[2], transposed, v);        // the forward's v_s
            mat_vec(J + 9 * i, sb[0], sb[1], sb[2], !transposed, a);    // a_t
        }
    } else {   // padding: far away, nothing carried
        px = py = pz = 1.0e6;
    }
    if (!mixed) {
        EA1F64 s1 = {px, py, pz, isig, G[0], G[1], G[2], v[0], v[1], v[2]};
        EA2F64 s2 = {px, py, pz, 0.0, a[0], a[1], a[2], sb[0], sb[1], sb[2]};
        ((EA1F64*)p1)[o] = s1;
        ((EA2F64*)p2)[o] = s2;
    } else {
        const double k = zeta_norm(K) * isig * isig * isig;
        const float xh = (float)px, yh = (float)py, zh = (float)pz;
        const float4 lo = make_float4((float)(px - (double)xh), (float)(py - (double)yh), (float)(pz - (double)zh), 0.f);
        EA1Mx s1;
        s1.a = make_float4(xh, yh, zh, (float)(isig * isig));
        s1.b = lo;
        s1.g = make_float4((float)(k * G[0]), (float)(k * G[1]), (float)(k * G[2]), 0.f);
        s1.v = make_float4((float)(k * v[0]), (float)(k * v[1]), (float)(k * v[2]), 0.f);
        EA2Mx s2;
        s2.h = make_float4(xh, yh, zh, 0.f);
        s2.l = lo;
        s2.a = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
        s2.sb = make_float4((float)sb[0], (float)sb[1], (float)sb[2], 0.f);
        ((EA1Mx*)p1)[o] = s1;
        ((EA2Mx*)p2)[o] = s2;
        estr_tile_box(o, n, xh, yh, zh, s1.a.w, box);   // whole warps (n_pad is a multiple of 32)
    }
}

__device__ __forceinline__ void write_partial(double* partial, int nacc, int64_t nt_pad, int64_t t, const double* acc)
{
    double* p = partial + (int64_t)blockIdx.y * nacc * nt_pad + t;
    for (int k = 0; k < nacc; k++) p[k * nt_pad] = acc[k];
}

// ------------------------------------------------------------------ FP64 passes
// Pass 1: lanes are targets t (Morton position), the tile holds sources.
template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
ea1_f64(int64_t n, const TgtPos* __restrict__ tgt, const EA2F64* __restrict__ self, int64_t n_pad,
        const EA1F64* __restrict__ src, int64_t per_split, double* __restrict__ partial)
{
    __shared__ EA1F64 tile[UJ_TILE];
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const EA2F64 me = self[t < n ? t : n_pad - 1];     // a_t, Sbar_t (zero for static targets)
    double acc[NACC1] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int64_t s0 = (int64_t)blockIdx.y * per_split, s1 = min(s0 + per_split, n_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < UJ_TILE; j++) {
            const EA1F64& p = tile[j];
            if (base + j == t) continue;
            const double dx = me.x - p.x, dy = me.y - p.y, dz = me.z - p.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double r = sqrt(r2);
            const double z = zeta_f64<K>(r * p.isig) * p.isig * p.isig * p.isig;
            const double w = p.gx * me.ax + p.gy * me.ay + p.gz * me.az - (p.vx * me.sx + p.vy * me.sy + p.vz * me.sz);
            acc[0] += z * p.gx; acc[1] += z * p.gy; acc[2] += z * p.gz;
            const double c = w * z * kappa_f64<K>(r2 * p.isig * p.isig) * p.isig * p.isig;
            acc[3] += c * dx; acc[4] += c * dy; acc[5] += c * dz;
        }
    }
    if (t < n) write_partial(partial, NACC1, n_pad, t, acc);
}

// Pass 2: lanes are sources s (Morton position), the tile holds targets.
template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
ea2_f64(int64_t n, const EA1F64* __restrict__ self, int64_t n_pad, const EA2F64* __restrict__ src,
        int64_t per_split, double* __restrict__ partial)
{
    __shared__ EA2F64 tile[UJ_TILE];
    const int64_t s = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const EA1F64 me = self[s < n ? s : n_pad - 1];     // Gamma_s, v_s (zero for static sources)
    double acc[NACC2];
#pragma unroll
    for (int k = 0; k < NACC2; k++) acc[k] = 0.0;
    const double isig2 = me.isig * me.isig;
    const int64_t s0 = (int64_t)blockIdx.y * per_split, s1 = min(s0 + per_split, n_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < UJ_TILE; j++) {
            const EA2F64& p = tile[j];
            if (base + j == s) continue;
            const double dx = me.x - p.x, dy = me.y - p.y, dz = me.z - p.z;   // x_s - x_t
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double ss = r2 * isig2;
            const double zh = zeta_f64<K>(sqrt(r2) * me.isig);            // the 1/sigma_s^3 comes at the end
            const double w = me.gx * p.ax + me.gy * p.ay + me.gz * p.az - (me.vx * p.sx + me.vy * p.sy + me.vz * p.sz);
            const double kp = kappa_f64<K>(ss);
            acc[0] += zh * p.ax; acc[1] += zh * p.ay; acc[2] += zh * p.az;
            acc[3] += zh * p.sx; acc[4] += zh * p.sy; acc[5] += zh * p.sz;
            const double c = zh * w * kp;
            acc[6] += c * dx; acc[7] += c * dy; acc[8] += c * dz;
            acc[9] += zh * w * (ss * kp + 3.0);
        }
    }
    if (s < n) write_partial(partial, NACC2, n_pad, s, acc);
}

// -------------------------------------------------------------- FP32-comp passes
// Both passes stream the other role's records per warp, 32 per tile,
// double-buffered with cp.async (no block-wide barrier), as the forward mixed
// Estr does; offsets from the warp's first particle are formed by df_offset
// for both roles (the self pair has r^2 == 0 exactly and is skipped).  A tile
// is skipped when every pair of it is past zeta_skip_s from the warp's box
// (pass 1 with each source's own sigma; pass 2 with the warp's smallest lane
// sigma), then an 8-pair sub-block when every pair of the warp is.  Sums:
// 8-pair FP32 partials added with compensation, FP64 every 8 evaluated tiles.
__device__ __forceinline__ void ea_cp16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void ea_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void ea_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int EA_WT = 32;
constexpr int EA_FLUSH = 8;

// Stage one 64-byte record per lane (four 16-byte copies).
template <class R>
__device__ __forceinline__ void ea_stage(R* d, const R* g)
{
    const float4* gs = reinterpret_cast<const float4*>(g);
    float4* ds = reinterpret_cast<float4*>(d);
    ea_cp16(ds, gs); ea_cp16(ds + 1, gs + 1); ea_cp16(ds + 2, gs + 2); ea_cp16(ds + 3, gs + 3);
    ea_commit();
}

// The warp's origin (lane 0's particle, double-float), this lane's offset and the
// bounding box of the warp's offsets.
struct EaFrame {
    float3 oh, ol, me;
    float bmin[3], bmax[3];
    __device__ __forceinline__ void init(const float4& h, const float4& l, bool valid)
    {
        oh = make_float3(__shfl_sync(0xffffffffu, h.x, 0), __shfl_sync(0xffffffffu, h.y, 0),
                         __shfl_sync(0xffffffffu, h.z, 0));
        ol = make_float3(__shfl_sync(0xffffffffu, l.x, 0), __shfl_sync(0xffffffffu, l.y, 0),
                         __shfl_sync(0xffffffffu, l.z, 0));
        me = valid ? make_float3(df_offset(h.x, l.x, oh.x, ol.x), df_offset(h.y, l.y, oh.y, ol.y),
                                 df_offset(h.z, l.z, oh.z, ol.z))
                   : make_float3(0.f, 0.f, 0.f);
        bmin[0] = bmax[0] = me.x; bmin[1] = bmax[1] = me.y; bmin[2] = bmax[2] = me.z;
#pragma unroll
        for (int m = 16; m > 0; m >>= 1)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                bmin[k] = fminf(bmin[k], __shfl_xor_sync(0xffffffffu, bmin[k], m));
                bmax[k] = fmaxf(bmax[k], __shfl_xor_sync(0xffffffffu, bmax[k], m));
            }
    }
    // the FP32 box of the warp's valid particles (high parts) to wb[0] (low), wb[1] (high)
    __device__ __forceinline__ static void abs_box(const float4& h, bool valid, float4* wb)
    {
        float v[6] = {valid ? h.x : 3.0e38f, valid ? h.y : 3.0e38f, valid ? h.z : 3.0e38f,
                      valid ? -h.x : 3.0e38f, valid ? -h.y : 3.0e38f, valid ? -h.z : 3.0e38f};
#pragma unroll
        for (int m = 16; m > 0; m >>= 1)
#pragma unroll
            for (int k = 0; k < 6; k++) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], m));
        if ((threadIdx.x & 31) == 0) {
            wb[0] = make_float4(v[0], v[1], v[2], 0.f);
            wb[1] = make_float4(-v[3], -v[4], -v[5], 0.f);
        }
        __syncwarp();
    }
    __device__ __forceinline__ float3 offset(const float4& h, const float4& l) const
    {
        return make_float3(df_offset(h.x, l.x, oh.x, ol.x), df_offset(h.y, l.y, oh.y, ol.y),
                           df_offset(h.z, l.z, oh.z, ol.z));
    }
    __device__ __forceinline__ float box_dist2(const float3& p) const
    {
        const float ex = fmaxf(fmaxf(bmin[0] - p.x, p.x - bmax[0]), 0.0f);
        const float ey = fmaxf(fmaxf(bmin[1] - p.y, p.y - bmax[1]), 0.0f);
        const float ez = fmaxf(fmaxf(bmin[2] - p.z, p.z - bmax[2]), 0.0f);
        return fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    }
};

// Pass 1: lanes are targets t (Morton position), the tiles hold sources.
template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
ea1_mx(int64_t n, const TgtPos* __restrict__ tgt, const EA2Mx* __restrict__ self, int64_t n_pad,
       const EA1Mx* __restrict__ src, const float4* __restrict__ box, int64_t per_split, double* __restrict__ partial)
{
    __shared__ EA1Mx stage[UJ_WARPS][2][EA_WT];
    __shared__ float4 offs[UJ_WARPS][2][EA_WT];
    __shared__ float4 wbox[UJ_WARPS][2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const EA2Mx me = self[t < n ? t : n_pad - 1];
    EaFrame fr;
    fr.init(me.h, me.l, t < n);
    EaFrame::abs_box(me.h, t < n, wbox[warp]);
    double acc[NACC1] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    float sm[NACC1], cm[NACC1];
#pragma unroll
    for (int k = 0; k < NACC1; k++) { sm[k] = 0.f; cm[k] = 0.f; }
    const int64_t s0 = (int64_t)blockIdx.y * per_split, s1 = min(s0 + per_split, n_pad);
    const int ntiles = (int)((s1 - s0) / EA_WT);
    const EA1Mx* wsrc = src + s0 + lane;
    const float4* tbox = box + 2 * (s0 / EA_WT);
    TileWalk walk;
    walk.init(ntiles);
    int cur = walk.next<K>(tbox, wbox[warp][0], wbox[warp][1], lane);
    if (cur >= 0) ea_stage(&stage[warp][0][lane], wsrc + (int64_t)cur * EA_WT);
    int in_flush = 0, buf = 0;
    while (cur >= 0) {
        const int nxt = walk.next<K>(tbox, wbox[warp][0], wbox[warp][1], lane);
        if (nxt >= 0) {
            ea_stage(&stage[warp][buf ^ 1][lane], wsrc + (int64_t)nxt * EA_WT);
            ea_wait<1>();
        } else {
            ea_wait<0>();
        }
        __syncwarp();
        bool beyond;
        {
            const EA1Mx& r = stage[warp][buf][lane];
            const float3 p = fr.offset(r.a, r.b);
            offs[warp][buf][lane] = make_float4(p.x, p.y, p.z, r.a.w);
            beyond = fr.box_dist2(p) * r.a.w > zeta_skip_s<K>();
        }
        __syncwarp();
        if (!(zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, beyond))) {
#pragma unroll 1
            for (int sub = 0; sub < EA_WT; sub += EA_SUB) {
                float sv[EA_SUB], r2v[EA_SUB];
                bool far = true;
#pragma unroll
                for (int jj = 0; jj < EA_SUB; jj++) {
                    const float4 h = offs[warp][buf][sub + jj];
                    const float dx = fr.me.x - h.x, dy = fr.me.y - h.y, dz = fr.me.z - h.z;
                    r2v[jj] = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    sv[jj] = r2v[jj] * h.w;
                    far = far && sv[jj] > zeta_skip_s<K>();
                }
                if (zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, far)) continue;
                float f[NACC1] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int jj = 0; jj < EA_SUB; jj++) {
                    const int j = sub + jj;
                    const float4 h = offs[warp][buf][j];
                    const float dx = fr.me.x - h.x, dy = fr.me.y - h.y, dz = fr.me.z - h.z;
                    float zh = zhat_f32<K>(sv[jj]);
                    zh = r2v[jj] == 0.0f ? 0.0f : zh;     // the self pair and coincident pairs
                    const float4 g = stage[warp][buf][j].g, v = stage[warp][buf][j].v;
                    const float wh = fmaf(g.x, me.a.x, fmaf(g.y, me.a.y, g.z * me.a.z)) -
                                     fmaf(v.x, me.sb.x, fmaf(v.y, me.sb.y, v.z * me.sb.z));
                    f[0] = fmaf(zh, g.x, f[0]); f[1] = fmaf(zh, g.y, f[1]); f[2] = fmaf(zh, g.z, f[2]);
                    const float c = zh * wh * kappa_f32<K>(sv[jj]) * h.w;
                    f[3] = fmaf(c, dx, f[3]); f[4] = fmaf(c, dy, f[4]); f[5] = fmaf(c, dz, f[5]);
                }
#pragma unroll
                for (int k = 0; k < NACC1; k++) comp_add(sm[k], cm[k], f[k]);
            }
            if (++in_flush == EA_FLUSH) {     // evaluated tiles only
                in_flush = 0;
#pragma unroll
                for (int k = 0; k < NACC1; k++) { acc[k] += (double)sm[k] + (double)cm[k]; sm[k] = cm[k] = 0.f; }
            }
        }
        __syncwarp();   // every lane is done with `buf` before it is refilled
        cur = nxt;
        buf ^= 1;
    }
#pragma unroll
    for (int k = 0; k < NACC1; k++) acc[k] += (double)sm[k] + (double)cm[k];
    if (t < n) write_partial(partial, NACC1, n_pad, t, acc);
}

// Pass 2: lanes are sources s (Morton position), the tiles hold targets.
template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
ea2_mx(int64_t n, const EA1Mx* __restrict__ self, const double* __restrict__ gam, const TgtPos* __restrict__ tgt,
       const double* __restrict__ J, const uint8_t* __restrict__ st, bool transposed, int64_t n_pad,
       const EA2Mx* __restrict__ src, const float4* __restrict__ box, int64_t per_split, double* __restrict__ partial)
{
    __shared__ EA2Mx stage[UJ_WARPS][2][EA_WT];
    __shared__ float4 offs[UJ_WARPS][2][EA_WT];
    __shared__ float4 wbox[UJ_WARPS][2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const EA1Mx me = self[s < n ? s : n_pad - 1];
    // this lane's Gamma_s and v_s unscaled (the pass-1 record carries ZNORM/sigma^3)
    float3 G = make_float3(0.f, 0.f, 0.f), V = make_float3(0.f, 0.f, 0.f);
    if (s < n) {
        const int64_t i = tgt[s].idx;
        if (!(st && st[i])) {
            const double g0 = gam[3 * i], g1 = gam[3 * i + 1], g2 = gam[3 * i + 2];
            double v[3];
            mat_vec(J + 9 * i, g0, g1, g2, transposed, v);
            G = make_float3((float)g0, (float)g1, (float)g2);
            V = make_float3((float)v[0], (float)v[1], (float)v[2]);
        }
    }
    EaFrame fr;
    fr.init(me.a, me.b, s < n);
    EaFrame::abs_box(me.a, s < n, wbox[warp]);
    const float isig2 = me.a.w;
    float i2min = s < n ? isig2 : 3.0e38f;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) i2min = fminf(i2min, __shfl_xor_sync(0xffffffffu, i2min, m));
    double acc[NACC2];
    float sm[NACC2], cm[NACC2];
#pragma unroll
    for (int k = 0; k < NACC2; k++) { acc[k] = 0.0; sm[k] = 0.f; cm[k] = 0.f; }
    const int64_t s0 = (int64_t)blockIdx.y * per_split, s1 = min(s0 + per_split, n_pad);
    const int ntiles = (int)((s1 - s0) / EA_WT);
    const EA2Mx* wsrc = src + s0 + lane;
    const float4* tbox = box + 2 * (s0 / EA_WT);
    TileWalk walk;   // target tiles, tested at the lanes' largest sigma
    walk.init(ntiles);
    int cur = walk.next<K>(tbox, wbox[warp][0], wbox[warp][1], lane, i2min);
    if (cur >= 0) ea_stage(&stage[warp][0][lane], wsrc + (int64_t)cur * EA_WT);
    int in_flush = 0, buf = 0;
    while (cur >= 0) {
        const int nxt = walk.next<K>(tbox, wbox[warp][0], wbox[warp][1], lane, i2min);
        if (nxt >= 0) {
            ea_stage(&stage[warp][buf ^ 1][lane], wsrc + (int64_t)nxt * EA_WT);
            ea_wait<1>();
        } else {
            ea_wait<0>();
        }
        __syncwarp();
        bool beyond;
        {
            const EA2Mx& r = stage[warp][buf][lane];
            const float3 p = fr.offset(r.h, r.l);
            offs[warp][buf][lane] = make_float4(p.x, p.y, p.z, 0.f);
            beyond = fr.box_dist2(p) * i2min > zeta_skip_s<K>();
        }
        __syncwarp();
        if (!(zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, beyond))) {
#pragma unroll 1
            for (int sub = 0; sub < EA_WT; sub += EA_SUB) {
                float sv[EA_SUB], r2v[EA_SUB];
                bool far = true;
#pragma unroll
                for (int jj = 0; jj < EA_SUB; jj++) {
                    const float4 h = offs[warp][buf][sub + jj];
                    const float dx = fr.me.x - h.x, dy = fr.me.y - h.y, dz = fr.me.z - h.z;
                    r2v[jj] = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    sv[jj] = r2v[jj] * isig2;
                    far = far && sv[jj] > zeta_skip_s<K>();
                }
                if (zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, far)) continue;
                float f[NACC2];
#pragma unroll
                for (int k = 0; k < NACC2; k++) f[k] = 0.f;
#pragma unroll
                for (int jj = 0; jj < EA_SUB; jj++) {
                    const int j = sub + jj;
                    const float4 h = offs[warp][buf][j];
                    const float dx = fr.me.x - h.x, dy = fr.me.y - h.y, dz = fr.me.z - h.z;
                    float zh = zhat_f32<K>(sv[jj]);
                    zh = r2v[jj] == 0.0f ? 0.0f : zh;
                    const float4 a = stage[warp][buf][j].a, sb = stage[warp][buf][j].sb;
                    const float w = fmaf(G.x, a.x, fmaf(G.y, a.y, G.z * a.z)) - fmaf(V.x, sb.x, fmaf(V.y, sb.y, V.z * sb.z));
                    const float kp = kappa_f32<K>(sv[jj]);
                    f[0] = fmaf(zh, a.x, f[0]); f[1] = fmaf(zh, a.y, f[1]); f[2] = fmaf(zh, a.z, f[2]);
                    f[3] = fmaf(zh, sb.x, f[3]); f[4] = fmaf(zh, sb.y, f[4]); f[5] = fmaf(zh, sb.z, f[5]);
                    const float zw = zh * w;
                    const float c = zw * kp;
                    f[6] = fmaf(c, dx, f[6]); f[7] = fmaf(c, dy, f[7]); f[8] = fmaf(c, dz, f[8]);
                    f[9] = fmaf(zw, fmaf(sv[jj], kp, 3.0f), f[9]);
                }
#pragma unroll
                for (int k = 0; k < NACC2; k++) comp_add(sm[k], cm[k], f[k]);
            }
            if (++in_flush == EA_FLUSH) {     // evaluated tiles only
                in_flush = 0;
#pragma unroll
                for (int k = 0; k < NACC2; k++) { acc[k] += (double)sm[k] + (double)cm[k]; sm[k] = cm[k] = 0.f; }
            }
        }
        __syncwarp();
        cur = nxt;
        buf ^= 1;
    }
#pragma unroll
    for (int k = 0; k < NACC2; k++) acc[k] += (double)sm[k] + (double)cm[k];
    if (s < n) write_partial(partial, NACC2, n_pad, s, acc);
}

// ---------------------------------------------------------------- epilogues
// Pass 1: x_t and J_t of every non-static target (Morton position t).
__global__ void ea1_epilogue(int64_t n, int nsplit, const double* __restrict__ partial, int64_t n_pad,
                             const TgtPos* __restrict__ tgt, const uint8_t* __restrict__ st,
                             const double* __restrict__ Sbar, bool transposed, double* xbar, double* Jbar)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int64_t i = tgt[t].idx;
    if (st && st[i]) return;
    double a[NACC1];
    for (int k = 0; k < NACC1; k++) {
        double s = 0.0;
        for (int sp = 0; sp < nsplit; sp++) s += partial[((int64_t)sp * NACC1 + k) * n_pad + t];
        a[k] = s;
    }
    for (int k = 0; k < 3; k++) xbar[3 * i + k] += a[3 + k];
    const double* sb = Sbar + 3 * i;
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++)   // J[p + 3q] = M[p][q]
            Jbar[9 * i + p + 3 * q] += transposed ? a[p] * sb[q] : sb[p] * a[q];
}

// Pass 2: x_s, Gamma_s, sigma_s and J_s of every non-static source (Morton position s);
// `scale` = (ZNORM/sigma^3, ZNORM/sigma^5, -ZNORM/sigma^4) applied to (A, B), X, Sg (FP64:
// A, B, Sg, X hold zeta itself, with ZNORM; mixed: zeta / ZNORM).
template <int K>
__global__ void ea2_epilogue(int64_t n, int nsplit, const double* __restrict__ partial, int64_t n_pad,
                             const TgtPos* __restrict__ tgt, const uint8_t* __restrict__ st,
                             const double* __restrict__ gam, const double* __restrict__ sig,
                             const double* __restrict__ J, bool transposed, bool mixed, double* xbar, double* gbar,
                             double* sbar, double* Jbar)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int64_t i = tgt[s].idx;
    if (st && st[i]) return;
    double a[NACC2];
    for (int k = 0; k < NACC2; k++) {
        double v = 0.0;
        for (int sp = 0; sp < nsplit; sp++) v += partial[((int64_t)sp * NACC2 + k) * n_pad + s];
        a[k] = v;
    }
    const double is = 1.0 / sig[i];
    const double zn = mixed ? zeta_norm(K) : 1.0;
    const double c3 = zn * is * is * is, c5 = c3 * is * is, c4 = -c3 * is;
    double A[3], B[3];
    for (int k = 0; k < 3; k++) { A[k] = c3 * a[k]; B[k] = c3 * a[3 + k]; }
    for (int k = 0; k < 3; k++) xbar[3 * i + k] += c5 * a[6 + k];
    sbar[i] += c4 * a[9];
    double MB[3];
    mat_vec(J + 9 * i, B[0], B[1], B[2], !transposed, MB);   // M B (transposed) or M^T B (classic)
    const double* G = gam + 3 * i;
    for (int k = 0; k < 3; k++) gbar[3 * i + k] += A[k] - MB[k];
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++)
            Jbar[9 * i + p + 3 * q] -= transposed ? G[p] * B[q] : B[p] * G[q];
}

template <int K>
cudaError_t launch_k(const EstrAdjArgs& a, const EstrAdjWork& w, int num_sms, cudaStream_t st, int64_t* launches)
{
    const int64_t n = a.n;
    const int64_t n_pad = round_up(n, UJ_TILE);
    const int nsplit = uj_num_splits(n, n, num_sms);
    const int64_t tiles = n_pad / UJ_TILE;
    const int64_t per_split = ((tiles + nsplit - 1) / nsplit) * UJ_TILE;
    const dim3 grid((unsigned)(n_pad / UJ_THREADS), (unsigned)nsplit);
    const int pb = 256;
    const unsigned pg = (unsigned)((n_pad + pb - 1) / pb), eg = (unsigned)((n + pb - 1) / pb);
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(n, a.x, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    const bool mixed = a.precision != 0;
    // FP32-comp: the tile boxes follow pack 1's 64-byte records (within its 80-byte slots)
    float4* box = (float4*)((EA1Mx*)w.pack1 + n_pad);
    ea_pack<K><<<pg, pb, 0, st>>>(n, n_pad, tgt, a.x, a.gam, a.sig, a.J, a.static_flags, a.Sbar, a.transposed, mixed,
                                  w.pack1, w.pack2, box);
    if (!mixed) {
        ea1_f64<K><<<grid, UJ_THREADS, 0, st>>>(n, tgt, (const EA2F64*)w.pack2, n_pad, (const EA1F64*)w.pack1,
                                                per_split, w.partial);
        ea1_epilogue<<<eg, pb, 0, st>>>(n, nsplit, w.partial, n_pad, tgt, a.static_flags, a.Sbar, a.transposed,
                                        a.xbar, a.Jbar);
        ea2_f64<K><<<grid, UJ_THREADS, 0, st>>>(n, (const EA1F64*)w.pack1, n_pad, (const EA2F64*)w.pack2, per_split,
                                                w.partial);
    } else {
        ea1_mx<K><<<grid, UJ_THREADS, 0, st>>>(n, tgt, (const EA2Mx*)w.pack2, n_pad, (const EA1Mx*)w.pack1, box,
                                               per_split, w.partial);
        ea1_epilogue<<<eg, pb, 0, st>>>(n, nsplit, w.partial, n_pad, tgt, a.static_flags, a.Sbar, a.transposed,
                                        a.xbar, a.Jbar);
        ea2_mx<K><<<grid, UJ_THREADS, 0, st>>>(n, (const EA1Mx*)w.pack1, a.gam, tgt, a.J, a.static_flags,
                                               a.transposed, n_pad, (const EA2Mx*)w.pack2, box, per_split,
                                               w.partial);
    }
    ea2_epilogue<K><<<eg, pb, 0, st>>>(n, nsplit, w.partial, n_pad, tgt, a.static_flags, a.gam, a.sig, a.J,
                                       a.transposed, mixed, a.xbar, a.gbar, a.sbar, a.Jbar);
    *launches += 5;
    return cudaGetLastError();
}

}  // namespace

EstrAdjSizes estr_adjoint_sizes(int64_t n, int num_sms)
{
    const int64_t n_pad = round_up(n, UJ_TILE);
    EstrAdjSizes z;
    // the larger of the FP64 (80 B) and mixed (64 B) records; pack 1's mixed tile boxes
    // (1 B a particle) fit in the difference
    z.pack = (size_t)n_pad * 80;
    z.partial = (size_t)uj_num_splits(n, n, num_sms) * NACC2 * (size_t)n_pad * sizeof(double);
    return z;
}

cudaError_t launch_estr_adjoint(const EstrAdjArgs& a, const EstrAdjWork& w, int num_sms, cudaStream_t st,
                                int64_t* launches)
{
    static_assert(sizeof(EA1F64) == 80 && sizeof(EA2F64) == 80 && sizeof(EA1Mx) == 64 && sizeof(EA2Mx) == 64,
                  "pack records");
    if (a.n <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_k<K_SING>(a, w, num_sms, st, launches);
    case K_GAUS: return launch_k<K_GAUS>(a, w, num_sms, st, launches);
    case K_GAUSERF: return launch_k<K_GAUSERF>(a, w, num_sms, st, launches);
    case K_WNKLMNS: return launch_k<K_WNKLMNS>(a, w, num_sms, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
