// uj.cu -- all-pairs U and J kernels (the P2P pair loop of
// src/FLOWVPM_fmm.jl:102-168, over all sources as UJ_direct does,
// src/FLOWVPM_UJ.jl:35).
//
// Layout: one target per thread, UJ_THREADS targets per block; sources are
// packed once per call into a padded payload array and streamed through shared
// memory in tiles of UJ_TILE.  gridDim.y splits the sources when there are too
// few target blocks to fill the GPU; each split then writes FP64 partial sums
// to scratch and uj_reduce adds them, in split order, to the outputs.
#include "internal.h"
#include "vpm_math.cuh"

namespace vpm {

static_assert(UJ_TILE == UJ_THREADS, "one source loaded per thread per tile");
static_assert(UJ_TILE % UJ_BLOCK == 0, "FP32 blocks must tile the shared tile");

static inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

size_t uj_src_pack_bytes(int64_t ns, int precision)
{
    const int64_t n = round_up(ns, UJ_TILE);
    return (size_t)n * (precision ? sizeof(SrcMixed) : sizeof(SrcF64));
}

size_t uj_tgt_pack_bytes(int64_t nt, int precision)
{
    return precision ? (size_t)round_up(nt, UJ_THREADS) * sizeof(SrcMixed) : 0;
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
    // no empty splits
    const int64_t per = (tiles + nsplit - 1) / nsplit;
    nsplit = (tiles + per - 1) / per;
    return (int)nsplit;
}

size_t uj_partial_bytes(int64_t nt, int nsplit)
{
    return nsplit > 1 ? (size_t)nsplit * 12 * (size_t)round_up(nt, UJ_THREADS) * sizeof(double) : 0;
}

// ------------------------------------------------------------------ packing
template <int K>
__global__ void pack_src_mixed(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
                               const double* __restrict__ gs, const double* __restrict__ sgs,
                               SrcMixed* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ns_pad) return;
    SrcMixed p;
    if (i < ns) {
        const double x = xs[3 * i], y = xs[3 * i + 1], z = xs[3 * i + 2];
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        const double sig = (K == K_SING) ? 1.0 : sgs[i];
        const double isig = 1.0 / sig;
        const double isig2 = isig * isig;
        const double k = -C4 * isig2 * isig;
        p.a = make_float4(xh, yh, zh, (float)isig2);
        p.b = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
        p.c = make_float4((float)(k * gs[3 * i]), (float)(k * gs[3 * i + 1]), (float)(k * gs[3 * i + 2]), 0.f);
    } else {  // padding: no strength, at the origin, unit core
        p.a = make_float4(0.f, 0.f, 0.f, 1.f);
        p.b = make_float4(0.f, 0.f, 0.f, 0.f);
        p.c = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    out[i] = p;
}

__global__ void pack_tgt_mixed(int64_t nt, const double* __restrict__ xt, SrcMixed* __restrict__ out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const double x = xt[3 * i], y = xt[3 * i + 1], z = xt[3 * i + 2];
    const float xh = (float)x, yh = (float)y, zh = (float)z;
    SrcMixed p;
    p.a = make_float4(xh, yh, zh, 0.f);
    p.b = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh), 0.f);
    p.c = make_float4(0.f, 0.f, 0.f, 0.f);
    out[i] = p;
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
        p.gz_sig = make_double2(gs[3 * i + 2], sig);
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

// ----------------------------------------------------------- pair: mixed
// FP32 regular form (vpm_math.cuh).  With c = dx x Gamma'' (Gamma'' =
// -Gamma/(4 pi sigma^3)):  U += G c ;  J_ij += (H/sigma^2) c_i dx_j ;
// W += G Gamma''  (the Kronecker term, folded into J once per target).
template <int K>
__device__ __forceinline__ void pair_mixed(const float3& th, const float3& tl, const SrcMixed& p,
                                           float (&u)[3], float (&jj)[9], float (&w)[3])
{
    const float dx = (th.x - p.a.x) + (tl.x - p.b.x);
    const float dy = (th.y - p.a.y) + (tl.y - p.b.y);
    const float dz = (th.z - p.a.z) + (tl.z - p.b.z);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float s = r2 * p.a.w;
    float G, H;
    kernel_GH<K>(s, G, H);
    const bool nz = r2 > 0.0f;
    G = nz ? G : 0.0f;
    H = nz ? H : 0.0f;
    const float cx = fmaf(dy, p.c.z, -dz * p.c.y);
    const float cy = fmaf(dz, p.c.x, -dx * p.c.z);
    const float cz = fmaf(dx, p.c.y, -dy * p.c.x);
    u[0] = fmaf(G, cx, u[0]);
    u[1] = fmaf(G, cy, u[1]);
    u[2] = fmaf(G, cz, u[2]);
    w[0] = fmaf(G, p.c.x, w[0]);
    w[1] = fmaf(G, p.c.y, w[1]);
    w[2] = fmaf(G, p.c.z, w[2]);
    const float hb = H * p.a.w;
    const float bx = hb * cx, by = hb * cy, bz = hb * cz;
    jj[0] = fmaf(bx, dx, jj[0]);
    jj[1] = fmaf(by, dx, jj[1]);
    jj[2] = fmaf(bz, dx, jj[2]);
    jj[3] = fmaf(bx, dy, jj[3]);
    jj[4] = fmaf(by, dy, jj[4]);
    jj[5] = fmaf(bz, dy, jj[5]);
    jj[6] = fmaf(bx, dz, jj[6]);
    jj[7] = fmaf(by, dz, jj[7]);
    jj[8] = fmaf(bz, dz, jj[8]);
}

// --------------------------------------------------------------- epilogue
__device__ __forceinline__ void write_uj(int64_t t, const double (&acc)[12], double* U, int64_t ldU,
                                         double* J, int64_t ldJ, double* partial, int64_t nt_pad)
{
    if (partial) {
        double* p = partial + (int64_t)blockIdx.y * 12 * nt_pad + t;
#pragma unroll
        for (int k = 0; k < 12; k++) p[k * nt_pad] = acc[k];
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++) U[t * ldU + k] += acc[k];
#pragma unroll
        for (int k = 0; k < 9; k++) J[t * ldJ + k] += acc[3 + k];
    }
}

__global__ void uj_reduce(int64_t nt, int nsplit, const double* __restrict__ partial, int64_t nt_pad,
                          double* U, int64_t ldU, double* J, int64_t ldJ)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    for (int k = 0; k < 12; k++) {
        double s = 0.0;
        for (int sp = 0; sp < nsplit; sp++) s += partial[((int64_t)sp * 12 + k) * nt_pad + t];
        if (k < 3) U[t * ldU + k] += s;
        else J[t * ldJ + (k - 3)] += s;
    }
}

// ------------------------------------------------------------ main kernels
template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
uj_f64_kernel(int64_t nt, const double* __restrict__ xt, int64_t ns_pad, const SrcF64* __restrict__ src,
              int64_t per_split, double* U, int64_t ldU, double* J, int64_t ldJ,
              double* partial, int64_t nt_pad)
{
    __shared__ SrcF64 tile[UJ_TILE];
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    const double tx = valid ? xt[3 * t] : 1.0e3;
    const double ty = valid ? xt[3 * t + 1] : 1.0e3;
    const double tz = valid ? xt[3 * t + 2] : 1.0e3;
    double acc[12];
#pragma unroll
    for (int k = 0; k < 12; k++) acc[k] = 0.0;
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll 2
        for (int j = 0; j < UJ_TILE; j++) pair_f64<K>(tx, ty, tz, tile[j], acc);
    }
    if (valid) write_uj(t, acc, U, ldU, J, ldJ, partial, nt_pad);
}

template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
uj_mixed_kernel(int64_t nt, const SrcMixed* __restrict__ tgt, int64_t ns_pad,
                const SrcMixed* __restrict__ src, int64_t per_split, double* U, int64_t ldU,
                double* J, int64_t ldJ, double* partial, int64_t nt_pad)
{
    __shared__ SrcMixed tile[UJ_TILE];
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    float3 th = make_float3(1.0e4f, 1.0e4f, 1.0e4f), tl = make_float3(0.f, 0.f, 0.f);
    if (valid) {
        const float4 a = tgt[t].a, b = tgt[t].b;
        th = make_float3(a.x, a.y, a.z);
        tl = make_float3(b.x, b.y, b.z);
    }
    double dU[3] = {0.0, 0.0, 0.0}, dW[3] = {0.0, 0.0, 0.0};
    double dJ[9];
#pragma unroll
    for (int k = 0; k < 9; k++) dJ[k] = 0.0;
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll 1
        for (int sb = 0; sb < UJ_TILE; sb += UJ_BLOCK) {
            float u[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f};
            float jj[9];
#pragma unroll
            for (int k = 0; k < 9; k++) jj[k] = 0.f;
#pragma unroll 4
            for (int j = 0; j < UJ_BLOCK; j++) pair_mixed<K>(th, tl, tile[sb + j], u, jj, w);
#pragma unroll
            for (int k = 0; k < 3; k++) { dU[k] += (double)u[k]; dW[k] += (double)w[k]; }
#pragma unroll
            for (int k = 0; k < 9; k++) dJ[k] += (double)jj[k];
        }
    }
    if (!valid) return;
    // Kronecker term of src/FLOWVPM_fmm.jl:148-159: W = sum aux2 * Gamma
    dJ[1] -= dW[2];
    dJ[2] += dW[1];
    dJ[3] += dW[2];
    dJ[5] -= dW[0];
    dJ[6] -= dW[1];
    dJ[7] += dW[0];
    double acc[12] = {dU[0], dU[1], dU[2], dJ[0], dJ[1], dJ[2], dJ[3], dJ[4], dJ[5], dJ[6], dJ[7], dJ[8]};
    write_uj(t, acc, U, ldU, J, ldJ, partial, nt_pad);
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
    if (a.precision == 0) {
        SrcF64* src = (SrcF64*)w.src_pack;
        pack_src_f64<K><<<(unsigned)((ns_pad + pb - 1) / pb), pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs, src);
        uj_f64_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.nt, a.xt, ns_pad, src, per_split, a.U, a.ldU,
                                                       a.J, a.ldJ, partial, nt_pad);
        *launches += 2;
    } else {
        SrcMixed* src = (SrcMixed*)w.src_pack;
        pack_src_mixed<K><<<(unsigned)((ns_pad + pb - 1) / pb), pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs, src);
        const SrcMixed* tgt = src;
        *launches += 1;
        if (!a.self) {
            SrcMixed* tp = (SrcMixed*)w.tgt_pack;
            pack_tgt_mixed<<<(unsigned)((a.nt + pb - 1) / pb), pb, 0, st>>>(a.nt, a.xt, tp);
            tgt = tp;
            *launches += 1;
        }
        uj_mixed_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, ns_pad, src, per_split, a.U, a.ldU,
                                                         a.J, a.ldJ, partial, nt_pad);
        *launches += 1;
    }
    if (partial) {
        uj_reduce<<<(unsigned)((a.nt + pb - 1) / pb), pb, 0, st>>>(a.nt, nsplit, partial, nt_pad, a.U, a.ldU,
                                                                 a.J, a.ldJ);
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
