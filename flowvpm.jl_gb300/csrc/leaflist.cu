// leaflist.cu -- near-field P2P over octree leaf pairs: the direct leg of
// UJ_fmm (FastMultipole's direct_list, src/FLOWVPM_UJ.jl:90-100) and the Estr
// pass over the same list (Estr_fmm!, src/FLOWVPM_subfilterscale_models.jl:94-188).
//
// The host builds the octree and the leaf-pair list (tree.cpp); particles are
// processed in the tree's Morton order, so every leaf is a contiguous range.
// One block per target leaf, one target per thread (leaves hold at most
// LEAF_MAX particles); the block walks its list of source leaves, staging each
// source leaf in shared memory.  Pair math is that of the all-pairs kernels
// (uj_pair.cuh for FP32-comp, the reference formula for FP64); Estr uses the
// same factored form as estr.cu with the self pair excluded by position.
#include "internal.h"
#include "tree.h"
#include "uj_pair.cuh"
#include "vpm_math.cuh"

namespace vpm {

constexpr int LEAF_MAX = LEAF_SIZE_MAX;   // threads per block = largest leaf
constexpr int MID_LEAVES = 4;      // source leaves summed in FP32 before the FP64 add

static_assert(LEAF_MAX % 32 == 0 && LEAF_MAX % 4 == 0, "whole warps, 4-source groups");

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
    p.gz_sig = make_double2(gs[3 * i + 2], sig);
    out[o] = p;
}

// Estr source payloads in Morton order (v = J^T Gamma or J Gamma, zero for static sources).
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
    const double* J = Js + 9 * i;
    double vx, vy, vz;
    if (transposed) {
        vx = J[0] * gx + J[1] * gy + J[2] * gz; vy = J[3] * gx + J[4] * gy + J[5] * gz; vz = J[6] * gx + J[7] * gy + J[8] * gz;
    } else {
        vx = J[0] * gx + J[3] * gy + J[6] * gz; vy = J[1] * gx + J[4] * gy + J[7] * gz; vz = J[2] * gx + J[5] * gy + J[8] * gz;
    }
    const double isig = 1.0 / sgs[i];
    if (precision) {
        const double k = off ? 0.0 : zeta_norm(K) * isig * isig * isig;
        SrcEstrMixed p;
        p.x = x[3 * i]; p.y = x[3 * i + 1]; p.z = x[3 * i + 2];
        p.isig2 = (float)(isig * isig); p.pad = 0.f;
        p.g = make_float4((float)(k * gx), (float)(k * gy), (float)(k * gz), 0.f);
        p.v = make_float4((float)(k * vx), (float)(k * vy), (float)(k * vz), 0.f);
        ((SrcEstrMixed*)out)[o] = p;
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

// ------------------------------------------------------------- UJ, FP32-comp
template <int K>
__global__ void __launch_bounds__(LEAF_MAX)
leaf_uj_mixed(const TgtPos* __restrict__ tgt, const int32_t* __restrict__ lb, const int32_t* __restrict__ le,
              const int32_t* __restrict__ row, const int32_t* __restrict__ col,
              const SrcMixed* __restrict__ src, double* U, double* J)
{
    __shared__ SrcMixed tile[LEAF_MAX];
    __shared__ float4 off[LEAF_MAX / 32][LEAF_MAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int leaf = blockIdx.x;
    const int64_t t = (int64_t)lb[leaf] + threadIdx.x;
    const bool valid = t < le[leaf];
    double tx = 3.0e4, ty = 3.0e4, tz = 3.0e4;
    int32_t idx = 0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    // warp origin: lane 0's target if valid, else the leaf's first target
    const int64_t t0 = (int64_t)lb[leaf] + warp * 32;
    const bool w_any = t0 < le[leaf];
    const TgtPos p0 = tgt[w_any ? t0 : (int64_t)lb[leaf]];
    const double ox = p0.x, oy = p0.y, oz = p0.z;
    const float3 th = make_float3((float)tx, (float)ty, (float)tz);
    const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y), (float)(tz - (double)th.z));
    const float3 oh = make_float3((float)ox, (float)oy, (float)oz);
    const float3 ol = make_float3((float)(ox - (double)oh.x), (float)(oy - (double)oh.y), (float)(oz - (double)oh.z));
    const float3 to = valid ? make_float3((float)(tx - ox), (float)(ty - oy), (float)(tz - oz))
                            : make_float3(3.0e4f, 3.0e4f, 3.0e4f);
    float b2 = valid ? fmaf(to.x, to.x, fmaf(to.y, to.y, to.z * to.z)) : 0.0f;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) b2 = fmaxf(b2, __shfl_xor_sync(0xffffffffu, b2, m));
    const float r2n = fmaxf(4.0f * b2, 1.0e-30f);
    const float sfar = s_far<K>();

    double dU[3] = {0.0, 0.0, 0.0}, dW[3] = {0.0, 0.0, 0.0}, dJ[8];
    float mu[3] = {0.f, 0.f, 0.f}, mw[3] = {0.f, 0.f, 0.f}, mj[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { dJ[k] = 0.0; mj[k] = 0.f; }
    int in_mid = 0;
    const int e0 = row[leaf], e1 = row[leaf + 1];
    for (int e = e0; e < e1; e++) {
        const int sl = col[e];
        const int64_t sb = lb[sl];
        const int cnt = le[sl] - lb[sl];
        __syncthreads();
        if (threadIdx.x < cnt) {
            tile[threadIdx.x] = src[sb + threadIdx.x];
        } else {   // padding: far away, no strength
            tile[threadIdx.x].a = make_float4(1.0e6f, 1.0e6f, 1.0e6f, 1.f);
            tile[threadIdx.x].b = make_float4(0.f, 0.f, 0.f, 1.f);
            tile[threadIdx.x].gam = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        const int ng = (cnt + 3) / 4;
        for (int j = lane; j < 4 * ng; j += 32) {
            const float4 a = tile[j].a, b = tile[j].b;
            const float thr = singular_tail<K>() ? fmaxf(sfar * a.w, r2n) : b.w * b.w;
            off[warp][j] = make_float4((a.x - oh.x) + (b.x - ol.x), (a.y - oh.y) + (b.y - ol.y),
                                       (a.z - oh.z) + (b.z - ol.z), thr);
        }
        __syncwarp();
        float u[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f}, jq[8];
#pragma unroll
        for (int k = 0; k < 8; k++) jq[k] = 0.f;
        for (int g = 0; g < ng; g++) pair4_mixed<K>(to, th, tl, r2n, off[warp], tile, 4 * g, u, jq, w);
#pragma unroll
        for (int k = 0; k < 3; k++) { mu[k] += u[k]; mw[k] += w[k]; }
#pragma unroll
        for (int k = 0; k < 8; k++) mj[k] += jq[k];
        if (++in_mid == MID_LEAVES || e + 1 == e1) {
#pragma unroll
            for (int k = 0; k < 3; k++) { dU[k] += (double)mu[k]; dW[k] += (double)mw[k]; mu[k] = 0.f; mw[k] = 0.f; }
#pragma unroll
            for (int k = 0; k < 8; k++) { dJ[k] += (double)mj[k]; mj[k] = 0.f; }
            in_mid = 0;
        }
    }
    if (!valid) return;
    double j9[9];
#pragma unroll
    for (int k = 0; k < 8; k++) j9[k] = -3.0 * dJ[k];
    j9[8] = 3.0 * (dJ[0] + dJ[4]);
    j9[1] -= dW[2]; j9[2] += dW[1]; j9[3] += dW[2]; j9[5] -= dW[0]; j9[6] -= dW[1]; j9[7] += dW[0];
#pragma unroll
    for (int k = 0; k < 3; k++) U[3 * (int64_t)idx + k] += dU[k];
#pragma unroll
    for (int k = 0; k < 9; k++) J[9 * (int64_t)idx + k] += j9[k];
}

// --------------------------------------------------------------------- UJ, FP64
template <int K>
__device__ __forceinline__ void leaf_pair_f64(double tx, double ty, double tz, const SrcF64& s, double (&acc)[12])
{
    const double dx = tx - s.xy.x, dy = ty - s.xy.y, dz = tz - s.z_isig.x;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 != 0.0) {
        const double rinv = rsqrt(r2);
        const double isig = s.z_isig.y;
        double g, dg;
        g_dgdr_f64<K>(r2 * rinv * isig, g, dg);
        const double r3inv = rinv * rinv * rinv;
        const double gx = s.gxy.x, gy = s.gxy.y, gz = s.gz_sig.x;
        const double k = -C4 * r3inv;
        const double c1 = k * (dy * gz - dz * gy), c2 = k * (dz * gx - dx * gz), c3 = k * (dx * gy - dy * gx);
        acc[0] += g * c1; acc[1] += g * c2; acc[2] += g * c3;
        const double aux = dg * isig * rinv - 3.0 * g * rinv * rinv;
        const double aux2 = -C4 * g * r3inv;
        const double a1 = aux * c1, a2 = aux * c2, a3 = aux * c3;
        acc[3] += a1 * dx; acc[4] += a2 * dx - aux2 * gz; acc[5] += a3 * dx + aux2 * gy;
        acc[6] += a1 * dy + aux2 * gz; acc[7] += a2 * dy; acc[8] += a3 * dy - aux2 * gx;
        acc[9] += a1 * dz - aux2 * gy; acc[10] += a2 * dz + aux2 * gx; acc[11] += a3 * dz;
    }
}

template <int K>
__global__ void __launch_bounds__(LEAF_MAX)
leaf_uj_f64(const TgtPos* __restrict__ tgt, const int32_t* __restrict__ lb, const int32_t* __restrict__ le,
            const int32_t* __restrict__ row, const int32_t* __restrict__ col,
            const SrcF64* __restrict__ src, double* U, double* J)
{
    __shared__ SrcF64 tile[LEAF_MAX];
    const int leaf = blockIdx.x;
    const int64_t t = (int64_t)lb[leaf] + threadIdx.x;
    const bool valid = t < le[leaf];
    double tx = 1.0e3, ty = 1.0e3, tz = 1.0e3;
    int32_t idx = 0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    double acc[12];
#pragma unroll
    for (int k = 0; k < 12; k++) acc[k] = 0.0;
    for (int e = row[leaf]; e < row[leaf + 1]; e++) {
        const int sl = col[e];
        const int cnt = le[sl] - lb[sl];
        __syncthreads();
        if (threadIdx.x < cnt) tile[threadIdx.x] = src[(int64_t)lb[sl] + threadIdx.x];
        __syncthreads();
        for (int j = 0; j < cnt; j++) leaf_pair_f64<K>(tx, ty, tz, tile[j], acc);
    }
    if (!valid) return;
#pragma unroll
    for (int k = 0; k < 3; k++) U[3 * (int64_t)idx + k] += acc[k];
#pragma unroll
    for (int k = 0; k < 9; k++) J[9 * (int64_t)idx + k] += acc[3 + k];
}

// ------------------------------------------------------------------------- Estr
template <int K, bool MIXED>
__global__ void __launch_bounds__(LEAF_MAX)
leaf_estr(const TgtPos* __restrict__ tgt, const int32_t* __restrict__ lb, const int32_t* __restrict__ le,
          const int32_t* __restrict__ row, const int32_t* __restrict__ col, const void* __restrict__ srcv,
          const double* __restrict__ Jt, const uint8_t* __restrict__ static_t, bool transposed, double* SFS)
{
    __shared__ __align__(16) unsigned char tile_raw[LEAF_MAX * (MIXED ? sizeof(SrcEstrMixed) : sizeof(SrcEstrF64))];
    __shared__ float4 s_hi[LEAF_MAX], s_lo[LEAF_MAX];   // mixed: double-float source positions
    const int leaf = blockIdx.x;
    const int64_t t = (int64_t)lb[leaf] + threadIdx.x;
    const bool in = t < le[leaf];
    double tx = 1.0e3, ty = 1.0e3, tz = 1.0e3;
    int32_t idx = 0;
    if (in) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const bool valid = in && !(static_t && static_t[idx]);
    const float3 th = make_float3((float)tx, (float)ty, (float)tz);
    const float3 tl = make_float3((float)(tx - (double)th.x), (float)(ty - (double)th.y), (float)(tz - (double)th.z));
    double zg[3] = {0.0, 0.0, 0.0}, zv[3] = {0.0, 0.0, 0.0};
    for (int e = row[leaf]; e < row[leaf + 1]; e++) {
        const int sl = col[e];
        const int64_t sb = lb[sl];
        const int cnt = le[sl] - lb[sl];
        __syncthreads();
        if (threadIdx.x < cnt) {
            if (MIXED) {
                const SrcEstrMixed p = ((const SrcEstrMixed*)srcv)[sb + threadIdx.x];
                ((SrcEstrMixed*)tile_raw)[threadIdx.x] = p;
                const float xh = (float)p.x, yh = (float)p.y, zh = (float)p.z;
                s_hi[threadIdx.x] = make_float4(xh, yh, zh, p.isig2);
                s_lo[threadIdx.x] = make_float4((float)(p.x - (double)xh), (float)(p.y - (double)yh),
                                                (float)(p.z - (double)zh), 0.f);
            } else {
                ((SrcEstrF64*)tile_raw)[threadIdx.x] = ((const SrcEstrF64*)srcv)[sb + threadIdx.x];
            }
        }
        __syncthreads();
        float fg[3] = {0.f, 0.f, 0.f}, fv[3] = {0.f, 0.f, 0.f};
        for (int j = 0; j < cnt; j++) {
            if (sb + j == t) continue;   // the self pair (sources and targets share the order)
            if (MIXED) {
                const SrcEstrMixed& p = ((const SrcEstrMixed*)tile_raw)[j];
                const float4 h = s_hi[j], l = s_lo[j];
                const float dx = (th.x - h.x) + (tl.x - l.x);
                const float dy = (th.y - h.y) + (tl.y - l.y);
                const float dz = (th.z - h.z) + (tl.z - l.z);
                const float z = zhat_f32<K>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * h.w);
                fg[0] = fmaf(z, p.g.x, fg[0]); fg[1] = fmaf(z, p.g.y, fg[1]); fg[2] = fmaf(z, p.g.z, fg[2]);
                fv[0] = fmaf(z, p.v.x, fv[0]); fv[1] = fmaf(z, p.v.y, fv[1]); fv[2] = fmaf(z, p.v.z, fv[2]);
            } else {
                const SrcEstrF64& p = ((const SrcEstrF64*)tile_raw)[j];
                const double dx = p.xy.x - tx, dy = p.xy.y - ty, dz = p.z_isig.x - tz;
                const double isig = p.z_isig.y;
                const double z = zeta_f64<K>(sqrt(dx * dx + dy * dy + dz * dz) * isig) * isig * isig * isig;
                zg[0] += z * p.gxy.x; zg[1] += z * p.gxy.y; zg[2] += z * p.gz_vx.x;
                zv[0] += z * p.gz_vx.y; zv[1] += z * p.vyz.x; zv[2] += z * p.vyz.y;
            }
        }
        if (MIXED) {
#pragma unroll
            for (int k = 0; k < 3; k++) { zg[k] += (double)fg[k]; zv[k] += (double)fv[k]; }
        }
    }
    if (!valid) return;
    const double* Jp = Jt + 9 * (int64_t)idx;
    double s[3];
    if (transposed) {
        s[0] = Jp[0] * zg[0] + Jp[1] * zg[1] + Jp[2] * zg[2];
        s[1] = Jp[3] * zg[0] + Jp[4] * zg[1] + Jp[5] * zg[2];
        s[2] = Jp[6] * zg[0] + Jp[7] * zg[1] + Jp[8] * zg[2];
    } else {
        s[0] = Jp[0] * zg[0] + Jp[3] * zg[1] + Jp[6] * zg[2];
        s[1] = Jp[1] * zg[0] + Jp[4] * zg[1] + Jp[7] * zg[2];
        s[2] = Jp[2] * zg[0] + Jp[5] * zg[1] + Jp[8] * zg[2];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) SFS[3 * (int64_t)idx + k] += s[k] - zv[k];
}

// ---------------------------------------------------------------------- launcher
size_t leaf_work_bytes(int64_t n, int64_t nleaves, int64_t npairs_leaf)
{
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    return al(n * sizeof(TgtPos)) + al(n * sizeof(SrcEstrF64)) + al(n * sizeof(int32_t)) +
           2 * al(nleaves * sizeof(int32_t)) + al((nleaves + 1) * sizeof(int32_t)) + al(npairs_leaf * sizeof(int32_t));
}

template <int K>
static cudaError_t launch_leaf_k(const LeafArgs& a, const LeafLists& L, void* work, cudaStream_t st,
                                 int64_t* launches)
{
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const int64_t n = a.n;
    const int64_t nl = (int64_t)L.leaf_begin.size();
    char* p = (char*)work;
    TgtPos* tgt = (TgtPos*)p;            p += al(n * sizeof(TgtPos));
    void* src = p;                       p += al(n * sizeof(SrcEstrF64));
    int32_t* perm = (int32_t*)p;         p += al(n * sizeof(int32_t));
    int32_t* lb = (int32_t*)p;           p += al(nl * sizeof(int32_t));
    int32_t* le = (int32_t*)p;           p += al(nl * sizeof(int32_t));
    int32_t* row = (int32_t*)p;          p += al((nl + 1) * sizeof(int32_t));
    int32_t* col = (int32_t*)p;
    // host -> device copies of the lists (narrowed to int32: n < 2^31)
    std::vector<int32_t> hb(nl), he(nl), hr(nl + 1);
    for (int64_t l = 0; l < nl; l++) { hb[l] = (int32_t)L.leaf_begin[l]; he[l] = (int32_t)L.leaf_end[l]; }
    for (int64_t l = 0; l <= nl; l++) hr[l] = (int32_t)L.row[l];
    cudaError_t e;
    if ((e = cudaMemcpyAsync(perm, L.perm.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(lb, hb.data(), nl * sizeof(int32_t), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(le, he.data(), nl * sizeof(int32_t), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(row, hr.data(), (nl + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(col, L.col.data(), L.col.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st)))
        return e;
    // the host vectors must outlive the copies
    if ((e = cudaStreamSynchronize(st))) return e;
    const unsigned g = (unsigned)((n + 255) / 256);
    tgt_from_perm<<<g, 256, 0, st>>>(n, a.x, perm, tgt);
    if (a.precision) {
        leaf_pack_mixed<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, perm, (SrcMixed*)src);
        leaf_uj_mixed<K><<<(unsigned)nl, LEAF_MAX, 0, st>>>(tgt, lb, le, row, col, (const SrcMixed*)src, a.U, a.J);
    } else {
        leaf_pack_f64<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, perm, (SrcF64*)src);
        leaf_uj_f64<K><<<(unsigned)nl, LEAF_MAX, 0, st>>>(tgt, lb, le, row, col, (const SrcF64*)src, a.U, a.J);
    }
    *launches += 3;
    if (a.sfs) {
        leaf_pack_estr<K><<<g, 256, 0, st>>>(n, a.x, a.gam, a.sig, a.J, a.static_flags, a.transposed, perm,
                                              a.precision, src);
        if (a.precision)
            leaf_estr<K, true><<<(unsigned)nl, LEAF_MAX, 0, st>>>(tgt, lb, le, row, col, src, a.J, a.static_flags,
                                                                  a.transposed, a.SFS);
        else
            leaf_estr<K, false><<<(unsigned)nl, LEAF_MAX, 0, st>>>(tgt, lb, le, row, col, src, a.J, a.static_flags,
                                                                   a.transposed, a.SFS);
        *launches += 2;
    }
    return cudaGetLastError();
}

cudaError_t launch_leaflist(const LeafArgs& a, const LeafLists& L, void* work, cudaStream_t st, int64_t* launches)
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
