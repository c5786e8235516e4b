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

size_t estr_src_pack_bytes(int64_t ns, int precision)
{
    const int64_t n = round_up(ns, UJ_TILE);
    return (size_t)n * (precision ? sizeof(SrcEstrMixed) : sizeof(SrcEstrF64));
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
                                const TgtPos* __restrict__ order, SrcEstrMixed* __restrict__ out)
{
    // with `order` (sources = targets) the pack follows the targets' Morton order
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= ns_pad) return;
    SrcEstrMixed p;
    p.pad = 0.f;
    if (o < ns) {
        const int64_t i = order ? (int64_t)order[o].idx : o;
        const double isig = 1.0 / sgs[i];
        const double isig2 = isig * isig;
        p.x = xs[3 * i]; p.y = xs[3 * i + 1]; p.z = xs[3 * i + 2];
        p.isig2 = (float)isig2;
        const bool off = static_s && static_s[i];
        const double k = off ? 0.0 : zeta_norm(K) * isig2 * isig;
        const double gx = gs[3 * i], gy = gs[3 * i + 1], gz = gs[3 * i + 2];
        double vx = 0.0, vy = 0.0, vz = 0.0;   // the zeta field (Js null) needs no v
        if (Js) stretch_vec(Js + i * ldJs, gx, gy, gz, transposed, vx, vy, vz);
        p.g = make_float4((float)(k * gx), (float)(k * gy), (float)(k * gz), 0.f);
        p.v = make_float4((float)(k * vx), (float)(k * vy), (float)(k * vz), 0.f);
    } else {
        p.x = p.y = p.z = 0.0;
        p.isig2 = 1.f;
        p.g = p.v = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    out[o] = p;
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

// With DZ (the weight difference of the dynamic procedure's test filter,
// dynamic.cu) each weight zeta~(r, sigma_s) is replaced by
// zeta~(r, alpha sigma_s) - zeta~(r, sigma_s) = zeta~(r, sigma_s) (ratio - 1),
// ratio - 1 from zeta_ratio_m1 with the factors fd = (alpha^-3 - 1, alpha^-3, alpha^-2 - 1).
template <int K, bool ZETA, bool DZ = false>
__global__ void __launch_bounds__(UJ_THREADS)
estr_mixed_kernel(int64_t nt, const TgtPos* __restrict__ tgt, const double* __restrict__ Jt, int64_t ldJt,
                  const uint8_t* __restrict__ static_t, int64_t ns_pad, const SrcEstrMixed* __restrict__ src,
                  int64_t per_split, bool self, bool transposed, double* SFS, int64_t ldS, double* partial,
                  int64_t nt_pad, float3 fd = make_float3(0.f, 0.f, 0.f))
{
    __shared__ SrcEstrMixed tile[UJ_TILE];
    __shared__ float4 off[UJ_WARPS][UJ_TILE];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    int64_t idx = -1;
    if (t < nt) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
    }
    const bool valid = t < nt && (ZETA || !(static_t && static_t[idx]));
    const double ox = __shfl_sync(0xffffffffu, tx, 0);
    const double oy = __shfl_sync(0xffffffffu, ty, 0);
    const double oz = __shfl_sync(0xffffffffu, tz, 0);
    const float3 to = t < nt ? make_float3((float)(tx - ox), (float)(ty - oy), (float)(tz - oz))
                             : make_float3(3.0e4f, 3.0e4f, 3.0e4f);
    double zg[3] = {0.0, 0.0, 0.0}, zv[3] = {0.0, 0.0, 0.0};
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < UJ_TILE / 32; q++) {
            const int j = lane + 32 * q;
            off[warp][j] = make_float4((float)(tile[j].x - ox), (float)(tile[j].y - oy),
                                       (float)(tile[j].z - oz), tile[j].isig2);
        }
        __syncwarp();
#pragma unroll 1
        for (int sb = 0; sb < UJ_TILE; sb += UJ_BLOCK) {
            // compensated FP32 sums over the block (see comp_add), FP64 across blocks
            float sg[3] = {0.f, 0.f, 0.f}, cg[3] = {0.f, 0.f, 0.f}, sv[3] = {0.f, 0.f, 0.f}, cv[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
            for (int sub = 0; sub < UJ_BLOCK; sub += ESTR_SUB) {
                // s of the sub-block's sources; the sub-block is skipped when every pair of the warp
                // is past zeta_skip_s (zeta/zeta(0) < 1e-13 there)
                float sv8[ESTR_SUB], r28[ESTR_SUB];
                bool far = true;
#pragma unroll
                for (int jj = 0; jj < ESTR_SUB; jj++) {
                    const float4 a = off[warp][sb + sub + jj];
                    const float dx = to.x - a.x, dy = to.y - a.y, dz = to.z - a.z;
                    r28[jj] = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    sv8[jj] = r28[jj] * a.w;
                    far = far && sv8[jj] > zeta_skip_s<K>();
                }
                if (zeta_skip_s<K>() > 0.0f && __all_sync(0xffffffffu, far)) continue;
                float fg[3] = {0.f, 0.f, 0.f}, fv[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int jj = 0; jj < ESTR_SUB; jj++) {
                    const int j = sb + sub + jj;
                    float z = zhat_f32<K>(sv8[jj]);
                    if constexpr (DZ) z *= zeta_ratio_m1<K>(sv8[jj], fd);
                    if constexpr (!ZETA) z = (r28[jj] == 0.0f) ? 0.0f : z;
                    const float4 g = tile[j].g;
                    fg[0] = fmaf(z, g.x, fg[0]);
                    fg[1] = fmaf(z, g.y, fg[1]);
                    fg[2] = fmaf(z, g.z, fg[2]);
                    if constexpr (!ZETA) {
                        const float4 v = tile[j].v;
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
#pragma unroll
            for (int k = 0; k < 3; k++) {
                zg[k] += (double)sg[k] + (double)cg[k];
                if constexpr (!ZETA) zv[k] += (double)sv[k] + (double)cv[k];
            }
        }
        __syncwarp();
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
        SrcEstrMixed* src = (SrcEstrMixed*)w.src_pack;
        pack_estr_mixed<K><<<pgrid, pb, 0, st>>>(a.ns, ns_pad, a.xs, a.gs, a.sgs, a.zeta ? nullptr : a.Js, a.ldJs,
                                                  static_s, a.transposed, a.self ? tgt : nullptr, src);
        if (a.zeta)
            estr_mixed_kernel<K, true><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad, src,
                                                                    per_split, a.self, a.transposed, a.SFS, a.ldS,
                                                                    partial, nt_pad);
        else if (a.dz_alpha > 0.0) {
            const double al = a.dz_alpha;
            const float3 fd = make_float3((float)(1.0 / (al * al * al) - 1.0), (float)(1.0 / (al * al * al)),
                                          (float)(1.0 / (al * al) - 1.0));
            estr_mixed_kernel<K, false, true><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad,
                                                                           src, per_split, a.self, a.transposed,
                                                                           a.SFS, a.ldS, partial, nt_pad, fd);
        } else
            estr_mixed_kernel<K, false><<<grid, UJ_THREADS, 0, st>>>(a.nt, tgt, a.Jt, a.ldJt, static_t, ns_pad, src,
                                                                     per_split, a.self, a.transposed, a.SFS, a.ldS,
                                                                     partial, nt_pad);
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
