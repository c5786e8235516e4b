// adjoint.cu -- reverse mode of the UJ pair sum (replaces the unwired rrule
// of src/FLOWVPM_rrules.jl:179-330).
//
// For L with dL/dU = Ubar and dL/dJ = Jbar, each pair (t, s) contributes
//     phi = Ubar_t . u(dx, Gamma_s, sigma_s) + Jbar_t : j(dx, Gamma_s, sigma_s),
// dx = x_t - x_s, with u and j the pair terms of src/FLOWVPM_fmm.jl:112-160.
// Writing q(r) = -g(rho)/(4 pi r^3), A = q, B = q'/r, c = dx x Gamma:
//     u = A c,   j_ab = B c_a dx_b + A eps_abl Gamma_l,
//     phi = A P + B Q,  P = Ubar.c + wbar.Gamma,  Q = c.(Jbar dx),  wbar_l = eps_abl Jbar_ab
// and
//     dphi/d(dx)   = (B P + (B'/r) Q) dx + A (Gamma x Ubar) + B (Gamma x Jbar dx + Jbar^T c)
//     dphi/dGamma  = A (Ubar x dx + wbar) + B ((Jbar dx) x dx)
//     dphi/dsigma  = (dA/dsigma) P + (dB/dsigma) Q
// with q'' (hence the kernels' g'') in B'.  x_t gets +dphi/d(dx), x_s gets
// -dphi/d(dx).
//
// Layout: one target per thread (Morton order, as in uj.cu), sources staged in
// shared memory.  Target-side sums stay in registers; each source's 7 sums
// (x, Gamma, sigma) are reduced across the warp with shuffles, across the
// block's 4 warps in shared memory, then added to the outputs with one FP64
// atomic per source and block (so the summation order of those sums is not
// fixed).  Arithmetic is FP64 throughout.
#include "internal.h"
#include "vpm_math.cuh"

namespace vpm {

// (g, g', g'') of kernel K at rho, FP64 (derivatives of src/FLOWVPM_kernel.jl:45-84).
// Beyond rho = 9 (Gaussian-erf) / 3.5 (Gaussian) g = 1 and g' = g'' = 0 to FP64.
template <int K>
__device__ __forceinline__ void g_d1_d2_f64(double rho, double& g, double& d1, double& d2)
{
    if constexpr (K == K_SING) {
        g = 1.0; d1 = 0.0; d2 = 0.0;
    } else if constexpr (K == K_GAUS) {
        if (rho > 3.5) { g = 1.0; d1 = 0.0; d2 = 0.0; }
        else {
            const double r3 = rho * rho * rho;
            const double e = exp(-r3);
            g = 1.0 - e; d1 = 3.0 * rho * rho * e; d2 = (6.0 * rho - 9.0 * r3 * rho) * e;
        }
    } else if constexpr (K == K_GAUSERF) {
        if (rho > 9.0) { g = 1.0; d1 = 0.0; d2 = 0.0; }
        else {
            const double e = C2 * exp(-0.5 * rho * rho);
            g = erf(rho * INV_SQRT2) - rho * e;
            d1 = rho * rho * e;
            d2 = (2.0 * rho - rho * rho * rho) * e;
        }
    } else {
        const double q = rho * rho + 1.0;
        const double iq = 1.0 / q;
        const double iq25 = iq * iq * sqrt(iq);           // q^-2.5
        g = rho * rho * rho * (rho * rho + 2.5) * iq25;
        d1 = 7.5 * rho * rho * iq25 * iq;
        d2 = 7.5 * rho * (2.0 - 5.0 * rho * rho) * iq25 * iq * iq;
    }
}

// The 7 derivatives of phi for one pair: o[0..2] = dphi/d(dx), o[3..5] = dphi/dGamma,
// o[6] = dphi/dsigma.  Pairs with r^2 == 0 give zeros.
template <int K>
__device__ __forceinline__ void adj_pair_f64(double dx, double dy, double dz, const SrcF64& s,
                                             const double (&Ub)[3], const double (&Jb)[9], const double (&wb)[3],
                                             double (&o)[7])
{
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 == 0.0) {
#pragma unroll
        for (int k = 0; k < 7; k++) o[k] = 0.0;
        return;
    }
    const double isig = s.z_isig.y, sig = s.gz_sig.y;
    const double rinv = rsqrt(r2);
    const double r = r2 * rinv;
    const double rho = r * isig;
    double g, g1, g2;
    g_d1_d2_f64<K>(rho, g, g1, g2);
    const double ri2 = rinv * rinv, ri3 = ri2 * rinv, ri4 = ri2 * ri2, ri5 = ri4 * rinv;
    const double A = -C4 * g * ri3;
    const double B = -C4 * (g1 * isig * ri4 - 3.0 * g * ri5);
    const double qpp = -C4 * (g2 * isig * isig * ri3 - 6.0 * g1 * isig * ri4 + 12.0 * g * ri5);
    const double Bpr = (qpp - B) * ri2;
    const double dA = C4 * g1 * rho * isig * ri3;
    const double dB = -C4 * (2.0 * g1 - rho * g2) * isig * isig * ri4;
    (void)sig;
    const double Gx = s.gxy.x, Gy = s.gxy.y, Gz = s.gz_sig.x;
    const double cx = dy * Gz - dz * Gy, cy = dz * Gx - dx * Gz, cz = dx * Gy - dy * Gx;
    const double JDx = Jb[0] * dx + Jb[3] * dy + Jb[6] * dz;
    const double JDy = Jb[1] * dx + Jb[4] * dy + Jb[7] * dz;
    const double JDz = Jb[2] * dx + Jb[5] * dy + Jb[8] * dz;
    const double JTcx = Jb[0] * cx + Jb[1] * cy + Jb[2] * cz;
    const double JTcy = Jb[3] * cx + Jb[4] * cy + Jb[5] * cz;
    const double JTcz = Jb[6] * cx + Jb[7] * cy + Jb[8] * cz;
    const double P = Ub[0] * cx + Ub[1] * cy + Ub[2] * cz + wb[0] * Gx + wb[1] * Gy + wb[2] * Gz;
    const double Q = cx * JDx + cy * JDy + cz * JDz;
    const double sc = B * P + Bpr * Q;
    o[0] = sc * dx + A * (Gy * Ub[2] - Gz * Ub[1]) + B * (Gy * JDz - Gz * JDy + JTcx);
    o[1] = sc * dy + A * (Gz * Ub[0] - Gx * Ub[2]) + B * (Gz * JDx - Gx * JDz + JTcy);
    o[2] = sc * dz + A * (Gx * Ub[1] - Gy * Ub[0]) + B * (Gx * JDy - Gy * JDx + JTcz);
    o[3] = A * (Ub[1] * dz - Ub[2] * dy + wb[0]) + B * (JDy * dz - JDz * dy);
    o[4] = A * (Ub[2] * dx - Ub[0] * dz + wb[1]) + B * (JDz * dx - JDx * dz);
    o[5] = A * (Ub[0] * dy - Ub[1] * dx + wb[2]) + B * (JDx * dy - JDy * dx);
    o[6] = (K == K_SING) ? 0.0 : dA * P + dB * Q;
}

template <int K>
__global__ void __launch_bounds__(UJ_THREADS)
uj_adjoint_f64_kernel(int64_t nt, const TgtPos* __restrict__ tgt, const double* __restrict__ Ubar,
                      const double* __restrict__ Jbar, int64_t ns, int64_t ns_pad,
                      const SrcF64* __restrict__ src, int64_t per_split, double* xbar, double* gbar,
                      double* sbar)
{
    __shared__ SrcF64 tile[UJ_TILE];
    __shared__ double red[UJ_WARPS][UJ_TILE][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * UJ_THREADS + threadIdx.x;
    const bool valid = t < nt;
    double tx = 3.0e4, ty = 3.0e4, tz = 3.0e4;
    int64_t idx = 0;
    double Ub[3] = {0.0, 0.0, 0.0}, Jb[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Jb[k] = 0.0;
    if (valid) {
        const TgtPos p = tgt[t];
        tx = p.x; ty = p.y; tz = p.z; idx = p.idx;
#pragma unroll
        for (int k = 0; k < 3; k++) Ub[k] = Ubar[3 * idx + k];
#pragma unroll
        for (int k = 0; k < 9; k++) Jb[k] = Jbar[9 * idx + k];
    }
    // wbar_l = eps_abl Jbar_ab with Jbar_ab at Jb[a + 3b]
    const double wb[3] = {Jb[1 + 3 * 2] - Jb[2 + 3 * 1], Jb[2 + 3 * 0] - Jb[0 + 3 * 2], Jb[0 + 3 * 1] - Jb[1 + 3 * 0]};
    double acc[3] = {0.0, 0.0, 0.0};
    const int64_t s0 = (int64_t)blockIdx.y * per_split;
    const int64_t s1 = min(s0 + per_split, ns_pad);
    for (int64_t base = s0; base < s1; base += UJ_TILE) {
        __syncthreads();
        tile[threadIdx.x] = src[base + threadIdx.x];
        __syncthreads();
        for (int j = 0; j < UJ_TILE; j++) {
            const SrcF64& s = tile[j];
            double o[7];
            adj_pair_f64<K>(tx - s.xy.x, ty - s.xy.y, tz - s.z_isig.x, s, Ub, Jb, wb, o);
            acc[0] += o[0]; acc[1] += o[1]; acc[2] += o[2];
            o[0] = -o[0]; o[1] = -o[1]; o[2] = -o[2];
#pragma unroll
            for (int k = 0; k < 7; k++) {
                double v = o[k];
#pragma unroll
                for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
                o[k] = v;
            }
            if (lane == 0) {
#pragma unroll
                for (int k = 0; k < 7; k++) red[warp][j][k] = o[k];
            }
        }
        __syncthreads();
        const int64_t si = base + threadIdx.x;
        if (si < ns) {
            double v[7];
#pragma unroll
            for (int k = 0; k < 7; k++) v[k] = red[0][threadIdx.x][k] + red[1][threadIdx.x][k] +
                                              red[2][threadIdx.x][k] + red[3][threadIdx.x][k];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                atomicAdd(&xbar[3 * si + k], v[k]);
                atomicAdd(&gbar[3 * si + k], v[3 + k]);
            }
            if (K != K_SING) atomicAdd(&sbar[si], v[6]);
        }
    }
    if (valid) {
#pragma unroll
        for (int k = 0; k < 3; k++) atomicAdd(&xbar[3 * idx + k], acc[k]);
    }
}

template <int K>
__global__ void pack_src_adj(int64_t ns, int64_t ns_pad, const double* __restrict__ xs,
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
    } else {  // padding: far away, no strength
        p.xy = make_double2(1.0e6, 1.0e6);
        p.z_isig = make_double2(1.0e6, 1.0);
        p.gxy = make_double2(0.0, 0.0);
        p.gz_sig = make_double2(0.0, 1.0);
    }
    out[i] = p;
}

template <int K>
static cudaError_t launch_adj_k(const AdjArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                                int64_t* launches)
{
    const int64_t ns_pad = (a.n + UJ_TILE - 1) / UJ_TILE * UJ_TILE;
    const int64_t nt_pad = (a.n + UJ_THREADS - 1) / UJ_THREADS * UJ_THREADS;
    const int nsplit = uj_num_splits(a.n, a.n, num_sms);
    const int64_t tiles = ns_pad / UJ_TILE;
    const int64_t per_split = ((tiles + nsplit - 1) / nsplit) * UJ_TILE;
    const TgtPos* tgt = nullptr;
    cudaError_t e = order_targets(a.n, a.x, w.order, w.order_bytes, st, launches, &tgt);
    if (e != cudaSuccess) return e;
    SrcF64* src = (SrcF64*)w.src_pack;
    pack_src_adj<K><<<(unsigned)((ns_pad + 255) / 256), 256, 0, st>>>(a.n, ns_pad, a.x, a.gam, a.sig, src);
    const dim3 grid((unsigned)(nt_pad / UJ_THREADS), (unsigned)nsplit);
    uj_adjoint_f64_kernel<K><<<grid, UJ_THREADS, 0, st>>>(a.n, tgt, a.Ubar, a.Jbar, a.n, ns_pad, src, per_split,
                                                          a.xbar, a.gbar, a.sbar);
    *launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_uj_adjoint(const AdjArgs& a, const Workspace& w, int num_sms, cudaStream_t st,
                              int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    switch (a.kernel) {
    case K_SING: return launch_adj_k<K_SING>(a, w, num_sms, st, launches);
    case K_GAUS: return launch_adj_k<K_GAUS>(a, w, num_sms, st, launches);
    case K_GAUSERF: return launch_adj_k<K_GAUSERF>(a, w, num_sms, st, launches);
    case K_WNKLMNS: return launch_adj_k<K_WNKLMNS>(a, w, num_sms, st, launches);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vpm
