// step.cu -- the per-particle work of one rVPM RK3 step on device arrays, one
// fused FP64 kernel per stage update, per relaxation and per dynamic-procedure
// coefficient update (the pair sums around them are the other kernels of this
// library).  Each restates the reference's arithmetic in its order:
//   * rk3_stage_kernel: update_particle_states of the rVPM low-storage RK3,
//     src/FLOWVPM_timeintegration.jl:463-532 (stretching, the SFS term, the
//     sigma update), and core spreading's RK3 branch, src/FLOWVPM_viscous.jl:175-192;
//   * relax_kernel: relax_pedrizzetti, src/FLOWVPM_relaxation.jl:62-81;
//   * dynamic_after_kernel: dynamicprocedure_pseudo3level_afterUJ with Lagrangian
//     averaging, bounds and the NaN check, src/FLOWVPM_subfilterscale.jl:541-673,
//     and clipping_backscatter, :287-296.
// Layout: x, gam, U, SFS, C [n,3]; J, M [n,9] (J column-major 3x3 per particle);
// sig [n].  Bound: HBM (a few hundred bytes a particle, no reuse).
#include "../../include/vpm_gb300.h"
#include "internal.h"

#include <cmath>

namespace vpm {

constexpr int STEP_THREADS = 256;

// (Gamma . grad')U (transposed) or (Gamma . grad)U (classic) from J
__device__ __forceinline__ void stretch3(const double* J, const double* G, bool transposed, double (&S)[3])
{
    if (transposed) {
        for (int k = 0; k < 3; k++) S[k] = J[3 * k] * G[0] + J[3 * k + 1] * G[1] + J[3 * k + 2] * G[2];
    } else {
        for (int i = 0; i < 3; i++) S[i] = J[i] * G[0] + J[i + 3] * G[1] + J[i + 6] * G[2];
    }
}

__global__ void __launch_bounds__(STEP_THREADS)
rk3_stage_kernel(int64_t n, double a, double b, double dt, double3 uinf, double zf, double zc, double zeta0,
                 double nu, bool transposed, double* __restrict__ x, double* __restrict__ gam,
                 double* __restrict__ sig, const double* __restrict__ U, const double* __restrict__ J,
                 const double* __restrict__ SFS, const double* __restrict__ C, double* __restrict__ M)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* m = M + 9 * i;
    double* X = x + 3 * i;
    double G[3] = {gam[3 * i], gam[3 * i + 1], gam[3 * i + 2]};
    const double ui[3] = {uinf.x, uinf.y, uinf.z};
    for (int k = 0; k < 3; k++) {
        m[k] = a * m[k] + dt * (U[3 * i + k] + ui[k]);
        X[k] += b * m[k];
    }
    double S[3];
    stretch3(J + 9 * i, G, transposed, S);
    const double gn2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
    const double s = sig[i];
    const double s3 = s * s * s;
    const double Ci = C ? C[3 * i] : 0.0;
    const double F[3] = {SFS ? SFS[3 * i] : 0.0, SFS ? SFS[3 * i + 1] : 0.0, SFS ? SFS[3 * i + 2] : 0.0};
    double mm4 = zf * (S[0] * G[0] + S[1] * G[1] + S[2] * G[2]);
    mm4 = mm4 - zc * (Ci * F[0] * G[0] + Ci * F[1] * G[1] + Ci * F[2] * G[2]) * s3 / zeta0;
    mm4 = gn2 > 0.0 ? mm4 / gn2 : 0.0;
    for (int k = 0; k < 3; k++) m[3 + k] = a * m[3 + k] + dt * (S[k] - 3.0 * mm4 * G[k] - Ci * F[k] * s3 / zeta0);
    m[7] = a * m[7] - dt * (s * mm4);
    for (int k = 0; k < 3; k++) gam[3 * i + k] = G[k] + b * m[3 + k];
    double sn = s + b * m[7];
    if (nu >= 0.0) {   // core spreading: d(sigma^2)/dt = 2 nu
        m[6] = a * m[6] + dt * 2.0 * nu;
        sn = sqrt(sn * sn + b * m[6]);
    }
    sig[i] = sn;
}

__global__ void __launch_bounds__(STEP_THREADS)
relax_kernel(int64_t n, double rlxf, const double* __restrict__ J, double* __restrict__ gam)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* j = J + 9 * i;
    const double w[3] = {j[5] - j[7], j[6] - j[2], j[1] - j[3]};   // vorticity from the velocity gradient
    const double nw = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (nw == 0.0) return;
    double* G = gam + 3 * i;
    const double nG = sqrt(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
    for (int k = 0; k < 3; k++) G[k] = (1.0 - rlxf) * G[k] + rlxf * (nG / nw) * w[k];
}

__device__ __forceinline__ double sgn(double v) { return v > 0.0 ? 1.0 : (v < 0.0 ? -1.0 : 0.0); }

__global__ void __launch_bounds__(STEP_THREADS)
dynamic_after_kernel(int64_t n, double alpha, double rlxf, double minC, double maxC, double zeta0, int flags,
                     const double* __restrict__ gam, const double* __restrict__ sig, const double* __restrict__ J,
                     const double* __restrict__ SFS, double* __restrict__ C, double* __restrict__ M,
                     int* __restrict__ nan_flag)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double G[3] = {gam[3 * i], gam[3 * i + 1], gam[3 * i + 2]};
    double* m = M + 9 * i;
    double* c = C + 3 * i;
    const double* F = SFS + 3 * i;
    if (flags & VPM_DYN_SUBTRACT) {   // M holds the test-filter values: take the differences
        double S[3];
        stretch3(J + 9 * i, G, (flags & VPM_TRANSPOSED) != 0, S);
        for (int k = 0; k < 3; k++) { m[k] -= S[k]; m[3 + k] -= F[k]; }
    }
    const double s = sig[i];
    double nume = (m[0] * G[0] + m[1] * G[1] + m[2] * G[2]) * (3.0 * alpha - 2.0);
    double deno = (m[3] * G[0] + m[4] * G[1] + m[5] * G[2]) / (zeta0 / (s * s * s));
    double c3 = c[2] == 0.0 ? deno : c[2];
    c3 = c3 == 0.0 ? 2.220446049250313e-16 : c3;
    nume = rlxf * nume + (1.0 - rlxf) * c[1];
    deno = rlxf * deno + (1.0 - rlxf) * c3;
    const double ratio = fabs(nume / deno);
    const bool big = ratio > maxC;
    if (big && fabs(deno) < fabs(c3)) deno = sgn(deno) * fabs(c3);
    if (big && fabs(nume / deno) >= maxC) nume = sgn(nume) * fabs(deno) * maxC;
    if (!big && ratio < minC) nume = sgn(nume) * fabs(deno) * minC;
    double c1 = nume / deno;
    if (isnan(c1)) atomicExch(nan_flag, 1);
    if (flags & VPM_DYN_FORCE_POSITIVE) c1 = c1 * sgn(c1);
    c[0] = c1;
    c[1] = nume;
    c[2] = deno;
    for (int k = 0; k < 9; k++) m[k] = 0.0;
    if ((flags & VPM_DYN_CLIP_BACKSCATTER) && c[0] * (G[0] * F[0] + G[1] * F[1] + G[2] * F[2]) < 0.0)
        c[0] = c[0] * 0.0;
}

static unsigned blocks(int64_t n) { return (unsigned)((n + STEP_THREADS - 1) / STEP_THREADS); }

cudaError_t launch_rk3_stage(const StageArgs& a, cudaStream_t st, int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    const double zf = (a.f + a.g) / (1.0 + 3.0 * a.f), zc = a.f / (1.0 + 3.0 * a.f);
    rk3_stage_kernel<<<blocks(a.n), STEP_THREADS, 0, st>>>(
        a.n, a.a, a.b, a.dt, make_double3(a.uinf[0], a.uinf[1], a.uinf[2]), zf, zc, a.zeta0, a.nu, a.transposed,
        a.x, a.gam, a.sig, a.U, a.J, a.SFS, a.C, a.M);
    *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_relax(int64_t n, double rlxf, const double* J, double* gam, cudaStream_t st, int64_t* launches)
{
    if (n <= 0) return cudaSuccess;
    relax_kernel<<<blocks(n), STEP_THREADS, 0, st>>>(n, rlxf, J, gam);
    *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_dynamic_after(const DynAfterArgs& a, int* nan_flag, cudaStream_t st, int64_t* launches)
{
    if (a.n <= 0) return cudaSuccess;
    dynamic_after_kernel<<<blocks(a.n), STEP_THREADS, 0, st>>>(a.n, a.alpha, a.rlxf, a.minC, a.maxC, a.zeta0,
                                                               a.flags, a.gam, a.sig, a.J, a.SFS, a.C, a.M,
                                                               nan_flag);
    *launches += 1;
    return cudaGetLastError();
}

}  // namespace vpm
