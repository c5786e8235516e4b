/*
 * vpm_oracle.h -- CPU oracle for the UJ hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C (C99 + OpenMP) restatement of FLOWVPM.jl v4.0.3's UJ_direct and the
 * consumers around it, used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py as the checker.  The product path
 * (libvpm_gb300.so) never links or calls it.
 *
 * Every function cites the reference file:line it restates.  All arithmetic is
 * FP64 in the reference's operation order; build with -ffp-contract=off so no
 * FMA contraction changes the rounding (Julia does not contract either).
 *
 * Parity pinning: the reference (Julia + FastMultipole.jl) cannot run in this
 * build environment, so no reference-produced UJ vectors exist.  The oracle is
 * pinned to the reference's own known-answer checks instead: the analytic
 * singular-pair formulas of scripts/check_fmm.jl:39-71 and the vortex-ring
 * velocity test of test/runtests_singlevortexring.jl:124-149 (see tests/).
 */
#ifndef VPM_ORACLE_H
#define VPM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* kernel ids and flags are the library's (include/vpm_gb300.h) */

/* erf after the reference's custom_erf64 (src/FLOWVPM_gpu_erf.jl:160-191),
 * the published fdlibm s_erf.c rational approximations. */
double oracle_erf_ref(double x);
/* (g, dg/dr) of a kernel at r = |x|/sigma, src/FLOWVPM_kernel.jl:45-84 */
void oracle_g_dgdr(int kernel, double r, double* g, double* dg);
/* zeta(r) of a kernel, src/FLOWVPM_kernel.jl:45-76 */
double oracle_zeta(int kernel, double r);

/* UJ_direct(pfield; sfs, reset, reset_sfs) on a column-major ld x np matrix
 * (ld = 46).  src/FLOWVPM_UJ.jl:21-37.  flags: VPM_RESET, VPM_RESET_SFS,
 * VPM_SFS, VPM_TRANSPOSED.  erf_mode 0 = reference custom_erf64, 1 = libm erf.
 * Returns 0, or -1 on a bad argument. */
int oracle_uj_direct(double* P, int64_t ld, int64_t np, int kernel, int flags,
                     int erf_mode, int nthreads);

/* U[nt*3] += and J[nt*9] += from sources (xs, gs, sgs): the pair loop of
 * src/FLOWVPM_fmm.jl:102-168, per target in source-index order.
 * compensated=1 sums with Neumaier compensation (a "truth" mode).
 * Targets [t0, t1) only, so a caller can time or check a subset. */
void oracle_uj_pairs(int64_t t0, int64_t t1, const double* xt,
                     int64_t ns, const double* xs, const double* gs, const double* sgs,
                     double* U, double* J, int kernel, int erf_mode, int compensated,
                     int nthreads);

/* SFS[nt*3] += Estr, src/FLOWVPM_subfilterscale_models.jl:16-41,61-74.
 * static_t/static_s may be NULL. transposed selects the scheme. */
void oracle_estr_pairs(int64_t t0, int64_t t1, const double* xt, const double* Jt,
                       const uint8_t* static_t,
                       int64_t ns, const double* xs, const double* gs, const double* sgs,
                       const double* Js, const uint8_t* static_s,
                       double* SFS, int kernel, int transposed, int nthreads);

/* zeta_direct: W_t += sum_s zeta(r/sigma_s)/sigma_s^3 Gamma_s, self pair included
 * (src/FLOWVPM_viscous.jl:467-488). */
void oracle_zeta_pairs(int64_t t0, int64_t t1, const double* xt, int64_t ns, const double* xs,
                       const double* gs, const double* sgs, double* W, int kernel, int nthreads);

/* Reverse mode of oracle_uj_pairs over one particle set (targets = sources,
 * pairs with r^2 == 0 skipped): given Ubar[n*3] = dL/dU and Jbar[n*9] = dL/dJ,
 * adds dL/dx to xbar[n*3], dL/dGamma to gbar[n*3] and dL/dsigma to sbar[n].
 * The per-pair derivative follows from differentiating src/FLOWVPM_fmm.jl:112-160
 * (it replaces the unwired rrule of src/FLOWVPM_rrules.jl:179-330), with the
 * kernels' second derivatives g''(rho).  FP64, targets in parallel, sources in
 * index order; source-side sums are accumulated per source in target order. */
void oracle_uj_adjoint(int64_t n, const double* x, const double* gam, const double* sig,
                       const double* Ubar, const double* Jbar, double* xbar, double* gbar,
                       double* sbar, int kernel, int nthreads);
/* Reverse mode of the self-induced Estr (src/FLOWVPM_subfilterscale_models.jl:16-92):
 * given Sbar[n,3] = dL/dSFS, adds dL/dx, dL/dGamma, dL/dsigma and dL/dJ to
 * xb[n,3], gb[n,3], sb[n], Jb[n,9]; st[n] static flags (may be NULL). */
void oracle_estr_adjoint(int64_t n, const double* x, const double* gam, const double* sig, const double* J,
                         const uint8_t* st, const double* Sbar, double* xb, double* gb, double* sb, double* Jb,
                         int kernel, int transposed, int nthreads);
/* (g, g', g'') of a kernel at rho (libm erf). */
void oracle_g_d1_d2(int kernel, double rho, double* g, double* d1, double* d2);

/* ---------------------------------------------- consumers of UJ (per particle) */

/* update_particle_states, rVPM low-storage RK stage,
 * src/FLOWVPM_timeintegration.jl:463-532 */
void oracle_update_particle_states(double* P, int64_t ld, int64_t np, double a, double b,
                                   double dt, const double* Uinf, double f, double g,
                                   double zeta0, int transposed);
/* relax_pedrizzetti / relax_correctedpedrizzetti on non-static particles,
 * src/FLOWVPM_relaxation.jl:62-81,112-142 */
void oracle_relax(double* P, int64_t ld, int64_t np, double rlxf, int corrected);

/* Settings of one rVPM RK3 step (src/FLOWVPM_timeintegration.jl:388-461). */
typedef struct {
    int kernel;          /* VPM_KERNEL_* */
    int transposed;      /* pfield.transposed */
    double f, g;         /* ReformulatedVPM(f, g), src/FLOWVPM_formulation.jl:31-37 */
    double Uinf[3];      /* freestream */
    int relaxation;      /* 0 none, 1 pedrizzetti, 2 correctedpedrizzetti */
    double rlxf;         /* relaxation factor */
    int sfs;             /* 0 NoSFS, 1 ConstantSFS, 2 DynamicSFS (pseudo3level) */
    double Cs;           /* ConstantSFS coefficient */
    double alpha, sfs_rlxf, minC, maxC; /* DynamicSFS, src/FLOWVPM_subfilterscale.jl:162-191 */
    int force_positive;  /* pseudo3level_positive_afterUJ */
    int clip_backscatter;/* clippings=(clipping_backscatter,) */
    int viscous;         /* 0 Inviscid, 1 CoreSpreading */
    double nu, sgm0, beta;
    double t_sgm;        /* CoreSpreading timer, updated by the step */
    int erf_mode;
    int nthreads;
} oracle_step_params;

/* One rungekutta3 step with UJ = the oracle's UJ_direct.
 * Returns 0; -2 if a core-spreading reset would be needed (zeta/RBF are not
 * restated); -3 on a NaN in the dynamic procedure (src/FLOWVPM_subfilterscale.jl:645-652). */
int oracle_rk3_step(double* P, int64_t ld, int64_t np, double dt, int relax,
                    oracle_step_params* prm);

#ifdef __cplusplus
}
#endif
#endif
