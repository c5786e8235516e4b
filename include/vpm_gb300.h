/*
 * vpm_gb300.h -- C ABI of the GB300-native UJ evaluator for FLOWVPM.jl particle
 * fields (libvpm_gb300.so).
 *
 * The library replaces the particle-to-particle evaluation behind the
 * `pfield.UJ` hook of FLOWVPM.jl (struct field `UJ::TUJ`,
 * src/FLOWVPM_particlefield.jl:81,127): the all-pairs regularized Biot-Savart
 * sum of velocity U and velocity gradient J (src/FLOWVPM_fmm.jl:102-168), the
 * SFS vortex-stretching pass Estr (src/FLOWVPM_subfilterscale_models.jl:16-92),
 * their reverse-mode adjoint (replacing src/FLOWVPM_rrules.jl:179-330) and the
 * near-field leaf-pair P2P leg of UJ_fmm (src/FLOWVPM_UJ.jl:90-125).
 *
 * Conventions shared by every entry point:
 *   - Plain pointers and sizes only; no exceptions cross the ABI.
 *   - Every call returns an int status: 0 = VPM_OK, negative = error.  The text
 *     of the last error of a context is returned by vpm_last_error().
 *   - Calls are synchronous on return (like the reference, which calls UJ
 *     serially from the main task), unless the name ends in `_async`.
 *   - A context is bound to one CUDA device and one stream and serialises its
 *     calls with a mutex.  Different contexts may be used from different
 *     threads.
 *   - Host particle matrices use the reference layout: column-major
 *     Matrix{Float64}(46, maxparticles), one 46-row column per particle
 *     (src/FLOWVPM_particlefield.jl:11,134,239-252).  Row numbers below are the
 *     reference's 1-based rows.
 *   - "_dev" entry points take device pointers (e.g. torch CUDA tensors).
 *     Particle vectors are per-particle interleaved: x[3*i+k], gamma[3*i+k],
 *     U[3*i+k], J[9*i + (k + 3*l)] = dU_k/dx_l (column-major 3x3, the same
 *     order as rows 16:24 of the reference, src/FLOWVPM_fmm.jl:160).
 */
#ifndef VPM_GB300_H
#define VPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VPM_ABI_VERSION 1
#define VPM_NFIELDS 46   /* rows per particle, src/FLOWVPM_particlefield.jl:11 */

typedef struct vpm_ctx vpm_ctx;

/* status codes */
enum {
    VPM_OK            =  0,
    VPM_ERR_ARG       = -1,  /* bad pointer, size, id or flag */
    VPM_ERR_CAPACITY  = -2,  /* device memory could not be grown to the request */
    VPM_ERR_CUDA      = -3,  /* a CUDA runtime call failed */
    VPM_ERR_NONFINITE = -4,  /* NaN/Inf found in an input or an output */
    VPM_ERR_TIMEOUT   = -5,  /* a bounded device wait gave up */
    VPM_ERR_NODEVICE  = -6,  /* no CUDA device / wrong architecture */
    VPM_ERR_STATE     = -7   /* context used after an unrecoverable error */
};

/* regularizing kernels, src/FLOWVPM.jl:129-132 (singular, gaussian,
 * gaussianerf, winckelmans); src/FLOWVPM_kernel.jl:45-84 */
enum {
    VPM_KERNEL_SINGULAR    = 0,
    VPM_KERNEL_GAUSSIAN    = 1,
    VPM_KERNEL_GAUSSIANERF = 2,
    VPM_KERNEL_WINCKELMANS = 3
};

/* arithmetic of the pair evaluation */
enum {
    VPM_FP64     = 0,  /* the reference's FP64 formula, FP64 throughout */
    VPM_FP32COMP = 1   /* FP32 pair math, double-float displacement, FP64 block reduction */
};

/* flags of vpm_uj, mirroring the keyword arguments of UJ_direct
 * (src/FLOWVPM_UJ.jl:21-37) and ParticleField.transposed */
enum {
    VPM_RESET      = 1,  /* reset=true: zero rows 10:27 of non-static particles first */
    VPM_RESET_SFS  = 2,  /* reset_sfs=true: zero rows 40:42 of non-static particles */
    VPM_SFS        = 4,  /* sfs=true: accumulate Estr into rows 40:42 after U,J */
    VPM_TRANSPOSED = 8,  /* transposed stretching scheme (pfield.transposed) */
    VPM_CHECK_FINITE = 16, /* scan outputs for NaN/Inf and return VPM_ERR_NONFINITE */
    /* near-field calls: reuse the context's last octree and leaf-pair lists when they were
     * built from the same x array, n, leaf_size and theta; the caller asserts that the
     * positions have not changed since (within one RK3 stage, for instance) */
    VPM_REUSE_LISTS = 256
};

/* flags of vpm_dynamic_after_dev (with VPM_TRANSPOSED), the settings of
 * DynamicSFS (src/FLOWVPM_subfilterscale.jl:204-268) */
enum {
    VPM_DYN_FORCE_POSITIVE   = 32,  /* force_positive: C = |C| */
    VPM_DYN_CLIP_BACKSCATTER = 64,  /* clipping_backscatter: C = 0 where C Gamma . SFS < 0 */
    VPM_DYN_SUBTRACT         = 128  /* M holds the test-filter values: subtract S(J) and SFS first */
};

/* Work per pair used for all throughput and roofline figures (flop: add, sub,
 * mul = 1, fma = 2; sqrt/exp/erf/reciprocals counted separately). */
#define VPM_FLOP_PER_UJ_PAIR   74
#define VPM_FLOP_PER_ESTR_PAIR 25
/* the reverse mode of a UJ pair (vpm_uj_adjoint_dev): the 7 derivatives of
 * Ubar.u + Jbar:j with respect to dx, Gamma and sigma, g, g' and g'' included */
#define VPM_FLOP_PER_UJ_ADJ_PAIR 186

/* ---------------------------------------------------------------- context */

/* Create a context on CUDA device `device`.  Fails with VPM_ERR_NODEVICE if
 * there is no device or it is not an sm_103 part. */
int vpm_ctx_create(vpm_ctx** out, int device);
int vpm_ctx_destroy(vpm_ctx* ctx);
/* Text of the last error of `ctx` (or, when ctx is NULL, of the calling
 * thread's last failed context-free call: vpm_ctx_create or
 * vpm_uj_dev_noalloc).  Valid until the next call on the same context. */
const char* vpm_last_error(const vpm_ctx* ctx);
/* Use `stream` (a cudaStream_t) for all later work of this context.  NULL
 * selects the context's own stream, a blocking stream: it is ordered with the
 * legacy default stream's work both ways.  To run on the legacy default stream
 * itself (a framework's stream 0), pass cudaStreamLegacy, not NULL. */
int vpm_ctx_set_stream(vpm_ctx* ctx, void* stream);
/* Bound, in seconds, on every host wait for device work of this context
 * (default 3600).  A wait that runs out returns VPM_ERR_TIMEOUT and marks the
 * context unusable. */
int vpm_ctx_set_timeout(vpm_ctx* ctx, double seconds);
/* Capacities, in pairs, of the near-field list builder's traversal buffers for
 * the next build of this context: node pairs of one frontier and near leaf
 * pairs (by default 40 n and 24 n, n >= 4096).  A build that overflows them
 * doubles them and traverses again, so they only trade device memory for
 * repeated traversals; the lists do not depend on them.  Library plumbing (the
 * reference's FastMultipole sizes its own lists). */
int vpm_ctx_set_near_capacity(vpm_ctx* ctx, int64_t frontier_pairs, int64_t near_pairs);
/* Library and ABI identification. */
int vpm_abi_version(void);
const char* vpm_build_info(void);
/* Number of kernel launches issued by this context since creation. */
int64_t vpm_launch_count(const vpm_ctx* ctx);
/* Measurement helper (no counterpart in the reference): FP32 FFMA throughput
 * of this device in TFLOP/s, from a pure FFMA-chain kernel timed with CUDA
 * events.  Used as the FP32-pipe roofline denominator. */
int vpm_probe_ffma(vpm_ctx* ctx, double* tflops);
/* The same for the FP64 pipe (pure DFMA chains): the roofline denominator of
 * the plain FP64 form. */
int vpm_probe_dfma(vpm_ctx* ctx, double* tflops);

/* -------------------------------------------------- reference-facing drop-in */

/* UJ_direct(pfield; sfs, reset, reset_sfs) on the host particle matrix.
 * Replaces src/FLOWVPM_UJ.jl:21-37 (pair math src/FLOWVPM_fmm.jl:102-168,
 * resets src/FLOWVPM_particlefield.jl:464-507, Estr
 * src/FLOWVPM_subfilterscale_models.jl:16-92).
 *   particles : host pointer, column-major ld x np doubles (ld must be 46)
 *   np        : number of particles in the field (pfield.np)
 * Semantics: if VPM_RESET, zero rows 10:27 of non-static particles; if
 * VPM_RESET_SFS, zero rows 40:42 of non-static particles; add U (rows 10:12)
 * and J (rows 16:24) induced on every particle by every particle, skipping
 * pairs with r^2 == 0; if VPM_SFS, then add Estr (rows 40:42) on non-static
 * targets from non-static sources, using the accumulated J. */
int vpm_uj(vpm_ctx* ctx, double* particles, int64_t ld, int64_t np,
           int kernel, int precision, int flags);

/* UJ_direct(source, target): U and J that field `src` induces on every
 * particle of field `tgt`, accumulated without reset.
 * Replaces src/FLOWVPM_UJ.jl:48-50. */
int vpm_uj_cross(vpm_ctx* ctx, const double* src, int64_t ld_src, int64_t ns,
                 double* tgt, int64_t ld_tgt, int64_t nt, int kernel, int precision);

/* ------------------------------------------------------ device-pointer API */

/* U[nt,3] += and J[nt,9] += the field of sources (xs, gs, sgs) at targets xt.
 * Pairs with r^2 == 0 are skipped (src/FLOWVPM_fmm.jl:118), so xt may alias xs.
 * Device pointers. */
int vpm_uj_dev(vpm_ctx* ctx, int64_t nt, const double* xt,
               int64_t ns, const double* xs, const double* gs, const double* sgs,
               double* U, double* J, int kernel, int precision);

/* SFS[nt,3] += Estr of sources on targets (src/FLOWVPM_subfilterscale_models.jl:16-41):
 *   SFS_t += zeta(r/sigma_s)/sigma_s^3 * (J_t - J_s)^T Gamma_s   (VPM_TRANSPOSED)
 *   SFS_t += zeta(r/sigma_s)/sigma_s^3 * (J_t - J_s)   Gamma_s   (otherwise)
 * static_t / static_s (may be NULL = none static) are 0/1 flags; static
 * targets are left untouched and static sources contribute nothing
 * (iterator default, src/FLOWVPM_particlefield.jl:368-373).  Device pointers. */
int vpm_estr_dev(vpm_ctx* ctx, int64_t nt, const double* xt, const double* Jt,
                 const uint8_t* static_t,
                 int64_t ns, const double* xs, const double* gs, const double* sgs,
                 const double* Js, const uint8_t* static_s,
                 double* SFS, int kernel, int precision, int flags);

/* Reverse mode of the self-induced UJ of one particle set (targets = sources):
 * given Ubar[n,3] = dL/dU and Jbar[n,9] = dL/dJ, adds dL/dx to xbar[n,3],
 * dL/dGamma to gbar[n,3] and dL/dsigma to sbar[n] (device pointers).
 * Replaces the unwired ChainRules rrule of src/FLOWVPM_rrules.jl:179-330 (the
 * pullback of U and J with respect to positions, strengths and core sizes).
 * precision must be VPM_FP64.  Source-side sums are added with atomics, so
 * their summation order (last bits) may differ between runs. */
int vpm_uj_adjoint_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                       const double* Ubar, const double* Jbar, double* xbar, double* gbar,
                       double* sbar, int kernel, int precision);

/* Reverse mode of the self-induced Estr of one particle set (targets = sources,
 * the pass of vpm_estr_dev): given SFSbar[n,3] = dL/dSFS, adds dL/dx to
 * xbar[n,3], dL/dGamma to gbar[n,3], dL/dsigma to sbar[n] and dL/dJ to
 * Jbar[n,9] (J enters Estr as an input: the caller chains Jbar into the UJ
 * adjoint).  static_flags (may be NULL) as in vpm_estr_dev: static particles
 * take no part and receive nothing.  flags: VPM_TRANSPOSED.  The reference's
 * rrule stops at "SFS pullback not implemented yet!"
 * (src/FLOWVPM_rrules.jl:153-157); this is that pullback, for
 * src/FLOWVPM_subfilterscale_models.jl:16-92.  Two passes over all pairs,
 * without atomics: results are deterministic.  Device pointers. */
int vpm_estr_adjoint_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                         const double* J, const uint8_t* static_flags, const double* SFSbar, double* xbar,
                         double* gbar, double* sbar, double* Jbar, int kernel, int precision, int flags);

/* The test-filter differences of the pseudo-three-level dynamic SFS procedure
 * (src/FLOWVPM_subfilterscale.jl:447-673) on device arrays, for one particle
 * set acting on itself (no static particles):
 *   dJ[n,9]   = J(alpha sigma) - J(sigma)
 *   dSFS[n,3] = SFS(alpha sigma; J + dJ) - SFS(sigma; J)
 * where J[n,9] is the caller's J at sigma and SFS(sigma'; J') is Estr with core
 * sizes sigma' and gradients J'.  The procedure forms M = S(J_alpha) - S(J)
 * and SFS_alpha - SFS from these (S the stretching, linear in J).  VPM_FP64
 * evaluates both filter widths and subtracts, as the reference does;
 * VPM_FP32COMP evaluates the differences directly from the kernels' g' and g''
 * (no difference of two FP32 sums), so they keep FP32 relative accuracy.
 * flags: VPM_TRANSPOSED.  0 < alpha < 1.  No counterpart in the reference (it
 * calls UJ twice). */
int vpm_dynamic_diff_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                         const double* J, double alpha, double* dJ, double* dSFS, int kernel, int precision,
                         int flags);

/* ------------------------------------------ per-particle work of a step */
/* The per-particle work of the rVPM RK3 step on device arrays (x, gam, U, SFS,
 * C [n,3]; J, M [n,9], J column-major 3x3 per particle; sig [n]), one fused
 * FP64 kernel each, in the reference's operation order.
 *
 * vpm_rk3_stage_dev: one stage (a, b) of update_particle_states
 * (src/FLOWVPM_timeintegration.jl:463-532) for ReformulatedVPM(f, g): M[0:3],
 * x from U + Uinf; M[3:6], gam from the stretching of J (flags: VPM_TRANSPOSED)
 * and, when SFS is given, the SFS term C[:,0] SFS sigma^3/zeta0 (C may then not
 * be NULL); M[7], sig.  nu >= 0 adds core spreading's stage
 * (src/FLOWVPM_viscous.jl:175-192): M[6] and sig = sqrt(sig^2 + b M[6]).
 * Uinf is a host array of 3.  No counterpart call in the reference (its loop). */
int vpm_rk3_stage_dev(vpm_ctx* ctx, int64_t n, double a, double b, double dt, const double* Uinf, double f,
                      double g, double zeta0, double nu, int flags, double* x, double* gam, double* sig,
                      const double* U, const double* J, const double* SFS, const double* C, double* M);

/* relax_pedrizzetti (src/FLOWVPM_relaxation.jl:62-81): gam = (1 - rlxf) gam +
 * rlxf |gam| w/|w|, w the vorticity of J, where |w| > 0. */
int vpm_relax_dev(vpm_ctx* ctx, int64_t n, double rlxf, const double* J, double* gam);

/* dynamicprocedure_pseudo3level_afterUJ (src/FLOWVPM_subfilterscale.jl:541-673)
 * with clipping_backscatter (:287-296): from the test-filter differences in
 * M[0:6] (or, with VPM_DYN_SUBTRACT, from the test-filter values there minus
 * the stretching of J and SFS) the coefficients C[:,0:3] are updated with
 * Lagrangian averaging (rlxf) and the bounds [minC, maxC]; M is zeroed.
 * flags: VPM_TRANSPOSED, VPM_DYN_*.  A NaN coefficient returns
 * VPM_ERR_NONFINITE (the reference's error()). */
int vpm_dynamic_after_dev(vpm_ctx* ctx, int64_t n, double alpha, double rlxf, double minC, double maxC,
                          double zeta0, int flags, const double* gam, const double* sig, const double* J,
                          const double* SFS, double* C, double* M);

/* zeta_direct(pfield) (src/FLOWVPM_viscous.jl:467-488), the RBF basis field of
 * core spreading: rows 16:18 (J[1:3]) of every particle, statics included, are
 * set to sum_s zeta(r/sigma_s)/sigma_s^3 Gamma_s over every source, the self
 * pair included.  Host 46-row matrix as vpm_uj; only rows 16:18 are written. */
int vpm_zeta(vpm_ctx* ctx, double* particles, int64_t ld_rows, int64_t np, int kernel, int precision);

/* The same sum on device arrays: W[nt,3] += sum_s zeta(|xt - xs|/sigma_s)/sigma_s^3 Gamma_s. */
int vpm_zeta_dev(vpm_ctx* ctx, int64_t nt, const double* xt, int64_t ns, const double* xs, const double* gs,
                 const double* sgs, double* W, int kernel, int precision);

/* Near-field leg of UJ_fmm (src/FLOWVPM_UJ.jl:90-125): builds an octree of the
 * n particles on the GPU (leaves of at most leaf_size particles,
 * 1 <= leaf_size <= 4096) and adds U[n,3], J[n,9] -- and, with VPM_SFS, Estr
 * into SFS[n,3] -- from the direct P2P of every leaf pair that fails the
 * multipole acceptance criterion theta * r < R1 + R2 (r: distance of the cell
 * centres, R: cell radii; src/FLOWVPM_particlefield.jl:28-36), as
 * FastMultipole's direct_list does.  The far field is not computed.  flags:
 * VPM_SFS, VPM_TRANSPOSED, VPM_REUSE_LISTS.  Device pointers; static_flags may be NULL.  stats
 * (may be NULL) receives {leaves, leaf pairs, particle pairs}.  The lists are
 * the ones vpm_leaflist_host builds, entry for entry. */
int vpm_p2p_leaflist_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                         const uint8_t* static_flags, double* U, double* J, double* SFS,
                         int leaf_size, double theta, int kernel, int precision, int flags,
                         int64_t* stats);

/* zeta_fmm(pfield) (src/FLOWVPM_viscous.jl:523-556): the RBF basis field over
 * the near field only (the reference's zeta_fmm evaluates FastMultipole's
 * direct_list and neglects the far field): W[n,3] += sum over the near leaf
 * pairs of vpm_p2p_leaflist_dev (same leaf_size, theta) of
 * zeta(r/sigma_s)/sigma_s^3 Gamma_s, every particle a target and the self pair
 * included.  Like the reference's loop it adds to W (the reference adds into
 * J[1:3] without zeroing them, unlike zeta_direct).  Device pointers; flags:
 * VPM_REUSE_LISTS; stats as vpm_p2p_leaflist_dev. */
int vpm_zeta_leaflist_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                          double* W, int leaf_size, double theta, int kernel, int precision, int flags,
                          int64_t* stats);

/* vpm_dynamic_diff_dev over the near field only: the differences of the two
 * evaluations of the near-field leg (vpm_p2p_leaflist_dev with VPM_SFS, same
 * leaf_size and theta) at core sizes alpha sigma and sigma, as the dynamic
 * procedure (src/FLOWVPM_subfilterscale.jl:447-673) takes them when UJ is
 * UJ_fmm.  J is the near-field J at sigma; dJ[n,9] and dSFS[n,3] are set.
 * flags: VPM_TRANSPOSED, VPM_REUSE_LISTS.
 * Static particles (static_flags, may be NULL) get no SFS, as in
 * vpm_p2p_leaflist_dev.  stats as there.  FP64 evaluates and subtracts;
 * FP32COMP evaluates the differences directly. */
int vpm_dynamic_diff_leaflist_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                                  const uint8_t* static_flags, const double* J, double alpha, double* dJ,
                                  double* dSFS, int leaf_size, double theta, int kernel, int precision, int flags,
                                  int64_t* stats);

/* The same near-field P2P over leaf-pair lists the caller supplies in host
 * memory (for instance FastMultipole's direct_list of the reference's own
 * tree): particle perm[p] is at tree position p (perm a permutation of
 * 0..n-1), leaf l holds the positions [leaf_begin[l], leaf_end[l]) (leaves
 * contiguous, non-empty, in order, covering 0..n-1), and its source leaves are
 * col[row[l] .. row[l+1]) (each row is sorted here; a repeated entry is an
 * error).  Other arguments as vpm_p2p_leaflist_dev; stats[2] receives the
 * particle pairs. */
int vpm_p2p_lists_dev(vpm_ctx* ctx, int64_t n, const double* x, const double* gam, const double* sig,
                      const uint8_t* static_flags, double* U, double* J, double* SFS,
                      const int32_t* perm, int64_t nleaves, const int64_t* leaf_begin,
                      const int64_t* leaf_end, const int64_t* row, const int32_t* col,
                      int kernel, int precision, int flags, int64_t* stats);

/* The octree leaf-pair lists of n positions, built on the host (no GPU).
 * Call once with perm == NULL to get sizes[0] = leaves, sizes[1] = leaf pairs;
 * then with perm[n], leaf_begin[leaves], leaf_end[leaves], row[leaves+1],
 * col[leaf pairs]: particle i of the tree order is perm[i], leaf l holds tree
 * positions [leaf_begin[l], leaf_end[l]), and its source leaves are
 * col[row[l] .. row[l+1]) in increasing order. */
int vpm_leaflist_host(int64_t n, const double* x, int leaf_size, double theta, int32_t* perm,
                      int64_t* leaf_begin, int64_t* leaf_end, int64_t* row, int32_t* col, int64_t* sizes);

/* The same lists built on the GPU from device positions x[n,3] (what
 * vpm_p2p_leaflist_dev uses), copied to the host arrays as vpm_leaflist_host
 * fills them.  sizes[0..2] = leaves, leaf pairs, particle pairs; with
 * perm == NULL only the sizes are returned. */
int vpm_leaflist_dev(vpm_ctx* ctx, int64_t n, const double* x, int leaf_size, double theta, int32_t* perm,
                     int64_t* leaf_begin, int64_t* leaf_end, int64_t* row, int32_t* col, int64_t* sizes);

/* ------------------------------------------------ allocation-free variant */

/* Size of the static device scratch array behind vpm_uj_dev_noalloc (64 MiB). */
#define VPM_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* vpm_uj_dev without any device allocation (no counterpart in the reference).
 * For callers that cannot call cudaMalloc -- their device memory is owned by
 * another allocator (a framework's caching pool, an arena reserved at
 * start-up) or they must not allocate once running.  Same arguments and
 * results as vpm_uj_dev, plus the caller's stream (a cudaStream_t; NULL = the
 * legacy default stream), on the current CUDA device, with no context.  The
 * call returns after the work on `stream` has finished.
 * Scratch lives in one file-scope __device__ array of VPM_NOALLOC_SCRATCH_BYTES
 * held by every GPU that loads it until the process exits; problems needing
 * more scratch than that (roughly N > 2^19 particles) return VPM_ERR_CAPACITY.
 * The first call on each device looks up the array's device address (with
 * that device current) and caches it.  All calls share the array: calls whose device work overlaps race on it.
 * Errors are described by vpm_last_error(NULL). */
int vpm_uj_dev_noalloc(int64_t nt, const double* xt,
                       int64_t ns, const double* xs, const double* gs, const double* sgs,
                       double* U, double* J, int kernel, int precision, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VPM_GB300_H */
