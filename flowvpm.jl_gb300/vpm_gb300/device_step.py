"""Device-resident rVPM time step: the particle state stays in GPU memory
across a step and between steps, and every particle-to-particle evaluation is a
call into libvpm_gb300 (all pairs, or the near-field leaf pairs).

The per-particle work around UJ is the reference's, restated on float64 CUDA
tensors in the reference's operation order:
  * rVPM low-storage RK3, src/FLOWVPM_timeintegration.jl:388-532;
  * the pseudo-three-level dynamic SFS procedure with Lagrangian averaging,
    bounds and the NaN check, src/FLOWVPM_subfilterscale.jl:447-673, and
    backscatter clipping, :287-296;
  * core spreading (RK3 branch), src/FLOWVPM_viscous.jl:175-220, with the
    core-size reset: zeta_direct (src/FLOWVPM_viscous.jl:467-488, through
    vpm_zeta_dev) and the RBF conjugate gradient (:314-454);
  * Pedrizzetti relaxation, src/FLOWVPM_relaxation.jl:62-81.
Static particles are not supported in this form (the host mirror has them).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from . import _lib
from .autodiff import STAGES, _stretch

EPS = 2.220446049250313e-16


@dataclass
class DeviceField:
    """SoA particle state on the device (float64), the rows of the reference's
    particle matrix that the step uses."""
    x: torch.Tensor            # [n,3]  X
    gam: torch.Tensor          # [n,3]  Gamma
    sig: torch.Tensor          # [n]    sigma
    kernel: int = _lib.KERNEL_GAUSSIANERF
    precision: int = _lib.FP32COMP
    f: float = 0.0             # ReformulatedVPM(f, g)
    g: float = 0.2
    transposed: bool = True
    t: float = 0.0
    nt: int = 0
    U: torch.Tensor = None     # [n,3]
    J: torch.Tensor = None     # [n,9]
    SFS: torch.Tensor = None   # [n,3]
    C: torch.Tensor = None     # [n,3]  C_INDEX rows (coefficient, Lagrangian numerator, denominator)
    M: torch.Tensor = None     # [n,9]  M_INDEX rows
    vol: torch.Tensor = None   # [n]    particle volumes (the RBF initial guess of a core-size reset)
    # near-field evaluation instead of all pairs (FMM near field: leaf size, theta)
    leaflist: tuple | None = None

    def __post_init__(self):
        n = self.x.shape[0]
        z = lambda k: torch.zeros(n, k, dtype=torch.float64, device=self.x.device)
        self.U = z(3) if self.U is None else self.U
        self.J = z(9) if self.J is None else self.J
        self.SFS = z(3) if self.SFS is None else self.SFS
        self.C = z(3) if self.C is None else self.C
        self.M = z(9) if self.M is None else self.M

    @property
    def n(self) -> int:
        return self.x.shape[0]


def uj(fld: DeviceField, ctx: _lib.Context, *, sfs: bool = False, reset: bool = True, reset_sfs: bool = False):
    """UJ_direct semantics on the device state (no static particles)."""
    if reset:
        fld.U.zero_()
        fld.J.zero_()
    if reset_sfs:
        fld.SFS.zero_()
    if fld.leaflist is None:
        ctx.uj_dev(fld.x, fld.x, fld.gam, fld.sig, fld.U, fld.J, fld.kernel, fld.precision)
        if sfs:
            ctx.estr_dev(fld.x, fld.J, fld.x, fld.gam, fld.sig, fld.J, fld.SFS, fld.kernel, fld.precision,
                         fld.transposed)
    else:
        leaf_size, theta = fld.leaflist
        ctx.p2p_leaflist_dev(fld.x, fld.gam, fld.sig, fld.U, fld.J, fld.SFS if sfs else None, leaf_size=leaf_size,
                             theta=theta, kernel=fld.kernel, precision=fld.precision, sfs=sfs,
                             transposed=fld.transposed)


@dataclass
class DynamicSFSParams:
    """DynamicSFS settings; defaults = SFS_Cd_twolevel_nobackscatter (src/FLOWVPM.jl:223).

    fused: with FP32-comp pair sums, take the test-filter differences from
    vpm_dynamic_diff_dev, or vpm_dynamic_diff_leaflist_dev for a near-field
    state (evaluated as differences, FP32 relative accuracy)
    instead of subtracting two separate evaluations (the reference's way,
    whose FP32 rounding the 1e-3 differences amplify to 1e-4 .. 1e-2)."""
    alpha: float = 0.999
    rlxf: float = 0.005
    minC: float = 0.0
    maxC: float = 1.0
    force_positive: bool = True
    clip_backscatter: bool = True
    fused: bool = True


@dataclass
class CoreSpreadingParams:
    """CoreSpreading(nu, sgm0; beta, itmax, tol, iterror), src/FLOWVPM_viscous.jl:62-112."""
    nu: float
    sgm0: float
    beta: float = 1.5
    t_sgm: float = 0.0
    itmax: int = 15
    tol: float = 1e-3
    iterror: bool = True


def zeta(fld: DeviceField, ctx: _lib.Context, reuse: bool = False) -> torch.Tensor:
    """zeta_direct: W[n,3] = sum_s zeta(r/sigma_s)/sigma_s^3 Gamma_s (self pair included);
    for a near-field state, zeta_fmm's sum over the near leaf pairs, into a zeroed W
    (the reference's zeta_fmm adds to J[1:3] without zeroing them; the conjugate
    gradient here takes each evaluation on its own, as with zeta_direct).  reuse: the
    positions are those of the previous near-field call (VPM_REUSE_LISTS)."""
    W = torch.zeros_like(fld.gam)
    if fld.leaflist is None:
        ctx.zeta_dev(fld.x, fld.x, fld.gam, fld.sig, W, fld.kernel, fld.precision)
    else:
        leaf_size, theta = fld.leaflist
        ctx.zeta_leaflist_dev(fld.x, fld.gam, fld.sig, W, leaf_size=leaf_size, theta=theta, kernel=fld.kernel,
                              precision=fld.precision, reuse=reuse)
    return W


def rbf_conjugategradient(fld: DeviceField, ctx: _lib.Context, target: torch.Tensor, p: CoreSpreadingParams):
    """src/FLOWVPM_viscous.jl:314-454 per component on device tensors: new
    strengths whose basis field reproduces `target` (to the relative residual tol)."""
    if fld.vol is None:
        raise ValueError("a core-size reset needs the particle volumes (DeviceField.vol)")
    tiny = 2 * EPS
    x = target * fld.vol[:, None]                 # x0 = omega_targ * vol
    fld.gam.copy_(x)
    r = target - zeta(fld, ctx)                   # r0 = b - A x0 (builds the lists at these positions)
    fld.gam.copy_(r)                              # p0 = r0
    rr0s = (r * r).sum(0).tolist()
    rrs = list(rr0s)
    flags = [math.sqrt(a) > p.tol or (a != 0 and math.sqrt(b / a) > p.tol) for a, b in zip(rr0s, rrs)]
    for it in range(1, int(p.itmax) + 1):
        if not any(flags):
            break
        Ap = zeta(fld, ctx, reuse=True)           # the positions do not move during the solve
        pAps = (fld.gam * Ap).sum(0).tolist()
        alphas = torch.tensor([rrs[i] / pAps[i] * flags[i] if flags[i] else 0.0 for i in range(3)],
                              dtype=torch.float64, device=x.device)
        prev_rrs = rrs
        x += alphas * fld.gam
        r -= alphas * Ap
        rrs = (r * r).sum(0).tolist()
        betas = [1.0 if abs(prev_rrs[i]) <= tiny else rrs[i] / prev_rrs[i] for i in range(3)]
        fld.gam.copy_(r + torch.tensor(betas, dtype=torch.float64, device=x.device) * fld.gam)
        flags = [flags[i] and (False if abs(rr0s[i]) <= tiny else math.sqrt(rrs[i] / rr0s[i]) > p.tol)
                 for i in range(3)]
        if it == p.itmax and any(flags) and p.iterror:
            raise RuntimeError(f"Maximum number of iterations {p.itmax} reached before convergence. "
                               f"Errors: {[math.sqrt(a / b) for a, b in zip(rrs, rr0s)]}, tolerance:{p.tol}")
    fld.gam.copy_(x)


def _zeta0(kernel: int) -> float:
    from .particlefield import standard_kernels
    return standard_kernels[kernel].zeta(0.0)


def _dynamic_before(fld, ctx, p: DynamicSFSParams):
    fld.sig *= p.alpha
    uj(fld, ctx, sfs=True, reset=True, reset_sfs=True)
    fld.M.zero_()
    fld.M[:, 0:3] = _stretch(fld.J, fld.gam, fld.transposed)
    fld.M[:, 3:6] = fld.SFS
    fld.sig /= p.alpha


def _dynamic_fused(fld, ctx, p: DynamicSFSParams):
    """M[0:3] = S(J_alpha) - S(J) and M[3:6] = SFS_alpha - SFS from the directly
    evaluated differences (after the stage's own UJ + Estr at sigma)."""
    dJ = torch.zeros_like(fld.J)
    dS = torch.zeros_like(fld.SFS)
    if fld.leaflist is None:
        ctx.dynamic_diff_dev(fld.x, fld.gam, fld.sig, fld.J, p.alpha, dJ, dS, fld.kernel, fld.precision,
                             fld.transposed)
    else:
        leaf_size, theta = fld.leaflist
        # the stage's UJ call has just built the lists at these positions
        ctx.dynamic_diff_leaflist_dev(fld.x, fld.gam, fld.sig, fld.J, p.alpha, dJ, dS, leaf_size=leaf_size,
                                      theta=theta, kernel=fld.kernel, precision=fld.precision,
                                      transposed=fld.transposed, reuse=True)
    fld.M.zero_()
    fld.M[:, 0:3] = _stretch(dJ, fld.gam, fld.transposed)
    fld.M[:, 3:6] = dS


def _dynamic_after(fld, ctx, p: DynamicSFSParams, zeta0: float, subtract: bool = True):
    """dynamicprocedure_pseudo3level_afterUJ + clipping_backscatter (vpm_dynamic_after_dev):
    with subtract, M holds the test-filter values; otherwise the differences."""
    ctx.dynamic_after_dev(p.alpha, p.rlxf, p.minC, p.maxC, zeta0, fld.gam, fld.sig, fld.J, fld.SFS, fld.C, fld.M,
                          force_positive=p.force_positive, clip_backscatter=p.clip_backscatter, subtract=subtract,
                          transposed=fld.transposed)


def rk3_step(fld: DeviceField, dt: float, ctx: _lib.Context, *, sfs: DynamicSFSParams | None = None,
             viscous: CoreSpreadingParams | None = None, relax_rlxf: float | None = None,
             Uinf=(0.0, 0.0, 0.0)):
    """One rungekutta3 step (+ relaxation when relax_rlxf is given) of the device state."""
    zeta0 = _zeta0(fld.kernel)
    f, g = fld.f, fld.g
    fld.M.zero_()
    fused = sfs is not None and sfs.fused and fld.precision == _lib.FP32COMP
    for a, b in STAGES:
        first = (a == 1 or a == 0)
        if sfs is not None and first and not fused:
            _dynamic_before(fld, ctx, sfs)
        uj(fld, ctx, sfs=sfs is not None, reset=True, reset_sfs=sfs is not None)
        if sfs is not None and first:
            if fused:
                _dynamic_fused(fld, ctx, sfs)
            _dynamic_after(fld, ctx, sfs, zeta0, subtract=not fused)
        # update_particle_states (src/FLOWVPM_timeintegration.jl:463-532) and core spreading's
        # stage (src/FLOWVPM_viscous.jl:175-192): one fused kernel
        with_sfs = sfs is not None
        ctx.rk3_stage_dev(a, b, dt, Uinf, f, g, zeta0, fld.x, fld.gam, fld.sig, fld.U, fld.J, fld.M,
                          SFS=fld.SFS if with_sfs else None, C=fld.C if with_sfs else None,
                          nu=viscous.nu if viscous is not None else None, transposed=fld.transposed)
        if viscous is not None:   # core spreading's growth timer, after the last stage
            if abs(b - 8 / 15) <= 1e-7:
                viscous.t_sgm += dt
                beta = math.sqrt(2 * viscous.nu * viscous.t_sgm / viscous.sgm0 ** 2 + 1)
                if beta >= viscous.beta:   # core-size reset (src/FLOWVPM_viscous.jl:199-219)
                    target = zeta(fld, ctx)
                    fld.sig.fill_(viscous.sgm0)
                    rbf_conjugategradient(fld, ctx, target, viscous)
                    viscous.t_sgm = 0.0
    if relax_rlxf is not None:   # relax_pedrizzetti (src/FLOWVPM_relaxation.jl:62-81)
        uj(fld, ctx)
        ctx.relax_dev(relax_rlxf, fld.J, fld.gam)
    fld.t += dt
    fld.nt += 1


def impulse(fld: DeviceField) -> torch.Tensor:
    """Linear impulse I = 1/2 sum x_p x Gamma_p."""
    return 0.5 * torch.cross(fld.x, fld.gam, dim=1).sum(0)


def energy(fld: DeviceField) -> float:
    """Kinetic-energy estimate E = 1/2 sum U_p . (x_p x Gamma_p), from the U of the last evaluation."""
    return float(0.5 * (fld.U * torch.cross(fld.x, fld.gam, dim=1)).sum())
