"""Host-side mirror of the reference's consumers of UJ: the rVPM low-storage RK3
(src/FLOWVPM_timeintegration.jl:388-532) and first-order Euler (:23-37,103-173), relaxation
(src/FLOWVPM_relaxation.jl), the SFS schemes with the pseudo-three-level dynamic
procedure (src/FLOWVPM_subfilterscale.jl) and the core-spreading viscous scheme
(src/FLOWVPM_viscous.jl:152-223).

These run per particle, O(N), vectorised over the non-static particles with
numpy in the reference's operation order; every particle-to-particle
evaluation goes through `pfield.UJ` -- the GB300 kernels when the field was
built with UJ=UJ_gb300.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .particlefield import (C_INDEX, GAMMA_INDEX, J_INDEX, M_INDEX, SFS_INDEX, SIGMA_INDEX,
                            STATIC_INDEX, U_INDEX, VOL_INDEX, X_INDEX, ClassicVPM, ParticleField,
                            ReformulatedVPM, _reset_particles)

EPS = 2.220446049250313e-16  # Julia eps()


def _live(pfield: ParticleField) -> np.ndarray:
    return np.nonzero(pfield.particles[STATIC_INDEX, :pfield.np] == 0)[0]


def _stretch(J, G, transposed: bool):
    """(Gamma . grad')U (transposed) or (Gamma . grad)U; J rows are column-major 3x3."""
    if transposed:
        return (J[0] * G[0] + J[1] * G[1] + J[2] * G[2],
                J[3] * G[0] + J[4] * G[1] + J[5] * G[2],
                J[6] * G[0] + J[7] * G[1] + J[8] * G[2])
    return (J[0] * G[0] + J[3] * G[1] + J[6] * G[2],
            J[1] * G[0] + J[4] * G[1] + J[7] * G[2],
            J[2] * G[0] + J[5] * G[1] + J[8] * G[2])


# ------------------------------------------------------------------ viscous
@dataclass
class Inviscid:
    """src/FLOWVPM_viscous.jl:38-58"""
    nu: float = 0.0


@dataclass
class CoreSpreading:
    """Core spreading, src/FLOWVPM_viscous.jl:62-223: RK3 spreading of the core
    sizes and, once sigma/sgm0 reaches beta, the core-size reset -- the basis
    field of the current strengths (`zeta`, default zeta_gb300 = zeta_direct on
    the GB300) becomes the target vorticity, sigma returns to sgm0 and new
    strengths come from the RBF conjugate gradient (rbf_conjugategradient)."""
    nu: float
    sgm0: float
    beta: float = 1.5
    t_sgm: float = 0.0
    zeta: object = None
    itmax: int = 15
    tol: float = 1e-3
    iterror: bool = True


def rbf_conjugategradient(pfield: ParticleField, cs: CoreSpreading):
    """src/FLOWVPM_viscous.jl:314-454, per component, over the non-static
    particles: the solution is built in M[1:3], the residual in M[4:6], the
    target vorticity is M[7:9]; Gamma holds the search direction while the
    basis field of it (zeta) lands in J[1:3]."""
    zeta = cs.zeta if cs.zeta is not None else _default_zeta()
    P = pfield.particles
    idx = _live(pfield)
    tiny = 2 * EPS
    P[27:30, idx] = P[33:36, idx] * P[VOL_INDEX, idx]          # x0 = omega_targ * vol
    P[GAMMA_INDEX, idx] = P[27:30, idx]
    zeta(pfield)
    P[30:33, idx] = P[33:36, idx] - P[15:18, idx]               # r0 = b - A x0
    P[GAMMA_INDEX, idx] = P[30:33, idx]                         # p0 = r0
    rr0s = (P[30:33, idx] ** 2).sum(1)
    rrs = rr0s.copy()
    with np.errstate(divide="ignore", invalid="ignore"):
        flags = (np.sqrt(rr0s) > cs.tol) | (np.sqrt(rrs / rr0s) > cs.tol)
    for it in range(1, int(cs.itmax) + 1):
        if not flags.any():
            break
        zeta(pfield)
        pAps = (P[GAMMA_INDEX, idx] * P[15:18, idx]).sum(1)
        with np.errstate(divide="ignore", invalid="ignore"):
            alphas = rrs / pAps * flags
        prev_rrs = rrs
        P[27:30, idx] += alphas[:, None] * P[GAMMA_INDEX, idx]
        P[30:33, idx] -= alphas[:, None] * P[15:18, idx]
        rrs = (P[30:33, idx] ** 2).sum(1)
        with np.errstate(divide="ignore", invalid="ignore"):
            betas = rrs / prev_rrs
        betas = np.where(np.abs(prev_rrs) <= tiny, 1.0, betas)
        P[GAMMA_INDEX, idx] = P[30:33, idx] + betas[:, None] * P[GAMMA_INDEX, idx]
        with np.errstate(divide="ignore", invalid="ignore"):
            flags = flags & np.where(np.abs(rr0s) <= tiny, False, np.sqrt(rrs / rr0s) > cs.tol)
        if it == cs.itmax and flags.any() and cs.iterror:
            raise RuntimeError(f"Maximum number of iterations {cs.itmax} reached before convergence. "
                               f"Errors: {np.sqrt(rrs / rr0s)}, tolerance:{cs.tol}")
    P[GAMMA_INDEX, idx] = P[27:30, idx]


def _default_zeta():
    from .uj import zeta_gb300
    return zeta_gb300


def viscousdiffusion(pfield: ParticleField, dt: float, aux1: float = 0.0, aux2: float = 0.0):
    scheme = pfield.viscous
    if isinstance(scheme, Inviscid):
        return
    if not isinstance(scheme, CoreSpreading):
        raise NotImplementedError(f"viscous scheme {type(scheme).__name__} is not supported")
    idx = _live(pfield)
    P = pfield.particles
    if pfield.integration is euler:                                 # src/FLOWVPM_viscous.jl:155-162
        s = P[SIGMA_INDEX, idx]
        P[SIGMA_INDEX, idx] = np.sqrt(s * s + 2 * scheme.nu * dt)
        proceed = True
    elif pfield.integration is rungekutta3:                         # :165-178
        M7 = aux1 * P[27 + 6, idx] + dt * 2 * scheme.nu
        P[27 + 6, idx] = M7
        s = P[SIGMA_INDEX, idx]
        P[SIGMA_INDEX, idx] = np.sqrt(s ** 2 + aux2 * M7)
        proceed = abs(aux2 - 8 / 15) <= 1e-7
    else:
        raise NotImplementedError(f"time integration scheme {pfield.integration} is not implemented in the "
                                  "core spreading viscous scheme")
    if proceed:
        scheme.t_sgm += dt
        beta_cur = math.sqrt(2 * scheme.nu * scheme.t_sgm / scheme.sgm0 ** 2 + 1)
        if beta_cur >= scheme.beta:
            zeta = scheme.zeta if scheme.zeta is not None else _default_zeta()
            zeta(pfield)                                        # basis field of the current strengths
            P[33:36, idx] = P[15:18, idx]                       # target vorticity in M[7:9]
            P[SIGMA_INDEX, idx] = scheme.sgm0                   # reset core sizes
            rbf_conjugategradient(pfield, scheme)
            scheme.t_sgm = 0.0


# ----------------------------------------------------------------- relaxation
@dataclass(frozen=True)
class Relaxation:
    """src/FLOWVPM_relaxation.jl:24-32"""
    relax: object
    nsteps_relax: int
    rlxf: float

    def __call__(self, pfield: ParticleField, idx=None):
        return self.relax(self.rlxf, pfield, idx)


def relax_pedrizzetti(rlxf: float, pfield: ParticleField, idx=None, corrected: bool = False):
    """src/FLOWVPM_relaxation.jl:62-81 (and the corrected form, :112-142),
    applied to the particles `idx` (default: all non-static)."""
    idx = _live(pfield) if idx is None else idx
    P = pfield.particles
    J = P[J_INDEX, idx]
    G = P[GAMMA_INDEX, idx]
    w1, w2, w3 = J[5] - J[7], J[6] - J[2], J[1] - J[3]
    nrmw = np.sqrt(w1 * w1 + w2 * w2 + w3 * w3)
    ok = nrmw != 0
    nrmw_s = np.where(ok, nrmw, 1.0)
    nrmG = np.sqrt(G[0] ** 2 + G[1] ** 2 + G[2] ** 2)
    newG = np.empty_like(G)
    newG[0] = (1 - rlxf) * G[0] + rlxf * nrmG * w1 / nrmw_s
    newG[1] = (1 - rlxf) * G[1] + rlxf * nrmG * w2 / nrmw_s
    newG[2] = (1 - rlxf) * G[2] + rlxf * nrmG * w3 / nrmw_s
    if corrected:
        b2 = 1 - 2 * (1 - rlxf) * rlxf * (1 - (G[0] * w1 + G[1] * w2 + G[2] * w3) / (nrmG * nrmw_s))
        newG = newG / np.sqrt(b2)
    P[GAMMA_INDEX, idx] = np.where(ok, newG, G)


def relax_correctedpedrizzetti(rlxf: float, pfield: ParticleField, idx=None):
    relax_pedrizzetti(rlxf, pfield, idx, corrected=True)


def _relax_none(rlxf, pfield, idx=None):
    return None


relaxation_none = norelaxation = Relaxation(_relax_none, -1, 0.0)     # src/FLOWVPM.jl:170
pedrizzetti = relaxation_pedrizzetti = Relaxation(relax_pedrizzetti, 1, 0.3)
correctedpedrizzetti = Relaxation(relax_correctedpedrizzetti, 1, 0.3)
relaxation_default = pedrizzetti


# ------------------------------------------------------------------------ SFS
class BeforeUJ: pass
class AfterUJ: pass


@dataclass(frozen=True)
class NoSFS:
    """src/FLOWVPM_subfilterscale.jl:63-77"""
    def __call__(self, pfield, stage, a=1, b=1):
        return None


noSFS = SFS_none = NoSFS()


def isSFSenabled(sfs) -> bool:
    return not isinstance(sfs, NoSFS)


def clipping_backscatter(pfield: ParticleField, idx) -> np.ndarray:
    """True where C*(Gamma . SFS) < 0, src/FLOWVPM_subfilterscale.jl:287-296"""
    P = pfield.particles
    C = P[C_INDEX.start, idx]
    G = P[GAMMA_INDEX, idx]
    S = P[SFS_INDEX, idx]
    return C * (G[0] * S[0] + G[1] * S[1] + G[2] * S[2]) < 0


@dataclass(frozen=True)
class ConstantSFS:
    """src/FLOWVPM_subfilterscale.jl:84-148"""
    Cs: float = 1.0
    clippings: tuple = ()

    def __call__(self, pfield, stage, a=1, b=1):
        if stage is AfterUJ and (a == 1 or a == 0):
            idx = _live(pfield)
            pfield.particles[C_INDEX.start, idx] = self.Cs
            for clip in self.clippings:
                m = clip(pfield, idx)
                pfield.particles[C_INDEX.start, idx[m]] = 0.0


@dataclass(frozen=True)
class DynamicSFS:
    """Dynamic procedure SFS scheme, src/FLOWVPM_subfilterscale.jl:157-268 with
    the pseudo-three-level procedure of :447-673."""
    alpha: float = 0.667
    rlxf: float = 0.005
    minC: float = 0.0
    maxC: float = 1.0
    force_positive: bool = False
    clippings: tuple = ()

    def __call__(self, pfield, stage, a=1, b=1):
        if not (a == 1 or a == 0):
            return
        if stage is BeforeUJ:
            dynamicprocedure_pseudo3level_beforeUJ(pfield, self)
        else:
            dynamicprocedure_pseudo3level_afterUJ(pfield, self)
            idx = _live(pfield)
            for clip in self.clippings:
                m = clip(pfield, idx)
                pfield.particles[C_INDEX.start, idx[m]] *= 0


def _check_bounds(minC, maxC):
    if minC < 0:
        raise ValueError(f"Invalid C bounds: Got a negative bound for minC ({minC})")
    if maxC < 0:
        raise ValueError(f"Invalid C bounds: Got a negative bound for maxC ({maxC})")
    if minC > maxC:
        raise ValueError(f"Invalid C bounds: minC > maxC ({minC} > {maxC})")


def dynamicprocedure_pseudo3level_beforeUJ(pfield: ParticleField, sfs: DynamicSFS):
    """src/FLOWVPM_subfilterscale.jl:447-539"""
    _check_bounds(sfs.minC, sfs.maxC)
    P = pfield.particles
    idx = _live(pfield)
    P[SIGMA_INDEX, idx] *= sfs.alpha
    pfield.UJ(pfield, sfs=True, reset=True, reset_sfs=True)
    P[M_INDEX, idx] = 0.0
    S = _stretch(P[J_INDEX, idx], P[GAMMA_INDEX, idx], pfield.transposed)
    for k in range(3):
        P[27 + k, idx] = S[k]
        P[27 + 3 + k, idx] = P[39 + k, idx]
    P[SIGMA_INDEX, idx] /= sfs.alpha


def dynamicprocedure_pseudo3level_afterUJ(pfield: ParticleField, sfs: DynamicSFS):
    """src/FLOWVPM_subfilterscale.jl:541-673"""
    _check_bounds(sfs.minC, sfs.maxC)
    P = pfield.particles
    idx = _live(pfield)
    G = P[GAMMA_INDEX, idx]
    S = _stretch(P[J_INDEX, idx], G, pfield.transposed)
    M = P[M_INDEX, idx]
    for k in range(3):
        M[k] -= S[k]
        M[3 + k] -= P[39 + k, idx]
    zeta0 = pfield.kernel.zeta(0.0)
    sigma = P[SIGMA_INDEX, idx]
    Cp = P[C_INDEX, idx]
    nume = M[0] * G[0] + M[1] * G[1] + M[2] * G[2]
    nume = nume * (3 * sfs.alpha - 2)
    deno = M[3] * G[0] + M[4] * G[1] + M[5] * G[2]
    deno = deno / (zeta0 / (sigma * sigma * sigma))
    C3 = Cp[2].copy()
    first = C3 == 0
    C3 = np.where(first, deno, C3)
    C3 = np.where(C3 == 0, EPS, C3)
    nume = sfs.rlxf * nume + (1 - sfs.rlxf) * Cp[1]
    deno = sfs.rlxf * deno + (1 - sfs.rlxf) * C3
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.abs(nume / deno)
        big = ratio > sfs.maxC
        deno = np.where(big & (np.abs(deno) < np.abs(C3)), np.sign(deno) * np.abs(C3), deno)
        ratio2 = np.abs(nume / deno)
        nume = np.where(big & (ratio2 >= sfs.maxC), np.sign(nume) * np.abs(deno) * sfs.maxC, nume)
        small = (~big) & (ratio < sfs.minC)
        nume = np.where(small, np.sign(nume) * np.abs(deno) * sfs.minC, nume)
        C1 = nume / deno
    if np.isnan(C1).any():
        raise FloatingPointError("NaN in dynamicprocedure_pseudo3level_afterUJ")
    if sfs.force_positive:
        C1 = C1 * np.sign(C1)
    P[C_INDEX.start, idx] = C1
    P[C_INDEX.start + 1, idx] = nume
    P[C_INDEX.start + 2, idx] = deno
    P[M_INDEX, idx] = 0.0


# src/FLOWVPM.jl:223 -- the recommended two-level dynamic model without backscatter
SFS_Cd_twolevel_nobackscatter = DynamicSFS(alpha=0.999, force_positive=True, clippings=(clipping_backscatter,))
SFS_Cd_threelevel_nobackscatter = DynamicSFS(alpha=0.667, force_positive=True, clippings=(clipping_backscatter,))
SFS_Cs_nobackscatter = ConstantSFS(Cs=1.0, clippings=(clipping_backscatter,))


# ----------------------------------------------------------- time integration
def update_particle_states(pfield: ParticleField, a, b, dt, Uinf, f, g, zeta0):
    """rVPM low-storage RK stage, src/FLOWVPM_timeintegration.jl:463-532."""
    P = pfield.particles
    idx = _live(pfield)
    C = P[C_INDEX.start, idx]
    M = P[M_INDEX, idx]
    G = P[GAMMA_INDEX, idx]
    U = P[U_INDEX, idx]
    SFS = P[SFS_INDEX, idx]
    X = P[X_INDEX, idx]
    sigma = P[SIGMA_INDEX, idx]
    for k in range(3):
        M[k] = a * M[k] + dt * (U[k] + Uinf[k])
        X[k] += b * M[k]
    MM = _stretch(P[J_INDEX, idx], G, pfield.transposed)
    Gnorm2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2]
    s3 = sigma * sigma * sigma
    pos = Gnorm2 > 0
    MM4 = (f + g) / (1 + 3 * f) * (MM[0] * G[0] + MM[1] * G[1] + MM[2] * G[2])
    MM4 = MM4 - f / (1 + 3 * f) * (C * SFS[0] * G[0] + C * SFS[1] * G[1] + C * SFS[2] * G[2]) * s3 / zeta0
    MM4 = np.where(pos, MM4 / np.where(pos, Gnorm2, 1.0), 0.0)
    for k in range(3):
        M[3 + k] = a * M[3 + k] + dt * (MM[k] - 3 * MM4 * G[k] - C * SFS[k] * s3 / zeta0)
    M[7] = a * M[7] - dt * (sigma * MM4)
    for k in range(3):
        G[k] += b * M[3 + k]
    sigma = sigma + b * M[7]
    P[M_INDEX, idx] = M
    P[X_INDEX, idx] = X
    P[GAMMA_INDEX, idx] = G
    P[SIGMA_INDEX, idx] = sigma


def rungekutta3(pfield: ParticleField, dt: float, *, relax: bool = False, custom_UJ=None):
    """Low-storage RK3 for the reformulated VPM, src/FLOWVPM_timeintegration.jl:388-461."""
    if isinstance(pfield.formulation, ClassicVPM):
        raise NotImplementedError(
            "rungekutta3 with ClassicVPM: the reference's method (src/FLOWVPM_timeintegration.jl:185-262) "
            "passes f and g, which it never defines, to update_particle_states and fails with UndefVarError")
    if not isinstance(pfield.formulation, ReformulatedVPM):
        raise NotImplementedError("rungekutta3 is mirrored for ReformulatedVPM formulations")
    Uinf = np.asarray(pfield.Uinf(pfield.t), dtype=np.float64)
    f, g = pfield.formulation.f, pfield.formulation.g
    zeta0 = pfield.kernel.zeta(0.0)
    P = pfield.particles
    P[M_INDEX, _live(pfield)] = 0.0
    UJ = pfield.UJ if custom_UJ is None else custom_UJ
    sfs_on = isSFSenabled(pfield.SFS)
    for a, b in ((0.0, 1 / 3), (-5 / 9, 15 / 16), (-153 / 128, 8 / 15)):
        pfield.SFS(pfield, BeforeUJ, a=a, b=b)
        UJ(pfield, reset_sfs=sfs_on, reset=True, sfs=sfs_on)
        pfield.SFS(pfield, AfterUJ, a=a, b=b)
        update_particle_states(pfield, a, b, dt, Uinf, f, g, zeta0)
        viscousdiffusion(pfield, dt, aux1=a, aux2=b)
    if relax:
        _reset_particles(pfield)
        pfield.UJ(pfield)
        pfield.relaxation(pfield)


def _euler_classic(pfield: ParticleField, dt: float, relax: bool, Uinf, zeta0):
    """The ClassicVPM update of src/FLOWVPM_timeintegration.jl:42-91.  The
    reference adds the stretching to Gamma one component at a time, in place,
    so the second component's stretching already sees the updated first and
    the third sees both; that order is kept."""
    P = pfield.particles
    idx = _live(pfield)
    C = P[C_INDEX.start, idx]
    X = P[X_INDEX, idx]
    U = P[U_INDEX, idx]
    for k in range(3):
        X[k] += dt * (U[k] + Uinf[k])
    J = P[J_INDEX, idx]
    G = P[GAMMA_INDEX, idx]
    if pfield.transposed:
        G[0] += dt * (J[0] * G[0] + J[1] * G[1] + J[2] * G[2])
        G[1] += dt * (J[3] * G[0] + J[4] * G[1] + J[5] * G[2])
        G[2] += dt * (J[6] * G[0] + J[7] * G[1] + J[8] * G[2])
    else:
        G[0] += dt * (J[0] * G[0] + J[3] * G[1] + J[6] * G[2])
        G[1] += dt * (J[1] * G[0] + J[4] * G[1] + J[7] * G[2])
        G[2] += dt * (J[2] * G[0] + J[5] * G[1] + J[8] * G[2])
    sigma = P[SIGMA_INDEX, idx]
    SFS = P[SFS_INDEX, idx]
    for k in range(3):
        G[k] -= dt * C * SFS[k] * (sigma * sigma * sigma) / zeta0
    P[X_INDEX, idx] = X
    P[GAMMA_INDEX, idx] = G
    if relax:
        pfield.relaxation(pfield, idx)
    viscousdiffusion(pfield, dt)


def euler(pfield: ParticleField, dt: float, *, relax: bool = False, custom_UJ=None):
    """First-order Euler step, src/FLOWVPM_timeintegration.jl:23-37 (the SFS
    model's hooks around one UJ) and the reformulated-VPM update of :103-173:
    X += dt (U + Uinf); Gamma += dt (S - 3 Z Gamma - C SFS sigma^3/zeta0);
    sigma -= dt sigma Z; then relaxation with the step's J, and viscous diffusion.
    ClassicVPM takes the update of :42-91 (_euler_classic)."""
    if not isinstance(pfield.formulation, (ReformulatedVPM, ClassicVPM)):
        raise NotImplementedError(f"euler: unknown formulation {type(pfield.formulation).__name__}")
    sfs_on = isSFSenabled(pfield.SFS)
    pfield.SFS(pfield, BeforeUJ)
    UJ = pfield.UJ if custom_UJ is None else custom_UJ
    UJ(pfield, reset_sfs=sfs_on, reset=True, sfs=sfs_on)
    pfield.SFS(pfield, AfterUJ)
    Uinf = np.asarray(pfield.Uinf(pfield.t), dtype=np.float64)
    if isinstance(pfield.formulation, ClassicVPM):
        _euler_classic(pfield, dt, relax, Uinf, pfield.kernel.zeta(0.0))
        return
    f, g = pfield.formulation.f, pfield.formulation.g
    zeta0 = pfield.kernel.zeta(0.0)
    P = pfield.particles
    idx = _live(pfield)
    C = P[C_INDEX.start, idx]
    X = P[X_INDEX, idx]
    U = P[U_INDEX, idx]
    for k in range(3):
        X[k] += dt * (U[k] + Uinf[k])
    G = P[GAMMA_INDEX, idx]
    SFS = P[SFS_INDEX, idx]
    sigma = P[SIGMA_INDEX, idx]
    MM = _stretch(P[J_INDEX, idx], G, pfield.transposed)
    Gnorm2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2]
    pos = Gnorm2 > 0
    MM4 = (f + g) / (1 + 3 * f) * (MM[0] * G[0] + MM[1] * G[1] + MM[2] * G[2])
    sigma3 = sigma * sigma * sigma                 # Julia's literal power
    MM4 = MM4 - f / (1 + 3 * f) * (C * SFS[0] * G[0] + C * SFS[1] * G[1] + C * SFS[2] * G[2]) * sigma3 / zeta0
    MM4 = np.where(pos, MM4 / np.where(pos, G[0] * G[0] + G[1] * G[1] + G[2] * G[2], 1.0), 0.0)
    for k in range(3):
        G[k] += dt * (MM[k] - 3 * MM4 * G[k] - C * SFS[k] * sigma3 / zeta0)
    sigma = sigma - dt * (sigma * MM4)
    P[X_INDEX, idx] = X
    P[GAMMA_INDEX, idx] = G
    P[SIGMA_INDEX, idx] = sigma
    if relax:   # per particle in the reference, with this step's J: the same as one pass over all
        pfield.relaxation(pfield, idx)
    viscousdiffusion(pfield, dt)


def _kernel_compatibility(viscous) -> tuple:
    """src/FLOWVPM.jl:259-267: the kernels each viscous scheme accepts."""
    from .particlefield import gaussian, gaussianerf, singular, winckelmans
    if isinstance(viscous, CoreSpreading):
        return (gaussianerf,)
    return (singular, gaussian, gaussianerf, winckelmans)


def run_vpm(pfield: ParticleField, dt: float, nsteps: int, *, runtime_function=None,
            static_particles_function=None, custom_UJ=None, save_path=None, save_pfield: bool = True,
            create_savepath: bool = True, run_name: str = "pfield", nsteps_save: int = 1,
            save_time: bool = True):
    """The stepping loop of run_vpm! (src/FLOWVPM_utils.jl:41-136): the
    kernel/viscous-scheme check, relaxation every nsteps_relax steps, static
    particles added by static_particles_function(pfield, t, dt) before each step
    and removed after it (unless it returns False), runtime_function(pfield, t,
    dt) after each step, which ends the run by returning True, and, with a
    save_path, the field saved by vpm_gb300.io.save at step 0, every nsteps_save
    steps, at the last step and at a runtime stop (:122-126; save_time=False
    stamps the files with nt instead of t).  Verbose output and the settings
    file are not written."""
    if save_path is not None and save_pfield and create_savepath:
        import os
        os.makedirs(save_path, exist_ok=True)
    if not any(pfield.kernel is k for k in _kernel_compatibility(pfield.viscous)):
        raise ValueError(f"Kernel {pfield.kernel} is not compatible with viscous scheme "
                         f"{type(pfield.viscous).__name__}; compatible kernels are "
                         f"{list(_kernel_compatibility(pfield.viscous))}")
    rlx = pfield.relaxation
    for i in range(nsteps + 1):
        relax = (rlx is not relaxation_none and rlx.nsteps_relax >= 1 and i > 0
                 and i % rlx.nsteps_relax == 0)
        org_np = pfield.np
        if i != 0:
            remove = static_particles_function(pfield, pfield.t, dt) if static_particles_function else None
            pfield.nextstep(dt, relax=relax, custom_UJ=custom_UJ)
            if remove is None or remove:
                for pi in range(pfield.np - 1, org_np - 1, -1):
                    pfield.remove_particle(pi)
        breakflag = bool(runtime_function is not None and runtime_function(pfield, pfield.t, dt))
        if save_pfield and save_path is not None and (i % nsteps_save == 0 or i == nsteps or breakflag):
            from . import io as vio
            vio.save(pfield, run_name, path=save_path, add_num=True,
                     overwrite_time=None if save_time else pfield.nt)
        if breakflag:
            break
