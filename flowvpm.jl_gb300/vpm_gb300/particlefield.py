"""Host-side mirror of FLOWVPM.jl's ParticleField and solver settings.

This is the reference-facing interface around the GB300 UJ: the same names,
argument meanings and error behaviour as FLOWVPM.jl v4.0.3, so a script written
against the reference reads the same here.  The particle storage is the
reference's column-major 46 x maxparticles Float64 matrix
(src/FLOWVPM_particlefield.jl:11,134), held as a Fortran-ordered numpy array so
its memory is byte-identical to the Julia matrix and can be handed to the C ABI
as is.  Row indices below are 0-based (the reference's minus one).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import _lib

NFIELDS = 46
# src/FLOWVPM_particlefield.jl:239-252, 0-based
X_INDEX = slice(0, 3)
GAMMA_INDEX = slice(3, 6)
SIGMA_INDEX = 6
VOL_INDEX = 7
CIRCULATION_INDEX = 8
U_INDEX = slice(9, 12)
VORTICITY_INDEX = slice(12, 15)
J_INDEX = slice(15, 24)
PSE_INDEX = slice(24, 27)
M_INDEX = slice(27, 36)
C_INDEX = slice(36, 39)
SFS_INDEX = slice(39, 42)
STATIC_INDEX = 42
U_PREV_INDEX = 43

MIN_MT_NP = 1000  # src/FLOWVPM.jl:50 (threading threshold; kept for reference)

# src/FLOWVPM.jl:62-66
const1 = 1 / (2 * math.pi) ** 1.5
const2 = math.sqrt(2 / math.pi)
const3 = 3 / (4 * math.pi)
const4 = 1 / (4 * math.pi)
sqr2 = math.sqrt(2)


# --------------------------------------------------------------------- kernels
@dataclass(frozen=True)
class Kernel:
    """A regularizing kernel (src/FLOWVPM_kernel.jl:23-28).  Only the four
    standard kernels cross the C ABI; `kid` is their VPM_KERNEL_* id."""
    name: str
    kid: int

    def zeta(self, r: float) -> float:
        """Basis function zeta(r), src/FLOWVPM_kernel.jl:45-74."""
        if self.kid == _lib.KERNEL_SINGULAR:
            return 1.0 if r == 0 else 0.0
        if self.kid == _lib.KERNEL_GAUSSIAN:
            return const3 * math.exp(-r * r * r)
        if self.kid == _lib.KERNEL_GAUSSIANERF:
            return const1 * math.exp(-r * r / 2)
        temp = r * r + 1
        temp2 = temp * temp * temp
        temp = temp2 * temp2 * temp
        return const4 * 7.5 / math.sqrt(temp)


# src/FLOWVPM.jl:129-133
singular = kernel_singular = Kernel("singular", _lib.KERNEL_SINGULAR)
gaussian = kernel_gaussian = Kernel("gaussian", _lib.KERNEL_GAUSSIAN)
gaussianerf = kernel_gaussianerf = Kernel("gaussianerf", _lib.KERNEL_GAUSSIANERF)
winckelmans = kernel_winckelmans = Kernel("winckelmans", _lib.KERNEL_WINCKELMANS)
kernel_default = gaussianerf
standard_kernels = (singular, gaussian, gaussianerf, winckelmans)


# ----------------------------------------------------------------- formulation
@dataclass(frozen=True)
class ClassicVPM:
    """src/FLOWVPM_formulation.jl:23"""


@dataclass(frozen=True)
class ReformulatedVPM:
    """src/FLOWVPM_formulation.jl:31-37"""
    f: float = 0.0
    g: float = 0.2

    @property
    def h(self) -> float:
        return (1 - 3 * self.g) / (1 + 3 * self.f)


formulation_classic = ClassicVPM()                            # src/FLOWVPM.jl:83
formulation_cVPM = cVPM = ReformulatedVPM(0.0, 0.0)          # :84
formulation_rVPM = rVPM = ReformulatedVPM(0.0, 1 / 5)         # :86
formulation_tube_continuity = ReformulatedVPM(1 / 2, 0.0)     # :94
formulation_tube_momentum = ReformulatedVPM(1 / 4, 1 / 4)     # :102
formulation_sphere_momentum = ReformulatedVPM(0.0, 1 / 5 + 1e-8)
formulation_default = rVPM


# ------------------------------------------------------------------ particles
class ParticleField:
    """Mirror of `ParticleField(maxparticles; ...)`, src/FLOWVPM_particlefield.jl:67-141.

    `UJ` is the particle-to-particle hook; it defaults to the GB300 FP64 UJ
    (the reference defaults to UJ_fmm, which is not built here)."""

    def __init__(self, maxparticles: int, *, formulation=formulation_default, viscous=None,
                 np: int = 0, nt: int = 0, t: float = 0.0, transposed: bool = True,
                 SFS=None, kernel: Kernel = kernel_default, UJ=None, Uinf=None,
                 relaxation=None, integration=None, useGPU: int = 1):
        from . import timeintegration as ti
        from .uj import UJ_gb300
        self.maxparticles = int(maxparticles)
        self.particles = _zeros_matrix(self.maxparticles)
        self.formulation = formulation
        self.viscous = viscous if viscous is not None else ti.Inviscid()
        self.np = int(np)
        self.nt = int(nt)
        self.t = float(t)
        self.kernel = kernel
        self.UJ = UJ if UJ is not None else UJ_gb300
        self.Uinf = Uinf if Uinf is not None else (lambda t: (0.0, 0.0, 0.0))
        self.SFS = SFS if SFS is not None else ti.noSFS
        self.integration = integration if integration is not None else ti.rungekutta3
        self.transposed = bool(transposed)
        self.relaxation = relaxation if relaxation is not None else ti.pedrizzetti
        self.useGPU = useGPU

    # ------------------------------------------------------------- particles
    def get_np(self) -> int:
        return self.np

    def add_particle(self, X, Gamma, sigma, *, vol=0.0, circulation=1.0, C=0.0, static=False):
        """src/FLOWVPM_particlefield.jl:160-191"""
        if self.np == self.maxparticles:
            raise RuntimeError(f"PARTICLE OVERFLOW. Max number of particles {self.maxparticles} has been reached")
        i = self.np
        self.np += 1
        P = self.particles
        P[X_INDEX, i] = X
        P[GAMMA_INDEX, i] = Gamma
        P[SIGMA_INDEX, i] = sigma
        P[VOL_INDEX, i] = vol
        P[CIRCULATION_INDEX, i] = circulation
        P[C_INDEX, i] = C
        P[STATIC_INDEX, i] = float(static)

    def add_particles(self, X, Gamma, sigma, *, vol=None, circulation=None, static=None):
        """Vectorised add_particle for n particles (X, Gamma: [n,3]; sigma: [n])."""
        X = np.asarray(X, dtype=np.float64)
        n = X.shape[0]
        if self.np + n > self.maxparticles:
            raise RuntimeError(f"PARTICLE OVERFLOW. Max number of particles {self.maxparticles} has been reached")
        sl = slice(self.np, self.np + n)
        P = self.particles
        P[X_INDEX, sl] = X.T
        P[GAMMA_INDEX, sl] = np.asarray(Gamma, dtype=np.float64).T
        P[SIGMA_INDEX, sl] = sigma
        P[VOL_INDEX, sl] = 0.0 if vol is None else vol
        P[CIRCULATION_INDEX, sl] = 1.0 if circulation is None else circulation
        P[C_INDEX, sl] = 0.0
        P[STATIC_INDEX, sl] = 0.0 if static is None else np.asarray(static, dtype=np.float64)
        self.np += n

    def remove_particle(self, i: int):
        """src/FLOWVPM_particlefield.jl:409-429 (0-based i)."""
        if i < 0 or i >= self.np:
            raise IndexError(f"Requested removal of particle {i}, but there is only {self.np} particles in the field.")
        last = self.np - 1
        if i != last:
            self.particles[:, i] = self.particles[:, last]
        self.particles[9:27, last] = 0.0
        self.np -= 1

    # views over the live particles, [n, k] (transposed views of the matrix)
    def view(self, rows) -> np.ndarray:
        return self.particles[rows, :self.np].T

    X = property(lambda self: self.view(X_INDEX))
    Gamma = property(lambda self: self.view(GAMMA_INDEX))
    sigma = property(lambda self: self.particles[SIGMA_INDEX, :self.np])
    U = property(lambda self: self.view(U_INDEX))
    J = property(lambda self: self.view(J_INDEX))
    SFS_values = property(lambda self: self.view(SFS_INDEX))
    static = property(lambda self: self.particles[STATIC_INDEX, :self.np] != 0)

    def isLES(self) -> bool:
        from .timeintegration import isSFSenabled
        return isSFSenabled(self.SFS)

    def nextstep(self, dt: float, *, relax: bool = False, update_U_prev: bool = True, custom_UJ=None):
        """src/FLOWVPM_particlefield.jl:435-460"""
        if self.np != 0:
            if custom_UJ is None:
                self.integration(self, dt, relax=relax)
            else:
                self.integration(self, dt, relax=relax, custom_UJ=custom_UJ)
        if update_U_prev:
            U = self.particles[U_INDEX, :self.np]
            self.particles[U_PREV_INDEX, :self.np] = np.sqrt(U[0] * U[0] + U[1] * U[1] + U[2] * U[2])
        self.t += dt
        self.nt += 1


def _zeros_matrix(maxparticles: int) -> np.ndarray:
    return np.zeros((NFIELDS, maxparticles), dtype=np.float64, order="F")


def _reset_particles(pfield: ParticleField):
    """src/FLOWVPM_particlefield.jl:464-475"""
    n = pfield.np
    live = pfield.particles[STATIC_INDEX, :n] == 0
    idx = np.nonzero(live)[0]
    pfield.particles[9:27, idx] = 0.0


def _reset_particles_sfs(pfield: ParticleField):
    """src/FLOWVPM_particlefield.jl:490-501"""
    n = pfield.np
    idx = np.nonzero(pfield.particles[STATIC_INDEX, :n] == 0)[0]
    pfield.particles[SFS_INDEX, idx] = 0.0
