"""The drop-in UJ hooks: `UJ_gb300` (FP64) and `UJ_gb300_mixed` (FP32-comp).

Both have the signature and semantics of `UJ_direct(pfield; rbf, sfs, reset,
reset_sfs)` (src/FLOWVPM_UJ.jl:21-37) and run through `vpm_uj` of the C ABI on
the particle matrix itself, so a ParticleField built with `UJ=UJ_gb300` runs
the time integration unchanged.  A kernel other than the four standard ones
cannot cross the ABI and raises, like the reference's own error() paths.
"""
from __future__ import annotations

from . import _lib
from .particlefield import ParticleField, standard_kernels


def _flags(pfield: ParticleField, sfs: bool, reset: bool, reset_sfs: bool) -> int:
    f = 0
    if reset:
        f |= _lib.RESET
    if reset_sfs:
        f |= _lib.RESET_SFS
    if sfs:
        f |= _lib.SFS
    if pfield.transposed:
        f |= _lib.TRANSPOSED
    return f


def _kernel_id(pfield: ParticleField) -> int:
    k = pfield.kernel
    if k not in standard_kernels:
        raise ValueError(f"UJ_gb300 supports only the standard kernels (singular, gaussian, gaussianerf, "
                         f"winckelmans); got {k!r}")
    return k.kid


def _uj(pfield: ParticleField, precision: int, rbf: bool, sfs: bool, reset: bool, reset_sfs: bool,
        ctx: _lib.Context | None):
    # rbf is accepted and ignored, as UJ_direct does (src/FLOWVPM_UJ.jl:21-37); UJ_fmm's
    # rbf=true evaluates zeta_fmm instead, which is zeta_fmm_gb300 here
    c = ctx if ctx is not None else _lib.default_context()
    c.uj(pfield.particles, pfield.np, _kernel_id(pfield), precision, _flags(pfield, sfs, reset, reset_sfs))


def UJ_gb300(pfield: ParticleField, *, rbf: bool = False, sfs: bool = False, reset: bool = True,
             reset_sfs: bool = False, ctx: _lib.Context | None = None, **optargs) -> None:
    """UJ_direct on the GB300 in FP64 (the reference formula)."""
    _uj(pfield, _lib.FP64, rbf, sfs, reset, reset_sfs, ctx)


def UJ_gb300_mixed(pfield: ParticleField, *, rbf: bool = False, sfs: bool = False, reset: bool = True,
                   reset_sfs: bool = False, ctx: _lib.Context | None = None, **optargs) -> None:
    """UJ_direct on the GB300 with FP32 pair math and FP64 block reduction."""
    _uj(pfield, _lib.FP32COMP, rbf, sfs, reset, reset_sfs, ctx)


def UJ_gb300_cross(source: ParticleField, target: ParticleField, *, precision: int = _lib.FP64,
                   ctx: _lib.Context | None = None) -> None:
    """UJ_direct(source, target), src/FLOWVPM_UJ.jl:48-50: accumulate, no reset."""
    c = ctx if ctx is not None else _lib.default_context()
    c.uj_cross(source.particles, source.np, target.particles, target.np, _kernel_id(source), precision)


def zeta_gb300(pfield: ParticleField, *, ctx: _lib.Context | None = None) -> None:
    """zeta_direct(pfield) (src/FLOWVPM_viscous.jl:467-488) on the GB300 in FP64:
    rows 16:18 (J[1:3]) of every particle receive the RBF basis field."""
    c = ctx if ctx is not None else _lib.default_context()
    c.zeta(pfield.particles, pfield.np, _kernel_id(pfield), _lib.FP64)


def zeta_gb300_mixed(pfield: ParticleField, *, ctx: _lib.Context | None = None) -> None:
    """zeta_direct on the GB300 with FP32 pair math and FP64 block reduction."""
    c = ctx if ctx is not None else _lib.default_context()
    c.zeta(pfield.particles, pfield.np, _kernel_id(pfield), _lib.FP32COMP)


def zeta_fmm_gb300(pfield: ParticleField, *, leaf_size: int = 64, theta: float = 0.4,
                   precision: int = _lib.FP64, ctx: _lib.Context | None = None) -> None:
    """zeta_fmm(pfield) (src/FLOWVPM_viscous.jl:523-556) on the GB300: rows 16:18
    (J[1:3]) of every particle, statics included, += the basis field summed over
    the near leaf pairs of the octree (leaf_size and theta play the parts of
    pfield.fmm.ncrit and .theta; the far field is neglected, as in the
    reference).  Like the reference it adds without zeroing the rows first;
    zeta_direct (zeta_gb300) sets them."""
    import numpy as np
    import torch
    c = ctx if ctx is not None else _lib.default_context()
    n = pfield.np
    if n == 0:
        return
    P = pfield.particles
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    W = d(P[15:18, :n].T)
    c.zeta_leaflist_dev(d(P[0:3, :n].T), d(P[3:6, :n].T), d(P[6, :n]), W, leaf_size=leaf_size, theta=theta,
                        kernel=_kernel_id(pfield), precision=precision)
    P[15:18, :n] = W.cpu().numpy().T
