"""Reverse-mode differentiation through UJ and the rVPM time step.

`UJFunction` is the torch.autograd.Function over the two C entry points
`vpm_uj_dev` (forward) and `vpm_uj_adjoint_dev` (backward, the hand-written
adjoint kernel, in the forward's precision).  It plays the role of the ChainRulesCore `rrule` that
src/FLOWVPM_rrules.jl:179-330 sketches but never wires in; a Julia binding
would wrap the same two calls in an rrule.

`EstrFunction` does the same for the SFS stretching pass Estr
(src/FLOWVPM_subfilterscale_models.jl:16-92) over `vpm_estr_dev` and its
adjoint `vpm_estr_adjoint_dev`, which also returns dL/dJ (J is an input of
Estr, so the gradient flows on into UJFunction's backward).  The reference's
rrule stops there ("SFS pullback not implemented yet!",
src/FLOWVPM_rrules.jl:153-157).

`rk3_step` is the reference's rVPM low-storage RK3 step
(src/FLOWVPM_timeintegration.jl:388-532, inviscid, no freestream) with
Pedrizzetti relaxation (src/FLOWVPM_relaxation.jl:62-81) and, optionally, the
constant-coefficient SFS scheme (ConstantSFS, src/FLOWVPM_subfilterscale.jl:88-150:
C = Cs set at the first stage of each step, with backscatter clipping
:287-296), written with torch tensor operations on device-resident state so
autograd can run through it; every particle-to-particle evaluation goes
through `UJFunction` / `EstrFunction`.  The clipping sets C by a comparison, a
piecewise-constant function of the state: C carries no gradient, as in any
autodiff of the reference.
`rollout` chains steps with per-step checkpointing.  The default keeps, per
step, its input state and the U, J of its UJ evaluations (O(N) each); the
backward pass re-runs the step's O(N) tensor algebra with autograd on those
kept values, so the O(N^2) pair sums are not evaluated again: their reverse
mode is the adjoint kernel, which recomputes the pair terms tile by tile.
checkpoint="recompute" keeps only each step's input state and re-runs the
whole step, UJ evaluations included (torch.utils.checkpoint).
"""
from __future__ import annotations

import math

import torch
import torch.utils.checkpoint as ckpt

from . import _lib

STAGES = ((0.0, 1 / 3), (-5 / 9, 15 / 16), (-153 / 128, 8 / 15))


class UJFunction(torch.autograd.Function):
    """(U[n,3], J[n,9]) of one particle set (x[n,3], gamma[n,3], sigma[n]), float64 CUDA tensors."""

    @staticmethod
    def forward(ctx, x, gam, sig, kernel: int, precision: int, vctx: _lib.Context):
        x, gam, sig = x.contiguous(), gam.contiguous(), sig.contiguous()
        n = x.shape[0]
        U = torch.zeros(n, 3, dtype=torch.float64, device=x.device)
        J = torch.zeros(n, 9, dtype=torch.float64, device=x.device)
        vctx.uj_dev(x, x, gam, sig, U, J, kernel, precision)
        ctx.save_for_backward(x, gam, sig)
        ctx.kernel = kernel
        ctx.precision = precision
        ctx.vctx = vctx
        return U, J

    @staticmethod
    def backward(ctx, Ubar, Jbar):
        x, gam, sig = ctx.saved_tensors
        n = x.shape[0]
        Ubar = torch.zeros(n, 3, dtype=torch.float64, device=x.device) if Ubar is None else Ubar.contiguous()
        Jbar = torch.zeros(n, 9, dtype=torch.float64, device=x.device) if Jbar is None else Jbar.contiguous()
        xb = torch.zeros_like(x)
        gb = torch.zeros_like(gam)
        sb = torch.zeros_like(sig)
        # the adjoint in the forward's precision (the FP32-comp adjoint covers all kernels but the Gaussian)
        prec = _lib.FP64 if ctx.kernel == _lib.KERNEL_GAUSSIAN else getattr(ctx, "precision", _lib.FP64)
        ctx.vctx.uj_adjoint_dev(x, gam, sig, Ubar, Jbar, xb, gb, sb, ctx.kernel, prec)
        return xb, gb, sb, None, None, None


def uj(x, gam, sig, kernel: int, precision: int = _lib.FP64, vctx: _lib.Context | None = None):
    return UJFunction.apply(x, gam, sig, kernel, precision, vctx or _lib.default_context())


def _stretch(J, G, transposed: bool = True):
    """(Gamma . grad')U or (Gamma . grad)U from J[n,9] (column-major 3x3 per particle).
    A broadcast product and a sum over 3 (elementwise kernels): as an einsum, torch runs
    it as cuBLAS batched matrix-vector products of 65,535 particles a launch, 16 launches
    and 4.1 ms at 2^20 particles."""
    Jm = J.view(-1, 3, 3)                      # Jm[:, j, i] = J[i + 3j] = du_i/dx_j
    if transposed:
        return (Jm * G.unsqueeze(1)).sum(2)    # S_k = sum_i du_i/dx_k G_i
    return (Jm * G.unsqueeze(2)).sum(1)        # S_i = sum_j du_i/dx_j G_j


class EstrFunction(torch.autograd.Function):
    """SFS[n,3] = Estr of one particle set on itself (x[n,3], gamma[n,3], sigma[n], J[n,9]),
    float64 CUDA tensors; no static particles."""

    @staticmethod
    def forward(ctx, x, gam, sig, J, kernel: int, precision: int, transposed: bool, vctx: _lib.Context):
        x, gam, sig, J = x.contiguous(), gam.contiguous(), sig.contiguous(), J.contiguous()
        SFS = torch.zeros_like(x)
        vctx.estr_dev(x, J, x, gam, sig, J, SFS, kernel, precision, transposed)
        ctx.save_for_backward(x, gam, sig, J)
        ctx.kernel, ctx.precision, ctx.transposed, ctx.vctx = kernel, precision, transposed, vctx
        return SFS

    @staticmethod
    def backward(ctx, Sbar):
        x, gam, sig, J = ctx.saved_tensors
        Sbar = torch.zeros_like(x) if Sbar is None else Sbar.contiguous()
        xb, gb, sb, Jb = torch.zeros_like(x), torch.zeros_like(gam), torch.zeros_like(sig), torch.zeros_like(J)
        ctx.vctx.estr_adjoint_dev(x, gam, sig, J, Sbar, xb, gb, sb, Jb, ctx.kernel, ctx.precision, ctx.transposed)
        return xb, gb, sb, Jb, None, None, None, None


def estr(x, gam, sig, J, kernel: int, precision: int = _lib.FP64, transposed: bool = True,
         vctx: _lib.Context | None = None):
    return EstrFunction.apply(x, gam, sig, J, kernel, precision, transposed, vctx or _lib.default_context())


class _KeptEstr(torch.autograd.Function):
    """Estr whose forward value was kept from an earlier evaluation on the same inputs."""

    @staticmethod
    def forward(ctx, x, gam, sig, J, SFS, kernel: int, precision: int, transposed: bool, vctx: _lib.Context):
        ctx.save_for_backward(x, gam, sig, J)
        ctx.kernel, ctx.precision, ctx.transposed, ctx.vctx = kernel, precision, transposed, vctx
        return SFS.clone()

    @staticmethod
    def backward(ctx, Sbar):
        xb, gb, sb, Jb, *_ = EstrFunction.backward(ctx, Sbar)
        return xb, gb, sb, Jb, None, None, None, None, None


class ConstantSFS:
    """The constant-coefficient SFS scheme of src/FLOWVPM_subfilterscale.jl:88-150:
    C = Cs on every particle at the first stage of a step, set to 0 where
    clipping_backscatter (src/FLOWVPM_subfilterscale.jl:287-296) finds C Gamma . SFS < 0."""

    def __init__(self, Cs: float = 1.0, clip_backscatter: bool = False):
        self.Cs = float(Cs)
        self.clip_backscatter = bool(clip_backscatter)


class DynamicSFS:
    """The dynamic-procedure SFS scheme of src/FLOWVPM_subfilterscale.jl:157-268 with the
    pseudo-three-level procedure of :447-673, at each step's first stage: U, J and Estr
    at the test filter alpha sigma and at sigma, the Lagrangian-averaged ratio
    C = <nu>/<delta> with the bounds [minC, maxC] (:592-656), force_positive, and
    backscatter clipping.  The per-particle state (C, numerator, denominator) is
    carried from step to step.  The bounds, force_positive and the clipping select
    branches by comparisons: the gradient follows the selected branch."""

    def __init__(self, alpha: float = 0.667, rlxf: float = 0.005, minC: float = 0.0, maxC: float = 1.0,
                 force_positive: bool = False, clip_backscatter: bool = False):
        if minC < 0 or maxC < 0 or minC > maxC:
            raise ValueError(f"invalid C bounds ({minC}, {maxC})")
        self.alpha, self.rlxf, self.minC, self.maxC = float(alpha), float(rlxf), float(minC), float(maxC)
        self.force_positive = bool(force_positive)
        self.clip_backscatter = bool(clip_backscatter)


EPS = 2.220446049250313e-16   # Julia eps(), the reference's guard of a zero denominator


def _dynamic_coefficient(sfs: DynamicSFS, gam, sig, J, SFS, MS, MF, Cprev, zeta0, transposed):
    """dynamicprocedure_pseudo3level_afterUJ (src/FLOWVPM_subfilterscale.jl:541-673) on
    device tensors: (C, numerator, denominator) per particle from the test-filter values
    MS = S(J_alpha), MF = SFS_alpha and the values J, SFS at sigma."""
    dS = MS - _stretch(J, gam, transposed)
    dF = MF - SFS
    nume = (dS * gam).sum(1) * (3 * sfs.alpha - 2)
    deno = (dF * gam).sum(1) / (zeta0 / sig ** 3)
    C3 = Cprev[:, 2]
    C3 = torch.where(C3 == 0, deno, C3)
    C3 = torch.where(C3 == 0, torch.full_like(C3, EPS), C3)
    nume = sfs.rlxf * nume + (1 - sfs.rlxf) * Cprev[:, 1]
    deno = sfs.rlxf * deno + (1 - sfs.rlxf) * C3
    with torch.no_grad():
        ratio = (nume / deno).abs()
        big = ratio > sfs.maxC
        swap_deno = big & (deno.abs() < C3.abs())
    deno = torch.where(swap_deno, torch.sign(deno) * C3.abs(), deno)
    with torch.no_grad():
        ratio2 = (nume / deno).abs()
        cap = big & (ratio2 >= sfs.maxC)
        floor = (~big) & (ratio < sfs.minC)
    nume = torch.where(cap, torch.sign(nume) * deno.abs() * sfs.maxC, nume)
    nume = torch.where(floor, torch.sign(nume) * deno.abs() * sfs.minC, nume)
    C1 = nume / deno
    if torch.isnan(C1).any():
        raise FloatingPointError("NaN in the dynamic procedure's coefficient")
    if sfs.force_positive:
        C1 = C1.abs()
    if sfs.clip_backscatter:
        with torch.no_grad():
            clip = C1 * (gam * SFS).sum(1) < 0
        C1 = torch.where(clip, torch.zeros_like(C1), C1)
    return torch.stack([C1, nume, deno], dim=1)


# zeta(0) of each kernel (src/FLOWVPM_kernel.jl; constants src/FLOWVPM.jl:62-66): singular,
# Gaussian, Gaussian-erf, Winckelmans
ZETA0 = {0: 1.0, 1: 3.0 / (4.0 * math.pi), 2: 1.0 / (2.0 * math.pi) ** 1.5, 3: 7.5 / (4.0 * math.pi)}


class _KeptUJ(torch.autograd.Function):
    """UJ whose forward values were kept from an earlier evaluation on the same
    inputs; its backward is the adjoint kernel, as for UJFunction."""

    @staticmethod
    def forward(ctx, x, gam, sig, U, J, kernel: int, precision: int, vctx: _lib.Context):
        ctx.save_for_backward(x, gam, sig)
        ctx.kernel = kernel
        ctx.precision = precision
        ctx.vctx = vctx
        return U.clone(), J.clone()

    @staticmethod
    def backward(ctx, Ubar, Jbar):
        xb, gb, sb, *_ = UJFunction.backward(ctx, Ubar, Jbar)
        return xb, gb, sb, None, None, None, None, None


def _uj_default(x, gam, sig, kernel, precision, vctx):
    return UJFunction.apply(x, gam, sig, kernel, precision, vctx)


def _estr_default(x, gam, sig, J, kernel, precision, transposed, vctx):
    return EstrFunction.apply(x, gam, sig, J, kernel, precision, transposed, vctx)


def rk3_step(x, gam, sig, dt: float, *, kernel: int, precision: int = _lib.FP64, f: float = 0.0,
             g: float = 0.2, relax: bool = True, rlxf: float = 0.3, transposed: bool = True,
             sfs: ConstantSFS | DynamicSFS | None = None, C=None, vctx: _lib.Context | None = None,
             uj_fn=None, estr_fn=None):
    """One rVPM RK3 step (+ Pedrizzetti relaxation, + the SFS term of `sfs`) on device
    tensors; differentiable.  With a DynamicSFS, C[n,3] is the per-particle state
    (coefficient, numerator, denominator; zeros at the start) and the step returns
    (x, gam, sig, C); otherwise (x, gam, sig).  uj_fn(x, gam, sig, kernel, precision,
    vctx) -> (U, J) and estr_fn(x, gam, sig, J, kernel, precision, transposed, vctx) -> SFS
    replace UJFunction / EstrFunction (checkpointing)."""
    vctx = vctx or _lib.default_context()
    uj_fn = uj_fn or _uj_default
    estr_fn = estr_fn or _estr_default
    zeta0 = ZETA0[kernel]
    dynamic = isinstance(sfs, DynamicSFS)
    if dynamic and C is None:
        C = torch.zeros(x.shape[0], 3, dtype=x.dtype, device=x.device)
    M0 = torch.zeros_like(x)
    M3 = torch.zeros_like(gam)
    M8 = torch.zeros_like(sig)
    Cs = None
    for a, b in STAGES:
        if dynamic and a == 0:   # BeforeUJ: the test filter alpha sigma
            sig_a = sig * sfs.alpha
            _, Ja = uj_fn(x, gam, sig_a, kernel, precision, vctx)
            MF = estr_fn(x, gam, sig_a, Ja, kernel, precision, transposed, vctx)
            MS = _stretch(Ja, gam, transposed)
        U, J = uj_fn(x, gam, sig, kernel, precision, vctx)
        Cterm = None
        if sfs is not None:
            SFS = estr_fn(x, gam, sig, J, kernel, precision, transposed, vctx)
            if a == 0:   # AfterUJ, first stage only
                if dynamic:
                    C = _dynamic_coefficient(sfs, gam, sig, J, SFS, MS, MF, C, zeta0, transposed)
                    Cs = C[:, 0]
                else:
                    with torch.no_grad():
                        Cs = torch.full_like(sig, sfs.Cs)
                        if sfs.clip_backscatter:
                            Cs = torch.where(Cs * (gam * SFS).sum(1) < 0, torch.zeros_like(Cs), Cs)
            Cterm = (Cs * sig ** 3 / zeta0)[:, None] * SFS            # C SFS sigma^3 / zeta0
        M0 = a * M0 + dt * U
        x = x + b * M0
        MM = _stretch(J, gam, transposed)
        Gn2 = (gam * gam).sum(1)
        pos = Gn2 > 0
        num = (f + g) / (1 + 3 * f) * (MM * gam).sum(1)
        if Cterm is not None and f != 0.0:
            num = num - f / (1 + 3 * f) * (Cterm * gam).sum(1)
        MM4 = torch.where(pos, num / torch.where(pos, Gn2, 1.0), torch.zeros_like(Gn2))
        dG = MM - 3 * MM4[:, None] * gam
        if Cterm is not None:
            dG = dG - Cterm
        M3 = a * M3 + dt * dG
        M8 = a * M8 - dt * (sig * MM4)
        gam = gam + b * M3
        sig = sig + b * M8
    if relax:
        U, J = uj_fn(x, gam, sig, kernel, precision, vctx)
        w = torch.stack([J[:, 5] - J[:, 7], J[:, 6] - J[:, 2], J[:, 1] - J[:, 3]], dim=1)
        nw = torch.sqrt((w * w).sum(1))
        nG = torch.sqrt((gam * gam).sum(1))
        ok = nw != 0
        newg = (1 - rlxf) * gam + rlxf * (nG / torch.where(ok, nw, 1.0))[:, None] * w
        gam = torch.where(ok[:, None], newg, gam)
    return (x, gam, sig, C) if dynamic else (x, gam, sig)


class _StepKeepUJ(torch.autograd.Function):
    """One rk3_step with per-step checkpointing that keeps the step's U, J (and SFS) values.
    The state is (x, gam, sig) or, with a DynamicSFS, (x, gam, sig, C)."""

    @staticmethod
    def forward(ctx, dt, kw, *state):
        kept, kept_sfs = [], []

        def record(x_, g_, s_, kernel, precision, vctx):
            U, J = UJFunction.apply(x_, g_, s_, kernel, precision, vctx)
            kept.append((U, J))
            return U, J

        def record_sfs(x_, g_, s_, J_, kernel, precision, transposed, vctx):
            S = EstrFunction.apply(x_, g_, s_, J_, kernel, precision, transposed, vctx)
            kept_sfs.append(S)
            return S
        with torch.no_grad():
            out = rk3_step(*state[:3], dt, C=state[3] if len(state) > 3 else None, uj_fn=record,
                           estr_fn=record_sfs, **kw)
        ctx.save_for_backward(*state)
        ctx.kept, ctx.kept_sfs, ctx.dt, ctx.kw = kept, kept_sfs, dt, kw
        return out

    @staticmethod
    def backward(ctx, *grads):
        state = [t.detach().requires_grad_() for t in ctx.saved_tensors]
        kept, kept_sfs = iter(ctx.kept), iter(ctx.kept_sfs)

        def replay(x_, g_, s_, kernel, precision, vctx):
            U, J = next(kept)
            return _KeptUJ.apply(x_, g_, s_, U, J, kernel, precision, vctx)

        def replay_sfs(x_, g_, s_, J_, kernel, precision, transposed, vctx):
            return _KeptEstr.apply(x_, g_, s_, J_, next(kept_sfs), kernel, precision, transposed, vctx)
        with torch.enable_grad():
            out = rk3_step(*state[:3], ctx.dt, C=state[3] if len(state) > 3 else None, uj_fn=replay,
                           estr_fn=replay_sfs, **ctx.kw)
        outs = [o for o, gr in zip(out, grads) if gr is not None]
        torch.autograd.backward(outs, [gr for gr in grads if gr is not None])
        return (None, None) + tuple(t.grad for t in state)


def rollout(x, gam, sig, dt: float, nsteps: int, *, checkpoint=True, C=None, **kw):
    """nsteps of rk3_step.  checkpoint=True: per-step checkpointing that keeps
    each step's UJ values (no pair sum is evaluated twice); "recompute": per-step
    checkpointing that re-runs each step in the backward pass; False: autograd
    keeps every intermediate.  With a DynamicSFS (kw["sfs"]) the state includes the
    coefficients C[n,3] (zeros when not given) and (x, gam, sig, C) is returned."""
    dynamic = isinstance(kw.get("sfs"), DynamicSFS)
    state = (x, gam, sig)
    if dynamic:
        state += (C if C is not None else torch.zeros(x.shape[0], 3, dtype=x.dtype, device=x.device),)
    for _ in range(nsteps):
        if checkpoint == "recompute":
            def step(*st):
                return rk3_step(*st[:3], dt, C=st[3] if len(st) > 3 else None, **kw)
            state = ckpt.checkpoint(step, *state, use_reentrant=False)
        elif checkpoint:
            state = _StepKeepUJ.apply(dt, kw, *state)
        else:
            state = rk3_step(*state[:3], dt, C=state[3] if dynamic else None, **kw)
    return tuple(state)


def ring_loss(x, gam, sig, *, kernel: int, precision: int = _lib.FP64, vctx: _lib.Context | None = None):
    """Kinetic-energy estimate E = 1/2 sum U_p . (x_p x Gamma_p) plus the
    strength-weighted axial centroid sum |Gamma_p| z_p / sum |Gamma_p|."""
    U, _ = UJFunction.apply(x, gam, sig, kernel, precision, vctx or _lib.default_context())
    E = 0.5 * (U * torch.cross(x, gam, dim=1)).sum()
    nG = torch.sqrt((gam * gam).sum(1))
    Z = (nG * x[:, 2]).sum() / nG.sum()
    return E + Z
