"""GPU adjoint of Estr (vpm_estr_adjoint_dev) and gradients of rVPM rollouts
with the constant-coefficient SFS model -- the pullback the reference's rrule
leaves unimplemented (src/FLOWVPM_rrules.jl:153-157).

* the adjoint kernels against the oracle's Estr adjoint (oracle_estr_adjoint,
  itself checked against central differences and 40-digit arithmetic on the
  CPU): FP64 normwise <= 1e-11 (all kernels, both schemes, static particles, a
  coincident pair), FP32-comp <= 2e-6 (J from the cloud's own UJ);
* the differentiable RK3 step with ConstantSFS (src/FLOWVPM_subfilterscale.jl:88-150)
  against the oracle's RK3 step with the same scheme: <= 1e-11 after 3 steps;
* the gradient of a ring rollout with the SFS term against central
  differences (h = 1e-6) of the FP64 forward on 64 seeded directions: <= 1e-5;
* the FP32-comp rollout gradient follows the FP64 one to 1e-4.
"""
import numpy as np
import pytest

import oracle
from helpers import normwise, random_cloud

pytestmark = pytest.mark.gpu
FP64, FP32COMP = 0, 1


def _dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)


def _z(*shape):
    import torch
    return torch.zeros(*shape, device="cuda", dtype=torch.float64)


def _flags(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a, dtype=np.uint8), device="cuda")


def _cmp(got, ref, tol, what):
    ref = np.asarray(ref)
    if not np.abs(ref).max() > 0:
        assert not np.abs(got).max() > 0, what
        return
    e = normwise(got, ref)[0]
    assert e <= tol, (what, e)


@pytest.mark.parametrize("n", [130, 700, 3000])
@pytest.mark.parametrize("transposed", [True, False])
@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_estr_adjoint_fp64_matches_oracle(ctx, k, transposed, n):
    X, G, s = random_cloud(n, seed=500 + n + k, box=0.15)
    X[7] = X[3]                                      # a coincident pair (r = 0, s != t)
    rng = np.random.default_rng(k + 10 * transposed)
    J = rng.normal(0, 1.0, (n, 9))
    static = (np.arange(n) % 11 == 4).astype(np.uint8)
    Sb = rng.normal(size=(n, 3))
    out = [_z(n, 3), _z(n, 3), _z(n), _z(n, 9)]
    ctx.estr_adjoint_dev(_dev(X), _dev(G), _dev(s), _dev(J), _dev(Sb), *out, k, FP64, transposed,
                         static=_flags(static))
    ref = oracle.estr_adjoint(X, G, s, J, Sb, k, transposed, static)
    for name, a, b in zip(("x", "Gamma", "sigma", "J"), out, ref):
        _cmp(a.cpu().numpy(), b, 1e-11, name)


@pytest.mark.parametrize("transposed", [True, False])
@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("n", [700, 3000])
def test_estr_adjoint_fp32comp_matches_oracle(ctx, k, transposed, n):
    """J is the cloud's own (smooth) velocity gradient, so J_t - J_s of near pairs is much
    smaller than J: the regime where Estr's factored sums cancel."""
    X, G, s = random_cloud(n, seed=600 + n + k, box=0.15, gamma_std=1.0)
    _, J = oracle.uj_pairs(X, X, G, s, k)
    static = (np.arange(n) % 13 == 5).astype(np.uint8)
    Sb = np.random.default_rng(k).normal(size=(n, 3))
    out = [_z(n, 3), _z(n, 3), _z(n), _z(n, 9)]
    ctx.estr_adjoint_dev(_dev(X), _dev(G), _dev(s), _dev(J), _dev(Sb), *out, k, FP32COMP, transposed,
                         static=_flags(static))
    ref = oracle.estr_adjoint(X, G, s, J, Sb, k, transposed, static)
    for name, a, b in zip(("x", "Gamma", "sigma", "J"), out, ref):
        _cmp(a.cpu().numpy(), b, 2e-6, name)


def test_estr_adjoint_singular_fp32comp_is_zero_without_coincident_pairs(ctx):
    """The singular kernel's zeta is the indicator of r = 0, and the FP32-comp Estr skips
    r = 0 (as its forward does): no gradient at all."""
    n = 500
    X, G, s = random_cloud(n, seed=7)
    J = np.random.default_rng(1).normal(size=(n, 9))
    out = [_z(n, 3), _z(n, 3), _z(n), _z(n, 9)]
    ctx.estr_adjoint_dev(_dev(X), _dev(G), _dev(s), _dev(J), _dev(np.ones((n, 3))), *out, 0, FP32COMP)
    assert all(float(t.abs().max()) == 0.0 for t in out)


def _ring(nphi=200, nper=7):
    import vpm_gb300.rings as rings
    X, G, s, _ = rings.ring_sections(1.0, 1.0, 0.1, nphi, nper, 0.05)
    return X, G, s


@pytest.mark.parametrize("clip", [False, True])
def test_constant_sfs_step_matches_oracle_step(ctx, clip):
    """rk3_step with ConstantSFS (FP64) against the oracle's RK3 step with the same
    scheme (src/FLOWVPM_timeintegration.jl:388-532, src/FLOWVPM_subfilterscale.jl:113-150),
    Pedrizzetti relaxation, 3 steps on the 1400-particle ring."""
    from vpm_gb300 import autodiff as ad
    X, G, s = _ring()
    n = X.shape[0]
    x, g, sg = _dev(X), _dev(G), _dev(s)
    sfs = ad.ConstantSFS(Cs=1.0, clip_backscatter=clip)
    for _ in range(3):
        x, g, sg = ad.rk3_step(x, g, sg, 0.01, kernel=2, precision=FP64, sfs=sfs, vctx=ctx)
    P = np.zeros((46, n), order="F")
    P[0:3] = X.T; P[3:6] = G.T; P[6] = s
    prm = oracle.StepParams(kernel=oracle.KERNEL_GAUSSIANERF, transposed=1, f=0.0, g=0.2, relaxation=1, rlxf=0.3,
                            sfs=1, Cs=1.0, clip_backscatter=int(clip))
    for _ in range(3):
        assert oracle.rk3_step(P, n, 0.01, prm, relax=True) == 0
    for name, a, b in (("x", x, P[0:3].T), ("Gamma", g, P[3:6].T), ("sigma", sg, P[6])):
        assert normwise(a.cpu().numpy(), b)[0] <= 1e-11, name


def _grad_and_fd(ctx, nsteps, ndirs, seed, sfs, precision=FP64):
    import torch
    from vpm_gb300 import autodiff as ad
    X, G, s = _ring()
    x0, g0, s0 = _dev(X), _dev(G), _dev(s)
    kw = dict(kernel=2, precision=precision, vctx=ctx, sfs=sfs)
    x, g, sg = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
    ad.ring_loss(*ad.rollout(x, g, sg, 0.01, nsteps, checkpoint=True, **kw), kernel=2, precision=precision,
                 vctx=ctx).backward()
    if ndirs == 0:
        return (x.grad, g.grad, sg.grad), []
    kw64 = dict(kw, precision=FP64)

    def loss(dx, dg, ds):
        with torch.no_grad():
            return float(ad.ring_loss(*ad.rollout(x0 + dx, g0 + dg, s0 + ds, 0.01, nsteps, checkpoint=False,
                                                  **kw64), kernel=2, precision=FP64, vctx=ctx))
    rng = np.random.default_rng(seed)
    h = 1e-6
    rels = []
    for _ in range(ndirs):
        d = rng.normal(size=x0.numel() + g0.numel() + s0.numel())
        d /= np.linalg.norm(d)
        dx = _dev(d[:x0.numel()].reshape(x0.shape))
        dg = _dev(d[x0.numel():x0.numel() + g0.numel()].reshape(g0.shape))
        ds = _dev(d[x0.numel() + g0.numel():])
        fd = (loss(h * dx, h * dg, h * ds) - loss(-h * dx, -h * dg, -h * ds)) / (2 * h)
        an = float((x.grad * dx).sum() + (g.grad * dg).sum() + (sg.grad * ds).sum())
        rels.append(abs(fd - an) / max(abs(an), 1e-300))
    return (x.grad, g.grad, sg.grad), rels


def test_sfs_rollout_gradient_on_64_directions(ctx):
    """10 RK3 steps of the ring with the ConstantSFS term (Cs = 1, no clipping: the
    clipping switch is piecewise constant and a difference across it is not a
    derivative) and relaxation: gradient vs central differences on 64 directions."""
    from vpm_gb300 import autodiff as ad
    _, rels = _grad_and_fd(ctx, 10, 64, 6400, ad.ConstantSFS(Cs=1.0))
    assert max(rels) <= 1e-5, max(rels)


def test_sfs_rollout_fp32comp_gradient_follows_fp64(ctx):
    from vpm_gb300 import autodiff as ad
    sfs = ad.ConstantSFS(Cs=1.0)
    g64, _ = _grad_and_fd(ctx, 3, 0, 0, sfs, FP64)
    g32, _ = _grad_and_fd(ctx, 3, 0, 0, sfs, FP32COMP)
    for a, b in zip(g32, g64):
        assert normwise(a.cpu().numpy(), b.cpu().numpy())[0] <= 1e-4


def _two_rings():
    import vpm_gb300.rings as rings
    X1, G1, s1, _ = rings.ring_sections(1.0, 1.0, 0.1, 40, 10, 0.05)
    X2, G2, s2, _ = rings.ring_sections(1.0, 0.7, 0.07, 28, 10, 0.035, O=(0, 0, 0.3))
    return np.vstack([X1, X2]), np.vstack([G1, G2]), np.concatenate([s1, s2])


@pytest.mark.parametrize("alpha,force_positive,clip", [(0.999, True, True), (0.667, False, False)])
def test_dynamic_sfs_step_matches_oracle_step(ctx, alpha, force_positive, clip):
    """rk3_step with the dynamic procedure (FP64: both filter widths evaluated and
    subtracted, as the reference does) against the oracle's RK3 step with the same
    scheme, 3 steps on a two-ring field; the coefficient state C is carried."""
    from vpm_gb300 import autodiff as ad
    X, G, s = _two_rings()
    n = X.shape[0]
    sfs = ad.DynamicSFS(alpha=alpha, rlxf=0.005, force_positive=force_positive, clip_backscatter=clip)
    st = (_dev(X), _dev(G), _dev(s), None)
    for _ in range(3):
        st = ad.rk3_step(*st[:3], 0.005, kernel=2, precision=FP64, sfs=sfs, C=st[3], relax=True, vctx=ctx)
    P = np.zeros((46, n), order="F")
    P[0:3] = X.T; P[3:6] = G.T; P[6] = s
    prm = oracle.StepParams(kernel=oracle.KERNEL_GAUSSIANERF, transposed=1, f=0.0, g=0.2, relaxation=1, rlxf=0.3,
                            sfs=2, alpha=alpha, sfs_rlxf=0.005, minC=0.0, maxC=1.0,
                            force_positive=int(force_positive), clip_backscatter=int(clip))
    for _ in range(3):
        assert oracle.rk3_step(P, n, 0.005, prm, relax=True) == 0
    for name, a, b in (("x", st[0], P[0:3].T), ("Gamma", st[1], P[3:6].T), ("sigma", st[2], P[6]),
                       ("C", st[3][:, 0], P[36])):
        assert normwise(a.cpu().numpy(), b)[0] <= 1e-10, name


def test_dynamic_sfs_rollout_gradient_on_32_directions(ctx):
    """5 RK3 steps of the two-ring field with the dynamic procedure (alpha = 0.667, the
    coefficient bounded to [0, 1], no clipping) and relaxation: the gradient of the loss
    with respect to the initial X, Gamma, sigma (C starting at zero) against central
    differences (h = 1e-6) of the FP64 forward on 32 seeded directions."""
    import torch
    from vpm_gb300 import autodiff as ad
    X, G, s = _two_rings()
    x0, g0, s0 = _dev(X), _dev(G), _dev(s)
    kw = dict(kernel=2, precision=FP64, vctx=ctx, sfs=ad.DynamicSFS(alpha=0.667, rlxf=0.005))
    x, g, sg = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
    out = ad.rollout(x, g, sg, 0.005, 5, checkpoint=True, **kw)
    ad.ring_loss(*out[:3], kernel=2, precision=FP64, vctx=ctx).backward()
    assert float(out[3][:, 0].detach().abs().max()) > 0          # the dynamic coefficient is active

    def loss(dx, dg, ds):
        with torch.no_grad():
            o = ad.rollout(x0 + dx, g0 + dg, s0 + ds, 0.005, 5, checkpoint=False, **kw)
            return float(ad.ring_loss(*o[:3], kernel=2, precision=FP64, vctx=ctx))
    rng = np.random.default_rng(3200)
    h = 1e-6
    rels = []
    for _ in range(32):
        d = rng.normal(size=x0.numel() + g0.numel() + s0.numel())
        d /= np.linalg.norm(d)
        dx = _dev(d[:x0.numel()].reshape(x0.shape))
        dg = _dev(d[x0.numel():x0.numel() + g0.numel()].reshape(g0.shape))
        ds = _dev(d[x0.numel() + g0.numel():])
        fd = (loss(h * dx, h * dg, h * ds) - loss(-h * dx, -h * dg, -h * ds)) / (2 * h)
        an = float((x.grad * dx).sum() + (g.grad * dg).sum() + (sg.grad * ds).sum())
        rels.append(abs(fd - an) / max(abs(an), 1e-300))
    assert max(rels) <= 1e-5, max(rels)


def test_dynamic_sfs_recompute_checkpointing_gives_the_same_gradient(ctx):
    from vpm_gb300 import autodiff as ad
    X, G, s = _two_rings()
    kw = dict(kernel=2, precision=FP64, vctx=ctx, sfs=ad.DynamicSFS(alpha=0.667, rlxf=0.005))
    grads = []
    for mode in (True, "recompute", False):
        x, g, sg = (_dev(a).requires_grad_() for a in (X, G, s))
        out = ad.rollout(x, g, sg, 0.005, 3, checkpoint=mode, **kw)
        ad.ring_loss(*out[:3], kernel=2, precision=FP64, vctx=ctx).backward()
        grads.append([t.grad.cpu().numpy() for t in (x, g, sg)])
    for other in grads[1:]:
        for a, b in zip(other, grads[0]):
            assert normwise(a, b)[0] <= 1e-12
