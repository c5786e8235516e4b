"""GPU adjoint of UJ (vpm_uj_adjoint_dev) and gradients of rVPM rollouts.

* the adjoint kernel against the oracle's adjoint (oracle_uj_adjoint, itself
  checked against finite differences on the CPU): normwise <= 1e-11;
* UJFunction (forward vpm_uj_dev, backward vpm_uj_adjoint_dev) against central
  differences of the FP64 GPU forward;
* the gradient of a ring rollout loss (kinetic-energy estimate + axial
  centroid) with respect to the initial X, Gamma, sigma against central
  differences (h = 1e-6) on random directions: relative error <= 1e-5;
* both per-step checkpointing forms give the same gradient as keeping every step.
"""
import numpy as np
import pytest

import oracle
from helpers import normwise, random_cloud

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()


@pytest.mark.parametrize("k", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [1, 130, 700])
def test_adjoint_kernel_matches_oracle(ctx, k, n):
    import torch
    X, G, s = random_cloud(n, seed=40 + n + k, box=0.15)
    rng = np.random.default_rng(k)
    Ub = rng.normal(size=(n, 3))
    Jb = rng.normal(size=(n, 9))
    xb, gb, sb = (torch.zeros(n, 3, device="cuda", dtype=torch.float64),
                  torch.zeros(n, 3, device="cuda", dtype=torch.float64),
                  torch.zeros(n, device="cuda", dtype=torch.float64))
    ctx.uj_adjoint_dev(_dev(X), _dev(G), _dev(s), _dev(Ub), _dev(Jb), xb, gb, sb, k)
    rx, rg, rs = oracle.uj_adjoint(X, G, s, Ub, Jb, k)
    if n > 1:
        assert normwise(xb.cpu().numpy(), rx)[0] <= 1e-11
        assert normwise(gb.cpu().numpy(), rg)[0] <= 1e-11
        if k != 0:
            assert normwise(sb.cpu().numpy(), rs)[0] <= 1e-11
    else:
        assert not xb.abs().sum() and not gb.abs().sum() and not sb.abs().sum()


@pytest.mark.parametrize("k", [2, 3])
def test_ujfunction_backward_matches_central_differences(ctx, k):
    import torch
    from vpm_gb300.autodiff import UJFunction
    n = 300
    X, G, s = random_cloud(n, seed=7, box=0.12, gamma_std=1.0, sig_lo=0.02, sig_hi=0.04)
    rng = np.random.default_rng(8)
    Ub = _dev(rng.normal(size=(n, 3)))
    Jb = _dev(rng.normal(size=(n, 9)))
    x, g, sg = _dev(X).requires_grad_(), _dev(G).requires_grad_(), _dev(s).requires_grad_()
    U, J = UJFunction.apply(x, g, sg, k, 0, ctx)
    L = (U * Ub).sum() + (J * Jb).sum()
    L.backward()

    def loss(dx, dg, ds):
        with torch.no_grad():
            U, J = UJFunction.apply(x + dx, g + dg, sg + ds, k, 0, ctx)
            return float((U * Ub).sum() + (J * Jb).sum())
    h = 1e-6
    for _ in range(4):
        dx = _dev(rng.normal(size=(n, 3)))
        dg = _dev(rng.normal(size=(n, 3)))
        ds = _dev(rng.normal(size=n)) * 0.02
        fd = (loss(h * dx, h * dg, h * ds) - loss(-h * dx, -h * dg, -h * ds)) / (2 * h)
        an = float((x.grad * dx).sum() + (g.grad * dg).sum() + (sg.grad * ds).sum())
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1.0), (fd, an)


def _ring_state(nphi=20, nper=7):
    import vpm_gb300.rings as rings
    X, G, s, _ = rings.ring_sections(1.0, 1.0, 0.1, nphi, nper, 0.05)
    return _dev(X), _dev(G), _dev(s)


def test_rollout_gradient_matches_central_differences(ctx):
    import torch
    from vpm_gb300 import autodiff as ad
    x0, g0, s0 = _ring_state()
    kw = dict(kernel=2, precision=0, vctx=ctx)
    x, g, s = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
    xf, gf, sf = ad.rollout(x, g, s, 0.01, 3, checkpoint=True, **kw)
    L = ad.ring_loss(xf, gf, sf, **kw)
    L.backward()

    def loss(dx, dg, ds):
        with torch.no_grad():
            a, b, c = ad.rollout(x0 + dx, g0 + dg, s0 + ds, 0.01, 3, checkpoint=False, **kw)
            return float(ad.ring_loss(a, b, c, **kw))
    rng = np.random.default_rng(3)
    h = 1e-6
    worst = 0.0
    for _ in range(8):
        d = rng.normal(size=x0.numel() + g0.numel() + s0.numel())
        d /= np.linalg.norm(d)
        dx = _dev(d[:x0.numel()].reshape(x0.shape))
        dg = _dev(d[x0.numel():x0.numel() + g0.numel()].reshape(g0.shape))
        ds = _dev(d[x0.numel() + g0.numel():])
        fd = (loss(h * dx, h * dg, h * ds) - loss(-h * dx, -h * dg, -h * ds)) / (2 * h)
        an = float((x.grad * dx).sum() + (g.grad * dg).sum() + (s.grad * ds).sum())
        rel = abs(fd - an) / max(abs(an), 1e-300)
        worst = max(worst, rel)
        assert rel <= 1e-5, (fd, an, rel)


def test_checkpointing_does_not_change_the_gradient(ctx):
    from vpm_gb300 import autodiff as ad
    grads = []
    for ck in (True, "recompute", False):
        x0, g0, s0 = _ring_state(nphi=12)
        x, g, s = x0.requires_grad_(), g0.requires_grad_(), s0.requires_grad_()
        xf, gf, sf = ad.rollout(x, g, s, 0.01, 2, checkpoint=ck, kernel=3, precision=0, vctx=ctx)
        ad.ring_loss(xf, gf, sf, kernel=3, precision=0, vctx=ctx).backward()
        grads.append([t.grad.cpu().numpy() for t in (x, g, s)])
    for other in grads[1:]:
        for a, b in zip(grads[0], other):
            assert normwise(a, b)[0] <= 1e-12


def test_rollout_matches_host_mirror_step(ctx):
    """The torch rk3_step is the same step as the host mirror's rungekutta3 +
    Pedrizzetti relaxation (the reference's update) on the same UJ."""
    import vpm_gb300 as vpm
    from vpm_gb300 import autodiff as ad
    x0, g0, s0 = _ring_state(nphi=16)
    xa, ga, sa = ad.rk3_step(x0, g0, s0, 0.01, kernel=2, precision=0, vctx=ctx)
    pf = vpm.ParticleField(x0.shape[0], kernel=vpm.gaussianerf, relaxation=vpm.pedrizzetti, UJ=vpm.UJ_gb300)
    pf.add_particles(x0.cpu().numpy(), g0.cpu().numpy(), s0.cpu().numpy())
    pf.nextstep(0.01, relax=True)
    assert normwise(xa.cpu().numpy(), pf.X)[0] <= 1e-12
    assert normwise(ga.cpu().numpy(), pf.Gamma)[0] <= 1e-12
    assert normwise(sa.cpu().numpy(), pf.sigma)[0] <= 1e-12


@pytest.mark.parametrize("k", [0, 2, 3])
@pytest.mark.parametrize("cloud", ["dense", "spread"])
def test_mixed_adjoint_kernel_matches_oracle(ctx, k, cloud):
    """The FP32-comp adjoint against the oracle's FP64 adjoint: normwise <= 2e-6
    (dense: every pair near; spread: mostly the singular form)."""
    import torch
    n = 3000
    X, G, s = random_cloud(n, seed=90 + k, box=0.15 if cloud == "dense" else 2.0)
    rng = np.random.default_rng(k + 5)
    Ub = rng.normal(size=(n, 3))
    Jb = rng.normal(size=(n, 9))
    z = lambda *sh: torch.zeros(*sh, device="cuda", dtype=torch.float64)
    xb, gb, sb = z(n, 3), z(n, 3), z(n)
    ctx.uj_adjoint_dev(_dev(X), _dev(G), _dev(s), _dev(Ub), _dev(Jb), xb, gb, sb, k, 1)
    rx, rg, rs = oracle.uj_adjoint(X, G, s, Ub, Jb, k)
    assert normwise(xb.cpu().numpy(), rx)[0] <= 2e-6
    assert normwise(gb.cpu().numpy(), rg)[0] <= 2e-6
    if k != 0:
        assert normwise(sb.cpu().numpy(), rs)[0] <= 2e-6


def test_mixed_rollout_gradient_follows_fp64(ctx):
    """A ring rollout differentiated in FP32-comp (forward and adjoint) against
    the FP64 gradient of the same rollout: relative difference <= 1e-4."""
    from vpm_gb300 import autodiff as ad
    grads = []
    for prec in (0, 1):
        x0, g0, s0 = _ring_state(nphi=40)
        x, g, s = x0.requires_grad_(), g0.requires_grad_(), s0.requires_grad_()
        kw = dict(kernel=2, precision=prec, vctx=ctx)
        ad.ring_loss(*ad.rollout(x, g, s, 0.01, 3, checkpoint=True, **kw), **kw).backward()
        grads.append([t.grad.cpu().numpy() for t in (x, g, s)])
    for a, b in zip(grads[1], grads[0]):
        assert normwise(a, b)[0] <= 1e-4


def test_fifty_step_rollout_gradient_on_64_directions(ctx):
    """The rollout check at the length the adjoint workload names -- 50 RK3 steps
    (dt = 0.01) with Pedrizzetti relaxation, per-step checkpointing -- on the
    1400-particle ring (200 sections x 7), against central differences (h = 1e-6)
    of the FP64 forward along 64 seeded random directions: relative error <= 1e-5."""
    import torch
    from vpm_gb300 import autodiff as ad
    x0, g0, s0 = _ring_state(nphi=200, nper=7)
    kw = dict(kernel=2, precision=0, vctx=ctx)   # rk3_step relaxes with rlxf = 0.3 by default
    x, g, s = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
    ad.ring_loss(*ad.rollout(x, g, s, 0.01, 50, checkpoint=True, **kw), **kw).backward()

    def loss(dx, dg, ds):
        with torch.no_grad():
            return float(ad.ring_loss(*ad.rollout(x0 + dx, g0 + dg, s0 + ds, 0.01, 50, checkpoint=False, **kw),
                                      **kw))
    rng = np.random.default_rng(64)
    h = 1e-6
    rels = []
    for _ in range(64):
        d = rng.normal(size=x0.numel() + g0.numel() + s0.numel())
        d /= np.linalg.norm(d)
        dx = _dev(d[:x0.numel()].reshape(x0.shape))
        dg = _dev(d[x0.numel():x0.numel() + g0.numel()].reshape(g0.shape))
        ds = _dev(d[x0.numel() + g0.numel():])
        fd = (loss(h * dx, h * dg, h * ds) - loss(-h * dx, -h * dg, -h * ds)) / (2 * h)
        an = float((x.grad * dx).sum() + (g.grad * dg).sum() + (s.grad * ds).sum())
        rels.append(abs(fd - an) / max(abs(an), 1e-300))
    assert max(rels) <= 1e-5, max(rels)
