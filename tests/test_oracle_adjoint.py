"""The oracle's UJ adjoint (oracle_uj_adjoint) against central finite
differences of the oracle's FP64 forward (CPU only).  This checks the per-pair
derivative used by the GPU adjoint kernel: L = sum(Ubar*U) + sum(Jbar*J)."""

import numpy as np
import pytest

import oracle


def _loss(x, g, s, Ub, Jb, k):
    U, J = oracle.uj_pairs(x, x, g, s, k)
    return float((Ub * U).sum() + (Jb * J).sum())


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_adjoint_matches_central_differences(k):
    rng = np.random.default_rng(10 + k)
    n = 14
    x = rng.uniform(0, 0.12, (n, 3))
    g = rng.normal(0, 1.0, (n, 3))
    s = rng.uniform(0.03, 0.06, n)
    Ub = rng.normal(size=(n, 3))
    Jb = rng.normal(size=(n, 9))
    xb, gb, sb = oracle.uj_adjoint(x, g, s, Ub, Jb, k)
    h = 1e-6
    for trial in range(6):
        dx = rng.normal(size=x.shape)
        dg = rng.normal(size=g.shape)
        ds = rng.normal(size=s.shape) * (0 if k == 0 else 1)
        # scale so each perturbation moves the inputs by ~h relative
        fd = (_loss(x + h * dx, g + h * dg, s + h * 0.05 * ds, Ub, Jb, k)
              - _loss(x - h * dx, g - h * dg, s - h * 0.05 * ds, Ub, Jb, k)) / (2 * h)
        an = (xb * dx).sum() + (gb * dg).sum() + 0.05 * (sb * ds).sum()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (trial, fd, an)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_kernel_second_derivative(k):
    for rho in (0.2, 0.9, 1.6, 2.5):
        g, d1, d2 = oracle.g_d1_d2(k, rho)
        h = 1e-5
        fd = (oracle.g_d1_d2(k, rho + h)[1] - oracle.g_d1_d2(k, rho - h)[1]) / (2 * h)
        assert abs(fd - d2) <= 1e-7 * max(1.0, abs(d2))
        assert abs(g - oracle.g_dgdr(k, rho)[0]) <= 1e-15 and abs(d1 - oracle.g_dgdr(k, rho)[1]) <= 1e-15


def _estr_loss(x, g, s, J, Sb, k, transposed, static):
    S = oracle.estr_pairs(x, J, x, g, s, J, k, transposed, static, static)
    return float((Sb * S).sum())


@pytest.mark.parametrize("transposed", [True, False])
@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_estr_adjoint_matches_central_differences(k, transposed):
    """oracle_estr_adjoint (the pullback of Estr, src/FLOWVPM_subfilterscale_models.jl:16-92,
    with respect to x, Gamma, sigma and J) against central differences of the oracle's
    FP64 Estr, statics included; two particles coincide (a pair at r = 0, s != t)."""
    rng = np.random.default_rng(30 + k + 4 * transposed)
    n = 16
    x = rng.uniform(0, 0.12, (n, 3))
    x[5] = x[9]
    g = rng.normal(0, 1.0, (n, 3))
    s = rng.uniform(0.03, 0.06, n)
    J = rng.normal(0, 1.0, (n, 9))
    static = (np.arange(n) % 6 == 2).astype(np.uint8)
    Sb = rng.normal(size=(n, 3))
    xb, gb, sb, Jb = oracle.estr_adjoint(x, g, s, J, Sb, k, transposed, static)
    assert not xb[static == 1].any() and not gb[static == 1].any() and not Jb[static == 1].any()
    h = 1e-6
    for trial in range(6):
        dx = rng.normal(size=x.shape)
        dx[5] = dx[9]          # keep the coincident pair coincident (r = 0 is not differentiable)
        dg = rng.normal(size=g.shape)
        ds = rng.normal(size=s.shape) * 0.05
        dJ = rng.normal(size=J.shape)
        fd = (_estr_loss(x + h * dx, g + h * dg, s + h * ds, J + h * dJ, Sb, k, transposed, static)
              - _estr_loss(x - h * dx, g - h * dg, s - h * ds, J - h * dJ, Sb, k, transposed, static)) / (2 * h)
        an = (xb * dx).sum() + (gb * dg).sum() + (sb * ds).sum() + (Jb * dJ).sum()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (trial, fd, an)
