"""Parity at the sizes of the stated workloads (GPU).

* random cloud, plain FP64 form (pair loop src/FLOWVPM_fmm.jl:102-168), the
  Gaussian-erf and Winckelmans kernels: N = 2^14 every target, N = 2^17 (the
  all-pairs self evaluation) and N = 2^20 (512 seeded targets against all 2^20
  sources) within 1e-12 normwise of the oracle, against both its plain and its
  compensated summation;
* the jet-like cloud with the FMM near field (UJ_fmm's direct leg,
  src/FLOWVPM_UJ.jl:90-125, and Estr_fmm!, src/FLOWVPM_subfilterscale_models.jl:94-188)
  at N = 2^20, leaf size 64, theta = 0.4: the GPU-built lists equal the host
  builder's entry for entry; FP64 and FP32-comp U, J, SFS on 256 seeded
  targets against the oracle over exactly the same leaf pairs;
* the list builder's overflow path: buffers that start far too small grow and
  the traversal is repeated, with lists equal to a normal build;
* the adjoint rollout at its stated size, the 32,000-particle ring (1000
  sections x 32): the gradient of a 5-step FP64 rollout against central
  differences (h = 1e-6) along 8 seeded directions.
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


def _zeros(n, k):
    import torch
    return torch.zeros(n, k, device="cuda", dtype=torch.float64)


def _check_fp64(Uh, Jh, X_t, X, G, s, k, tol=1e-12):
    """GPU FP64 against the oracle in plain and in compensated summation."""
    for comp in (False, True):
        Ur, Jr = oracle.uj_pairs(X_t, X, G, s, k, compensated=comp)
        eu, ej = normwise(Uh, Ur)[0], normwise(Jh, Jr)[0]
        assert eu <= tol and ej <= tol, (comp, eu, ej)


@pytest.mark.parametrize("k", [2, 3])
def test_fp64_random_cloud_2p14_every_target(ctx, k):
    n = 1 << 14
    X, G, s = random_cloud(n, seed=14)
    x = _dev(X)
    U, J = _zeros(n, 3), _zeros(n, 9)
    ctx.uj_dev(x, x, _dev(G), _dev(s), U, J, k, FP64)
    _check_fp64(U.cpu().numpy(), J.cpu().numpy(), X, X, G, s, k)


@pytest.mark.parametrize("k", [2, 3])
def test_fp64_random_cloud_2p17_all_pairs_subset(ctx, k):
    n = 1 << 17
    X, G, s = random_cloud(n, seed=17)
    x = _dev(X)
    U, J = _zeros(n, 3), _zeros(n, 9)
    ctx.uj_dev(x, x, _dev(G), _dev(s), U, J, k, FP64)
    sub = np.sort(np.random.default_rng(3).choice(n, 512, replace=False))
    _check_fp64(U.cpu().numpy()[sub], J.cpu().numpy()[sub], X[sub], X, G, s, k)


@pytest.mark.parametrize("k", [2, 3])
def test_fp64_random_cloud_2p20_seeded_targets(ctx, k):
    """512 seeded targets against every one of the 2^20 sources (the same kernel
    as the all-pairs call, whose 2^40 FP64 pairs take minutes)."""
    n = 1 << 20
    X, G, s = random_cloud(n, seed=20)
    sub = np.sort(np.random.default_rng(4).choice(n, 512, replace=False))
    U, J = _zeros(512, 3), _zeros(512, 9)
    ctx.uj_dev(_dev(X[sub]), _dev(X), _dev(G), _dev(s), U, J, k, FP64)
    _check_fp64(U.cpu().numpy(), J.cpu().numpy(), X[sub], X, G, s, k)


# ------------------------------------------------------------------ jet cloud
@pytest.fixture(scope="module")
def jet():
    """The jet-like cloud of the FMM workload at 2^20 and its host-built lists."""
    import vpm_gb300._lib as L
    from vpm_gb300 import workloads
    X, G, s = workloads.jet_cloud(1 << 20, seed=0)
    lists = L.leaflist_host(X, 64, 0.4)
    return X, G, s, lists


def test_jet_2p20_device_lists_equal_host_lists(ctx, jet):
    X, G, s, host = jet
    dev = ctx.leaflist_dev(_dev(X), 64, 0.4)
    for name, a, b in zip(("perm", "leaf_begin", "leaf_end", "row", "col"), dev[:5], host):
        assert np.array_equal(a, b), name
    perm, lb, le, row, col = host
    sz = le - lb
    assert dev[5] == int((sz[np.repeat(np.arange(len(lb)), np.diff(row))] * sz[col]).sum())


def _near_sources(lists, t_pos):
    perm, lb, le, row, col = lists
    leaf = np.searchsorted(lb, t_pos, side="right") - 1
    return np.concatenate([perm[lb[c]:le[c]] for c in col[row[leaf]:row[leaf + 1]]])


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
def test_jet_2p20_near_field_uj_and_sfs_match_oracle_over_same_lists(ctx, jet, prec):
    X, G, s, lists = jet
    n = X.shape[0]
    U, J, S = _zeros(n, 3), _zeros(n, 9), _zeros(n, 3)
    stats = ctx.p2p_leaflist_dev(_dev(X), _dev(G), _dev(s), U, J, S, leaf_size=64, theta=0.4, kernel=2,
                                 precision=prec, sfs=True)
    perm = lists[0]
    assert stats[0] == len(lists[1]) and stats[1] == len(lists[4])
    pos_of = np.empty(n, np.int64)
    pos_of[perm] = np.arange(n)
    tg = np.sort(np.random.default_rng(256).choice(n, 256, replace=False))
    Uh, Jh, Sh = U.cpu().numpy(), J.cpu().numpy(), S.cpu().numpy()
    Ur = np.zeros((256, 3)); Jr = np.zeros((256, 9)); Sr = np.zeros((256, 3))
    npairs = 0
    for i, t in enumerate(tg):
        src = _near_sources(lists, pos_of[t])
        npairs += len(src)
        Ur[i], Jr[i] = (a[0] for a in oracle.uj_pairs(X[t:t + 1], X[src], G[src], s[src], 2))
        src = src[src != t]
        # Estr over the same pairs, from the J this very call computed (as UJ_fmm's Estr does)
        Sr[i] = oracle.estr_pairs(X[t:t + 1], Jh[t:t + 1], X[src], G[src], s[src], Jh[src], 2, True)[0]
    assert npairs > 256 * 500   # a genuine near field at the jet's density
    tol_uj, tol_sfs = (1e-12, 1e-12) if prec == FP64 else (1e-6, 2e-6)
    assert normwise(Uh[tg], Ur)[0] <= tol_uj
    assert normwise(Jh[tg], Jr)[0] <= tol_uj
    assert normwise(Sh[tg], Sr)[0] <= tol_sfs


def test_list_builder_overflow_retries_to_equal_lists(ctx):
    import vpm_gb300
    X = random_cloud(20000, seed=12)[0]
    ref = ctx.leaflist_dev(_dev(X), 64, 0.4)
    small = vpm_gb300.Context(0)
    small.set_near_capacity(64, 64)   # the first frontiers and the near list overflow at once
    got = small.leaflist_dev(_dev(X), 64, 0.4)
    for name, a, b in zip(("perm", "leaf_begin", "leaf_end", "row", "col"), got[:5], ref[:5]):
        assert np.array_equal(a, b), name
    assert got[5] == ref[5]
    # a near list alone too small: one repeat with the counted size
    small.set_near_capacity(40 * 20000, 100)
    got = small.leaflist_dev(_dev(X), 64, 0.4)
    assert np.array_equal(got[4], ref[4]) and got[5] == ref[5]
    small.close()


# ------------------------------------------------------------ adjoint rollout
def test_rollout_gradient_32k_ring_eight_directions(ctx):
    """The ring of the adjoint workload at its stated size (32,000 particles),
    5 FP64 RK3 steps with relaxation, per-step checkpointing; central
    differences (h = 1e-6) of the FP64 forward on 8 seeded directions agree
    with the gradient to 1e-5 relative."""
    import torch
    import vpm_gb300.rings as rings
    from vpm_gb300 import autodiff as ad
    X, G, s, _ = rings.ring_sections(1.0, 1.0, 0.1, 1000, 32, 0.05)
    x0, g0, s0 = _dev(X), _dev(G), _dev(s)
    kw = dict(kernel=2, precision=FP64, vctx=ctx)
    steps = 5
    x, g, sg = x0.clone().requires_grad_(), g0.clone().requires_grad_(), s0.clone().requires_grad_()
    ad.ring_loss(*ad.rollout(x, g, sg, 0.01, steps, checkpoint=True, **kw), **kw).backward()

    def loss(dx, dg, ds):
        with torch.no_grad():
            return float(ad.ring_loss(*ad.rollout(x0 + dx, g0 + dg, s0 + ds, 0.01, steps, checkpoint=False, **kw),
                                      **kw))
    rng = np.random.default_rng(32000)
    h = 1e-6
    rels = []
    for _ in range(8):
        d = rng.normal(size=x0.numel() + g0.numel() + s0.numel())
        d /= np.linalg.norm(d)
        dx = _dev(d[:x0.numel()].reshape(x0.shape))
        dg = _dev(d[x0.numel():x0.numel() + g0.numel()].reshape(g0.shape))
        ds = _dev(d[x0.numel() + g0.numel():])
        fd = (loss(h * dx, h * dg, h * ds) - loss(-h * dx, -h * dg, -h * ds)) / (2 * h)
        an = float((x.grad * dx).sum() + (g.grad * dg).sum() + (sg.grad * ds).sum())
        rels.append(abs(fd - an) / max(abs(an), 1e-300))
    assert max(rels) <= 1e-5, rels
