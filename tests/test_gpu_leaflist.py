"""Near-field P2P over octree leaf pairs (vpm_p2p_leaflist_dev), the direct leg
of UJ_fmm (src/FLOWVPM_UJ.jl:90-125) and Estr_fmm! over the same list
(src/FLOWVPM_subfilterscale_models.jl:94-188).

* the lists built on the GPU equal the host builder's (vpm_leaflist_host)
  entry for entry, on uniform, ring-shaped and duplicate-heavy clouds;
* theta = 0 makes every leaf pair near: the result must equal the all-pairs UJ;
* theta = 0.4 (the reference tests' value): U, J and SFS against the oracle
  evaluated over exactly the same leaf pairs (taken from vpm_leaflist_host);
* lists supplied by the caller (vpm_p2p_lists_dev) give the same result, and
  malformed lists are rejected before any device work.
"""
import numpy as np
import pytest

import oracle
from helpers import normwise, random_cloud

pytestmark = pytest.mark.gpu
TOL = {0: 1e-12, 1: 1e-6}


def _dev(a):
    import torch
    return torch.tensor(a, device="cuda").contiguous()


def _zeros(n, k):
    import torch
    return torch.zeros(n, k, device="cuda", dtype=torch.float64)


def _oracle_over_lists(X, G, s, J_all, static, lists, kernel, with_estr):
    perm, lb, le, row, col = lists
    n = X.shape[0]
    U = np.zeros((n, 3)); J = np.zeros((n, 9)); S = np.zeros((n, 3))
    for l in range(len(lb)):
        tg = perm[lb[l]:le[l]]
        src = np.concatenate([perm[lb[c]:le[c]] for c in col[row[l]:row[l + 1]]])
        Ut, Jt = oracle.uj_pairs(X[tg], X[src], G[src], s[src], kernel)
        U[tg] = Ut; J[tg] = Jt
    if with_estr:
        for l in range(len(lb)):
            tg = perm[lb[l]:le[l]]
            for t in tg:
                if static[t]:
                    continue
                src = np.concatenate([perm[lb[c]:le[c]] for c in col[row[l]:row[l + 1]]])
                src = src[src != t]
                S[t] = oracle.estr_pairs(X[t:t + 1], J_all[t:t + 1], X[src], G[src], s[src], J_all[src], kernel,
                                         True, None, static[src].astype(np.uint8))[0]
    return U, J, S


def _cloud(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        return rng.uniform(0, 1, (n, 3))
    if kind == "ring":
        th = rng.uniform(0, 2 * np.pi, n)
        return np.stack([np.cos(th), np.sin(th), 0.01 * rng.normal(size=n)], axis=1)
    x = rng.uniform(0, 1, (n, 3))
    x[: n // 2] = x[0]           # half the particles on one point: a leaf at full key depth
    return x


@pytest.mark.parametrize("kind,n,leaf,theta", [("uniform", 20000, 64, 0.4), ("uniform", 5000, 8, 0.5),
                                               ("ring", 8000, 16, 0.4), ("dup", 4000, 64, 0.4),
                                               ("uniform", 3000, 32, 0.0), ("uniform", 1, 64, 0.4),
                                               ("uniform", 70, 64, 0.4)])
def test_device_lists_equal_host_lists(ctx, kind, n, leaf, theta):
    import vpm_gb300._lib as L
    X = _cloud(kind, n, 11)
    host = L.leaflist_host(X, leaf, theta)
    dev = ctx.leaflist_dev(_dev(X), leaf, theta)
    for name, a, b in zip(("perm", "leaf_begin", "leaf_end", "row", "col"), dev[:5], host):
        assert np.array_equal(a, b), name
    perm, lb, le, row, col = host
    assert dev[5] == sum(int((le[l] - lb[l]) * (le[col[row[l]:row[l + 1]]] - lb[col[row[l]:row[l + 1]]]).sum())
                         for l in range(len(lb)))


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("k", [2, 3])
def test_theta_zero_equals_all_pairs(ctx, k, prec):
    n = 2500
    X, G, s = random_cloud(n, seed=50 + k, box=0.5)
    U, J = _zeros(n, 3), _zeros(n, 9)
    leaves, lpairs, pairs = ctx.p2p_leaflist_dev(_dev(X), _dev(G), _dev(s), U, J, leaf_size=64, theta=0.0,
                                                 kernel=k, precision=prec)
    assert pairs == n * n and lpairs == leaves * leaves
    Ur, Jr = oracle.uj_pairs(X, X, G, s, k)
    assert normwise(U.cpu().numpy(), Ur)[0] <= TOL[prec]
    assert normwise(J.cpu().numpy(), Jr)[0] <= TOL[prec]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("k", [0, 2, 3])
def test_theta_04_matches_oracle_over_the_same_leaf_pairs(ctx, k, prec):
    import vpm_gb300._lib as L
    n = 6000
    X, G, s = random_cloud(n, seed=60 + k)
    lists = L.leaflist_host(X, 48, 0.4)
    U, J = _zeros(n, 3), _zeros(n, 9)
    stats = ctx.p2p_leaflist_dev(_dev(X), _dev(G), _dev(s), U, J, leaf_size=48, theta=0.4, kernel=k,
                                 precision=prec)
    perm, lb, le, row, col = lists
    assert stats[0] == len(lb) and stats[1] == len(col)
    assert stats[2] < n * n   # a genuine near field
    Ur, Jr, _ = _oracle_over_lists(X, G, s, None, None, lists, k, False)
    assert normwise(U.cpu().numpy(), Ur)[0] <= TOL[prec]
    assert normwise(J.cpu().numpy(), Jr)[0] <= TOL[prec]


@pytest.mark.parametrize("prec", [0, 1])
def test_leaflist_estr_with_statics(ctx, prec):
    import vpm_gb300._lib as L
    n = 1500
    X, G, s = random_cloud(n, seed=71, box=0.4)
    static = (np.arange(n) % 13 == 0)
    lists = L.leaflist_host(X, 32, 0.4)
    U, J, S = _zeros(n, 3), _zeros(n, 9), _zeros(n, 3)
    ctx.p2p_leaflist_dev(_dev(X), _dev(G), _dev(s), U, J, S, leaf_size=32, theta=0.4, kernel=2, precision=prec,
                         sfs=True, static=_dev(static.astype(np.uint8)))
    Jg = J.cpu().numpy()
    # the oracle's Estr uses the GPU's J (as UJ_fmm's Estr uses the J just computed)
    _, _, Sr = _oracle_over_lists(X, G, s, Jg, static, lists, 2, True)
    assert normwise(S.cpu().numpy(), Sr)[0] <= (1e-12 if prec == 0 else 2e-6)
    assert not S.cpu().numpy()[static].any()


@pytest.mark.parametrize("prec", [0, 1])
def test_large_leaves_and_duplicates(ctx, prec):
    """leaf_size above a warp, and 2000 particles on one point (a leaf larger than leaf_size)."""
    import vpm_gb300._lib as L
    n = 4000
    X = _cloud("dup", n, 5)
    rng = np.random.default_rng(6)
    G = rng.normal(0, 1e-3, (n, 3)); s = rng.uniform(0.01, 0.03, n)
    for leaf in (200, 64):
        lists = L.leaflist_host(X, leaf, 0.4)
        U, J = _zeros(n, 3), _zeros(n, 9)
        ctx.p2p_leaflist_dev(_dev(X), _dev(G), _dev(s), U, J, leaf_size=leaf, theta=0.4, kernel=2, precision=prec)
        Ur, Jr, _ = _oracle_over_lists(X, G, s, None, None, lists, 2, False)
        assert normwise(U.cpu().numpy(), Ur)[0] <= TOL[prec]
        assert normwise(J.cpu().numpy(), Jr)[0] <= TOL[prec]


@pytest.mark.parametrize("prec", [0, 1])
def test_caller_lists_match_built_lists(ctx, prec):
    import vpm_gb300._lib as L
    n = 5000
    X, G, s = random_cloud(n, seed=81)
    perm, lb, le, row, col = L.leaflist_host(X, 32, 0.4)
    # rows in a scrambled order: the library sorts each row
    rng = np.random.default_rng(2)
    col2 = col.copy()
    for l in range(len(lb)):
        rng.shuffle(col2[row[l]:row[l + 1]])
    U1, J1, S1 = _zeros(n, 3), _zeros(n, 9), _zeros(n, 3)
    U2, J2, S2 = _zeros(n, 3), _zeros(n, 9), _zeros(n, 3)
    st1 = ctx.p2p_leaflist_dev(_dev(X), _dev(G), _dev(s), U1, J1, S1, leaf_size=32, theta=0.4, kernel=2,
                               precision=prec, sfs=True)
    st2 = ctx.p2p_lists_dev(_dev(X), _dev(G), _dev(s), U2, J2, (perm, lb, le, row, col2), S2, kernel=2,
                            precision=prec, sfs=True)
    assert st1 == st2
    for a, b in ((U1, U2), (J1, J2), (S1, S2)):
        assert torch_equal(a, b)


def torch_equal(a, b):
    import torch
    return bool(torch.equal(a, b))


def test_malformed_caller_lists_are_rejected(ctx):
    import vpm_gb300._lib as L
    n = 500
    X, G, s = random_cloud(n, seed=82)
    perm, lb, le, row, col = L.leaflist_host(X, 32, 0.4)
    args = (_dev(X), _dev(G), _dev(s), _zeros(n, 3), _zeros(n, 9))
    bad_perm = perm.copy(); bad_perm[0] = bad_perm[1]
    gap = le.copy(); gap[0] -= 1
    dup = col.copy(); dup[1] = dup[0]
    oor = col.copy(); oor[0] = len(lb)
    for lists in ((bad_perm, lb, le, row, col), (perm, lb, gap, row, col), (perm, lb, le, row, dup),
                  (perm, lb, le, row, oor)):
        with pytest.raises(L.VPMError) as ei:
            ctx.p2p_lists_dev(*args, lists, kernel=2, precision=1)
        assert ei.value.code == L.ERR_ARG
