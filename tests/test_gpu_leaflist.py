"""Near-field P2P over octree leaf pairs (vpm_p2p_leaflist_dev), the direct leg
of UJ_fmm (src/FLOWVPM_UJ.jl:90-125) and Estr_fmm! over the same list
(src/FLOWVPM_subfilterscale_models.jl:94-188).

* theta = 0 makes every leaf pair near: the result must equal the all-pairs UJ;
* theta = 0.4 (the reference tests' value): U, J and SFS against the oracle
  evaluated over exactly the same leaf pairs (taken from vpm_leaflist_host).
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
    assert normwise(S.cpu().numpy(), Sr)[0] <= (1e-12 if prec == 0 else 1e-5)
    assert not S.cpu().numpy()[static].any()
