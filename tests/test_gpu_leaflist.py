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


@pytest.mark.parametrize("k,alpha", [(2, 0.999), (3, 0.999), (1, 0.999), (2, 0.667)])
def test_near_field_dynamic_differences(ctx, k, alpha):
    """vpm_dynamic_diff_leaflist_dev.  FP64 is the reference's way -- the near-field
    leg at alpha sigma and at sigma, subtracted -- and equals two vpm_p2p_leaflist_dev
    calls bit for bit; FP32-comp evaluates the differences directly and agrees with
    them to FP32 relative accuracy (subtracting two FP32 evaluations would leave
    ~1e-7 / (1 - alpha) of noise)."""
    from vpm_gb300 import workloads
    X, G, s = workloads.leapfrog_rings(3000, nper=10)
    n = X.shape[0]
    x, g, sg = _dev(np.ascontiguousarray(X)), _dev(np.ascontiguousarray(G)), _dev(np.ascontiguousarray(s))
    leaf, theta = 32, 0.4

    def near(sig):
        U, J, S = _zeros(n, 3), _zeros(n, 9), _zeros(n, 3)
        st = ctx.p2p_leaflist_dev(x, g, sig, U, J, S, leaf_size=leaf, theta=theta, kernel=k, precision=0, sfs=True)
        return J, S, st

    J0, S0, st0 = near(sg)
    Ja, Sa, _ = near(sg * alpha)
    assert st0[2] < n * n   # a genuine near field
    dJ_ref, dS_ref = (Ja - J0).cpu().numpy(), (Sa - S0).cpu().numpy()
    for prec, tolJ, tolS in ((0, 0.0, 0.0), (1, 2e-6, 2e-5)):
        dJ, dS = _zeros(n, 9), _zeros(n, 3)
        st = ctx.dynamic_diff_leaflist_dev(x, g, sg, J0, alpha, dJ, dS, leaf_size=leaf, theta=theta, kernel=k,
                                           precision=prec)
        assert st == st0
        if prec == 0:
            assert np.array_equal(dJ.cpu().numpy(), dJ_ref) and np.array_equal(dS.cpu().numpy(), dS_ref)
        else:
            eJ = normwise(dJ.cpu().numpy(), dJ_ref)[0]
            eS = normwise(dS.cpu().numpy(), dS_ref)[0]
            assert eJ <= tolJ and eS <= tolS, (eJ, eS)


def test_near_field_dynamic_differences_reject_bad_arguments(ctx):
    import vpm_gb300._lib as L
    n = 100
    X, G, s = random_cloud(n, seed=3)
    x, g, sg = _dev(X), _dev(G), _dev(s)
    J, dJ, dS = _zeros(n, 9), _zeros(n, 9), _zeros(n, 3)
    for kw in (dict(alpha=1.0), dict(alpha=0.0), dict(alpha=0.9, leaf_size=0), dict(alpha=0.9, theta=-1.0)):
        alpha = kw.pop("alpha")
        with pytest.raises(L.VPMError):
            ctx.dynamic_diff_leaflist_dev(x, g, sg, J, alpha, dJ, dS, **kw)
    # host memory where device pointers are required
    rc = ctx._L.vpm_dynamic_diff_leaflist_dev(ctx._h, n, X.ctypes.data, G.ctypes.data, s.ctypes.data, None,
                                              X.ctypes.data, 0.9, X.ctypes.data, X.ctypes.data, 32, 0.4, 2, 1, 0,
                                              None)
    assert rc == L.ERR_ARG


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("k", [1, 2, 3])
def test_near_field_zeta_matches_oracle_over_the_same_leaf_pairs(ctx, k, prec):
    """zeta_fmm (src/FLOWVPM_viscous.jl:523-556): the basis field summed over the
    near leaf pairs only, every particle a target, the self pair and a
    coincident pair included; W accumulates (+=) like the reference's loop."""
    import vpm_gb300._lib as L
    n = 5000
    X, G, s = random_cloud(n, seed=30 + k, box=0.5)
    X[9] = X[4]
    lists = L.leaflist_host(X, 32, 0.4)
    perm, lb, le, row, col = lists
    ref = np.zeros((n, 3))
    for l in range(len(lb)):
        tg = perm[lb[l]:le[l]]
        src = np.concatenate([perm[lb[c]:le[c]] for c in col[row[l]:row[l + 1]]])
        ref[tg] = oracle.zeta_pairs(X[tg], X[src], G[src], s[src], k)
    W = _zeros(n, 3)
    st = ctx.zeta_leaflist_dev(_dev(X), _dev(G), _dev(s), W, leaf_size=32, theta=0.4, kernel=k, precision=prec)
    assert st[2] < n * n and st[1] == len(col)
    assert normwise(W.cpu().numpy(), ref)[0] <= TOL[prec]
    ctx.zeta_leaflist_dev(_dev(X), _dev(G), _dev(s), W, leaf_size=32, theta=0.4, kernel=k, precision=prec)
    assert normwise(W.cpu().numpy(), 2 * ref)[0] <= TOL[prec]


def test_zeta_fmm_hook_adds_to_rows_16_18():
    """vpm.zeta_fmm_gb300 on the host matrix: rows 16:18 of every particle
    (statics included) += the near-field sum; nothing else changes."""
    import vpm_gb300 as vpm
    import vpm_gb300._lib as L
    n = 1200
    X, G, s = random_cloud(n, seed=77, box=0.4)
    static = np.zeros(n, bool)
    static[::13] = True
    pf = vpm.ParticleField(n + 3, kernel=vpm.gaussianerf)
    pf.add_particles(X, G, s, static=static)
    pf.particles[15:18, :n] = 0.5
    Q = pf.particles.copy(order="F")
    vpm.zeta_fmm_gb300(pf, leaf_size=16, theta=0.4)
    perm, lb, le, row, col = L.leaflist_host(X, 16, 0.4)
    ref = np.zeros((n, 3))
    for l in range(len(lb)):
        tg = perm[lb[l]:le[l]]
        src = np.concatenate([perm[lb[c]:le[c]] for c in col[row[l]:row[l + 1]]])
        ref[tg] = oracle.zeta_pairs(X[tg], X[src], G[src], s[src], 2)
    assert normwise(pf.particles[15:18, :n].T - 0.5, ref)[0] <= 1e-12
    other = [r for r in range(46) if r not in (15, 16, 17)]
    assert np.array_equal(pf.particles[other, :], Q[other, :])


def test_reused_lists_give_the_same_sums(ctx):
    """VPM_REUSE_LISTS: a call that reuses the lists of the previous call on the
    same positions gives the same bits as one that builds them; a call on other
    positions (another array) builds its own."""
    n = 6000
    X, G, s = random_cloud(n, seed=88, box=0.5)
    x, g, sg = _dev(X), _dev(G), _dev(s)
    out = []
    for reuse in (False, True):
        U, J, S = _zeros(n, 3), _zeros(n, 9), _zeros(n, 3)
        st = ctx.p2p_leaflist_dev(x, g, sg, U, J, S, leaf_size=32, theta=0.4, kernel=2, precision=1, sfs=True,
                                  reuse=reuse)
        out.append((st, U.cpu().numpy(), J.cpu().numpy(), S.cpu().numpy()))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)
    dJ, dS = _zeros(n, 9), _zeros(n, 3)
    dJ2, dS2 = _zeros(n, 9), _zeros(n, 3)
    Jd = _dev(out[0][2])
    ctx.dynamic_diff_leaflist_dev(x, g, sg, Jd, 0.999, dJ, dS, leaf_size=32, theta=0.4, reuse=True)
    ctx.dynamic_diff_leaflist_dev(x, g, sg, Jd, 0.999, dJ2, dS2, leaf_size=32, theta=0.4, reuse=False)
    assert torch_equal(dJ, dJ2) and torch_equal(dS, dS2)
    Y = random_cloud(n, seed=89, box=0.5)[0]
    W1, W2 = _zeros(n, 3), _zeros(n, 3)
    st_y = ctx.zeta_leaflist_dev(_dev(Y), g, sg, W1, leaf_size=32, theta=0.4, kernel=2, reuse=True)
    ctx.zeta_leaflist_dev(_dev(Y), g, sg, W2, leaf_size=32, theta=0.4, kernel=2)
    assert torch_equal(W1, W2) and st_y[1] > 0
