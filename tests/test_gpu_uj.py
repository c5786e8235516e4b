"""GPU parity of the UJ and Estr kernels against the oracle, through the C ABI.

Tolerances (normwise: max|err| / max|ref| per quantity, over all targets):
  FP64 kernels      <= 1e-12 for U, J and SFS
  FP32-comp kernels <= 1e-6 for U and J; <= 2e-6 for SFS computed from the
  FP32-comp J (the J error propagates: SFS sums differences of J), <= 3e-6 for
  SFS from an exact J on a smooth field (limited by the FP32 sums of the
  factored form, which cancel)
"""
import os

import numpy as np
import pytest

import oracle
from helpers import matrix_of, normwise, random_cloud

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FP64, FP32COMP = 0, 1
TOL_UJ = {FP64: 1e-12, FP32COMP: 1e-6}
TOL_SFS = {FP64: 1e-12, FP32COMP: 2e-6}
ALL_FLAGS = oracle.RESET | oracle.RESET_SFS | oracle.SFS | oracle.TRANSPOSED


def _compare_matrix(P, Q, n, prec, what=""):
    """P: GPU result, Q: oracle result (both 46 x >=n)."""
    untouched = list(range(0, 9)) + list(range(27, 39)) + list(range(42, 46))
    assert np.array_equal(P[untouched, :n], Q[untouched, :n]), f"{what}: untouched rows changed"
    assert np.array_equal(P[:, n:], Q[:, n:]), f"{what}: columns beyond np changed"
    for rows, tol, name in ((slice(9, 12), TOL_UJ[prec], "U"), (slice(15, 24), TOL_UJ[prec], "J"),
                            (slice(12, 15), 0.0, "omega"), (slice(24, 27), 0.0, "PSE"),
                            (slice(39, 42), TOL_SFS[prec], "SFS")):
        e = normwise(P[rows, :n], Q[rows, :n])[0]
        assert e <= tol, f"{what}: {name} normwise error {e:.3e} > {tol:.0e}"


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
@pytest.mark.parametrize("k", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [1, 2, 3, 33, 129, 1000, 2500])
def test_uj_matrix_parity(ctx, k, prec, n):
    X, G, s = random_cloud(n, seed=1000 + n, box=0.2)
    static = (np.arange(n) % 7) == 3
    P = matrix_of(X, G, s, static, extra=3, seed=n)
    Q = P.copy(order="F")
    oracle.uj_direct(Q, n, k, ALL_FLAGS)
    ctx.uj(P, n, k, prec, ALL_FLAGS)
    _compare_matrix(P, Q, n, prec, f"k={k} prec={prec} n={n}")


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
@pytest.mark.parametrize("flags", [0, oracle.RESET, oracle.RESET_SFS | oracle.SFS,
                                   oracle.RESET | oracle.SFS, oracle.RESET | oracle.RESET_SFS | oracle.SFS])
def test_uj_flag_semantics(ctx, flags, prec):
    n = 300
    X, G, s = random_cloud(n, seed=7, box=0.15)
    P = matrix_of(X, G, s, static=(np.arange(n) % 5 == 0), seed=11)
    Q = P.copy(order="F")
    oracle.uj_direct(Q, n, 2, flags)
    ctx.uj(P, n, 2, prec, flags)
    _compare_matrix(P, Q, n, prec, f"flags={flags}")


def test_zero_particles_is_a_no_op(ctx):
    P = np.zeros((46, 4), order="F")
    ctx.uj(P, 0, 2, FP64, ALL_FLAGS)
    assert not P.any()


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
def test_golden_cloud_fixture(ctx, prec):
    d = np.load(os.path.join(GOLD, "uj_cloud64.npz"))
    for k in range(4):
        P = np.asfortranarray(d["P0"].copy())
        ctx.uj(P, 64, k, prec, int(d["flags"]))
        _compare_matrix(P, d[f"P_k{k}"], 64, prec, f"golden k={k}")


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
def test_golden_check_fmm_kat(ctx, prec):
    kat = np.load(os.path.join(GOLD, "kat_check_fmm.npz"))
    P = np.zeros((46, 2), order="F")
    P[0:3] = kat["X"].T
    P[3:6] = kat["Gamma"].T
    P[6] = kat["sigma"]
    ctx.uj(P, 2, 0, prec, oracle.RESET)
    tol = 1e-14 if prec == FP64 else 1e-6
    for i in range(2):
        assert normwise(P[9:12, i], kat["U"][i])[0] <= tol
        assert normwise(P[15:24, i].reshape(3, 3, order="F"), kat["J"][i])[0] <= tol


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
@pytest.mark.parametrize("k", [2, 3])
def test_uj_dev_cross_parity(ctx, k, prec):
    import torch
    Xs, Gs, ss = random_cloud(700, seed=21, box=0.3)
    Xt, _, _ = random_cloud(333, seed=22, box=0.3)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    U = torch.zeros(333, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(333, 9, device="cuda", dtype=torch.float64)
    U += 1.0  # accumulate on top of existing values
    ctx.uj_dev(d(Xt), d(Xs), d(Gs), d(ss), U, J, k, prec)
    Ur, Jr = oracle.uj_pairs(Xt, Xs, Gs, ss, k)
    assert normwise(U.cpu().numpy() - 1.0, Ur)[0] <= TOL_UJ[prec]
    assert normwise(J.cpu().numpy(), Jr)[0] <= TOL_UJ[prec]


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
@pytest.mark.parametrize("transposed", [True, False])
def test_estr_dev_parity(ctx, prec, transposed):
    import torch
    n = 900
    X, G, s = random_cloud(n, seed=5, box=0.2)
    rng = np.random.default_rng(6)
    J = rng.normal(0, 1, (n, 9))
    st = (np.arange(n) % 9 == 0).astype(np.uint8)
    d = lambda a: torch.tensor(a, device="cuda").contiguous()
    SFS = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    ctx.estr_dev(d(X), d(J), d(X), d(G), d(s), d(J), SFS, 2, prec, transposed, d(st), d(st))
    ref = oracle.estr_pairs(X, J, X, G, s, J, 2, transposed, st, st)
    assert normwise(SFS.cpu().numpy(), ref)[0] <= TOL_SFS[prec]


@pytest.mark.parametrize("transposed", [True, False])
def test_mixed_estr_on_a_smooth_field(ctx, transposed):
    """On two coaxial rings J varies slowly from particle to particle, so each
    Estr term z (J_t - J_s)^T g is a difference of nearly equal J, and the sum
    over a target's neighbours cancels further.  With an exact J the FP32-comp
    Estr keeps 3e-6 there; the difference of SFS between the dynamic
    procedure's two filter widths (sigma and 0.999 sigma, each with its own J)
    -- a difference of nearly equal SFS -- keeps 5e-3."""
    import torch
    from vpm_gb300 import workloads
    X, G, s = workloads.leapfrog_rings(4000, nper=10)
    n = X.shape[0]
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    out = {}
    for alpha in (1.0, 0.999):
        sa = s * alpha
        _, J = oracle.uj_pairs(X, X, G, sa, 2)
        ref = oracle.estr_pairs(X, J, X, G, sa, J, 2, transposed)
        SFS = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
        ctx.estr_dev(d(X), d(J), d(X), d(G), d(sa), d(J), SFS, 2, FP32COMP, transposed)
        got = SFS.cpu().numpy()
        assert normwise(got, ref)[0] <= 3e-6, alpha
        out[alpha] = (got, ref)
    diff_got = out[0.999][0] - out[1.0][0]
    diff_ref = out[0.999][1] - out[1.0][1]
    assert normwise(diff_got, diff_ref)[0] <= 5e-3


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
def test_uj_cross_matrix(ctx, prec):
    Xs, Gs, ss = random_cloud(500, seed=31, box=0.2)
    Xt, Gt, st = random_cloud(200, seed=32, box=0.2)
    S = matrix_of(Xs, Gs, ss, seed=1)
    T = matrix_of(Xt, Gt, st, seed=2)
    T0 = T.copy(order="F")
    ctx.uj_cross(S, 500, T, 200, 2, prec)
    Ur, Jr = oracle.uj_pairs(Xt, Xs, Gs, ss, 2)
    assert normwise(T[9:12] - T0[9:12], Ur.T)[0] <= TOL_UJ[prec]
    assert normwise(T[15:24] - T0[15:24], Jr.T)[0] <= TOL_UJ[prec]
    assert np.array_equal(T[:9], T0[:9]) and np.array_equal(T[24:], T0[24:])


@pytest.mark.parametrize("n", [1 << 14])
@pytest.mark.parametrize("k", [2, 3])
def test_mixed_error_full_cloud(ctx, k, n):
    """The random-cloud workload at N=2^14: every target vs the oracle."""
    X, G, s = random_cloud(n, seed=0)
    P = matrix_of(X, G, s)
    ctx.uj(P, n, k, FP32COMP, oracle.RESET)
    Ur, Jr = oracle.uj_pairs(X, X, G, s, k)
    eU = normwise(P[9:12, :n].T, Ur)
    eJ = normwise(P[15:24, :n].T, Jr)
    assert eU[0] <= 1e-6 and eJ[0] <= 1e-6, (eU, eJ)


@pytest.mark.parametrize("n", [1 << 17, 1 << 20])
@pytest.mark.parametrize("k", [2, 3])
def test_large_cloud_subset_and_linearity(ctx, k, n):
    """Full-size random clouds: a seeded subset of targets vs the oracle over all
    sources, and U, J exactly linear in Gamma (doubling Gamma doubles every output bit-for-bit)."""
    import torch
    X, G, s = random_cloud(n, seed=1)
    d = lambda a: torch.tensor(a, device="cuda").contiguous()
    xt, gs, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    ctx.uj_dev(xt, xt, gs, sg, U, J, k, FP32COMP)
    U2 = torch.zeros_like(U)
    J2 = torch.zeros_like(J)
    ctx.uj_dev(xt, xt, 2 * gs, sg, U2, J2, k, FP32COMP)
    assert torch.equal(U2, 2 * U) and torch.equal(J2, 2 * J)
    rng = np.random.default_rng(2)
    sub = np.sort(rng.choice(n, 512, replace=False))
    Ur, Jr = oracle.uj_pairs(X[sub], X, G, s, k)
    Uh, Jh = U.cpu().numpy()[sub], J.cpu().numpy()[sub]
    assert normwise(Uh, Ur)[0] <= 1e-6 and normwise(Jh, Jr)[0] <= 1e-6


def test_argument_errors_leave_context_usable(ctx):
    import torch
    import vpm_gb300
    P = np.zeros((46, 4), order="F")
    with pytest.raises(vpm_gb300.VPMError) as ei:
        ctx.uj(P, 4, 7, FP64, 0)
    assert ei.value.code == vpm_gb300._lib.ERR_ARG and "kernel" in str(ei.value)
    with pytest.raises(vpm_gb300.VPMError):
        ctx.uj(P, 4, 2, 5, 0)
    # host pointers are rejected by the device-pointer API
    L = ctx._L
    h = np.zeros((4, 3))
    rc = L.vpm_uj_dev(ctx._h, 4, h.ctypes.data, 4, h.ctypes.data, h.ctypes.data, h.ctypes.data,
                      h.ctypes.data, h.ctypes.data, 2, 0)
    assert rc == vpm_gb300._lib.ERR_ARG
    X, G, s = random_cloud(10, seed=3)
    P = matrix_of(X, G, s)
    Q = P.copy(order="F")
    ctx.uj(P, 10, 2, FP64, oracle.RESET)
    oracle.uj_direct(Q, 10, 2, oracle.RESET)
    assert normwise(P[9:24], Q[9:24])[0] <= 1e-12


def test_nonfinite_outputs_are_reported(ctx):
    import vpm_gb300
    X, G, s = random_cloud(50, seed=4)
    G[7] = np.nan
    P = matrix_of(X, G, s)
    with pytest.raises(vpm_gb300.VPMError) as ei:
        ctx.uj(P, 50, 2, FP64, oracle.RESET | vpm_gb300._lib.CHECK_FINITE)
    assert ei.value.code == vpm_gb300._lib.ERR_NONFINITE


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_zeta_dev_parity(ctx, k, prec):
    """zeta_direct (src/FLOWVPM_viscous.jl:467-488), self pairs included."""
    import torch
    X, G, s = random_cloud(1500, seed=40 + k, box=0.3)
    X[7] = X[3]                              # a coincident pair
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    W = torch.zeros(X.shape[0], 3, device="cuda", dtype=torch.float64)
    x = d(X)
    ctx.zeta_dev(x, x, d(G), d(s), W, k, prec)
    ref = oracle.zeta_pairs(X, X, G, s, k)
    assert normwise(W.cpu().numpy(), ref)[0] <= TOL_UJ[prec]


@pytest.mark.parametrize("prec", [FP64, FP32COMP])
def test_zeta_matrix_writes_rows_16_18_of_every_particle(ctx, prec):
    n = 700
    X, G, s = random_cloud(n, seed=44, box=0.3)
    static = np.zeros(n, bool)
    static[::11] = True
    P = matrix_of(X, G, s, static=static, extra=5)
    P[15:18, :] = 7.0                        # overwritten, statics included
    Q = P.copy(order="F")
    ctx.zeta(P, n, 2, prec)
    ref = oracle.zeta_pairs(X, X, G, s, 2)
    assert normwise(P[15:18, :n].T, ref)[0] <= TOL_UJ[prec]
    other = [r for r in range(46) if r not in (15, 16, 17)]
    assert np.array_equal(P[other, :], Q[other, :])
    assert np.array_equal(P[:, n:], Q[:, n:])


@pytest.mark.parametrize("flags", [oracle.RESET | oracle.RESET_SFS | oracle.SFS | oracle.TRANSPOSED, 0])
def test_uj_matrix_staged_many_threads(ctx, flags):
    """vpm_uj stages X, Gamma, sigma and the static flag through compact pinned
    buffers and applies the sums on the host with UJ_direct's reset rules (over
    several host threads at this size); statics and pre-set rows included."""
    n = 40000
    X, G, s = random_cloud(n, seed=123, box=1.0)
    static = (np.arange(n) % 97) == 5
    P = matrix_of(X, G, s, static, extra=2, seed=5)
    Q = P.copy(order="F")
    oracle.uj_direct(Q, n, 2, flags)
    ctx.uj(P, n, 2, FP32COMP, flags)
    _compare_matrix(P, Q, n, FP32COMP, f"staged flags={flags}")
