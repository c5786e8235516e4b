"""The oracle against the mathematics (CPU only).

The reference's own tests pin UJ values only at the singular-pair closed form
and at 2-5 % physics tolerances.  Here the reference's formulas are evaluated
in 40-digit arithmetic (mpmath, exact erf and exp) and the oracle's FP64
restatement must agree to 1e-14 normwise (max |err| / max |truth| per
quantity), on small clouds whose pairs span rho = r/sigma from the kernels'
cores (rho ~ 0.3) to their singular tails (rho ~ 10):

* U and J, all four kernels: the pair loop of src/FLOWVPM_fmm.jl:102-168 with
  g, dg/drho of src/FLOWVPM_kernel.jl:45-84 and the constants of
  src/FLOWVPM.jl:62-66;
* Estr: src/FLOWVPM_subfilterscale_models.jl:16-41 (both schemes), zeta of
  src/FLOWVPM_kernel.jl;
* the UJ adjoint (oracle_uj_adjoint): against 40-digit central differences of
  the same 40-digit forward sum (step 1e-15, truncation error ~1e-30).

The cloud keeps rho >= 0.3 for every pair: below that, the reference's FP64
g(rho) = erf(rho/sqrt2) - sqrt(2/pi) rho e^{-rho^2/2} (and Gaussian's
1 - e^{-rho^3}) lose digits to cancellation by design, which is the
reference's behaviour, not the oracle's error; that regime is covered against
the GPU in FP64 by the other parity tests.
"""
import numpy as np
import pytest

import oracle
from helpers import normwise

mpmath = pytest.importorskip("mpmath")
mp = mpmath.mp

KERNELS = (oracle.KERNEL_SINGULAR, oracle.KERNEL_GAUSSIAN, oracle.KERNEL_GAUSSIANERF, oracle.KERNEL_WINCKELMANS)


def _consts():
    pi = mp.pi
    return {"c1": 1 / (2 * pi) ** mp.mpf(1.5), "c2": mp.sqrt(2 / pi), "c3": 3 / (4 * pi), "c4": 1 / (4 * pi)}


def g_dg(k, rho, C):
    """(g, dg/drho) of src/FLOWVPM_kernel.jl:45-84, exactly."""
    if k == oracle.KERNEL_SINGULAR:
        return mp.mpf(1), mp.mpf(0)
    if k == oracle.KERNEL_GAUSSIAN:
        e = mp.exp(-rho ** 3)
        return 1 - e, 3 * rho * rho * e
    if k == oracle.KERNEL_GAUSSIANERF:
        aux = C["c2"] * rho * mp.exp(-rho * rho / 2)
        return mp.erf(rho / mp.sqrt(2)) - aux, rho * aux
    q = rho * rho + 1
    return rho ** 3 * (rho * rho + mp.mpf(2.5)) / q ** mp.mpf(2.5), mp.mpf(7.5) * rho * rho / q ** mp.mpf(3.5)


def zeta(k, rho, C):
    if k == oracle.KERNEL_SINGULAR:
        return mp.mpf(1) if rho == 0 else mp.mpf(0)
    if k == oracle.KERNEL_GAUSSIAN:
        return C["c3"] * mp.exp(-rho ** 3)
    if k == oracle.KERNEL_GAUSSIANERF:
        return C["c1"] * mp.exp(-rho * rho / 2)
    return C["c4"] * mp.mpf(7.5) / (rho * rho + 1) ** mp.mpf(3.5)


def uj_exact(k, X, G, S, C):
    """U[n,3], J[n,9] (J[3*b + a] = du_a/dx_b) of the pair loop, src/FLOWVPM_fmm.jl:112-160."""
    n = len(X)
    U = [[mp.mpf(0)] * 3 for _ in range(n)]
    J = [[mp.mpf(0)] * 9 for _ in range(n)]
    for t in range(n):
        for s in range(n):
            dx = [X[t][i] - X[s][i] for i in range(3)]
            r2 = dx[0] ** 2 + dx[1] ** 2 + dx[2] ** 2
            if r2 == 0:
                continue
            r = mp.sqrt(r2)
            g, dg = g_dg(k, r / S[s], C)
            gx, gy, gz = G[s]
            r3inv = 1 / (r2 * r)
            crss = [-C["c4"] * r3inv * (dx[1] * gz - dx[2] * gy), -C["c4"] * r3inv * (dx[2] * gx - dx[0] * gz),
                    -C["c4"] * r3inv * (dx[0] * gy - dx[1] * gx)]
            for a in range(3):
                U[t][a] += g * crss[a]
            aux = dg / (S[s] * r) - 3 * g / r2
            aux2 = -C["c4"] * g * r3inv
            # Kronecker term: eps_{a b l} Gamma_l with the reference's signs
            kron = [[0, -gz, gy], [gz, 0, -gx], [-gy, gx, 0]]   # kron[b][a]: d u_a / d x_b term
            for b in range(3):
                for a in range(3):
                    J[t][3 * b + a] += aux * crss[a] * dx[b] + aux2 * kron[b][a]
    return U, J


def _cloud(n, seed, box=0.05, rho_min=0.3):
    """Seeded cloud with every pair at rho >= rho_min (redrawn until it holds)."""
    rng = np.random.default_rng(seed)
    while True:
        X = rng.uniform(0, box, (n, 3))
        s = rng.uniform(0.004, 0.012, n)
        G = rng.normal(0, 1e-3, (n, 3))
        d = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
        rho = d / s[None, :]
        np.fill_diagonal(rho, np.inf)
        if rho.min() >= rho_min:
            return X, G, s


def _mp(a):
    return [[mp.mpf(float(v)) for v in row] for row in a]


@pytest.mark.parametrize("k", KERNELS)
def test_oracle_uj_matches_40_digit_evaluation(k):
    mp.dps = 40
    C = _consts()
    X, G, s = _cloud(24, seed=100 + k)
    rho = np.sqrt(((X[:, None] - X[None]) ** 2).sum(-1)) / s[None, :]
    np.fill_diagonal(rho, np.nan)
    assert np.nanmin(rho) < 1.0 and np.nanmax(rho) > 8.0   # both the core and the tail are exercised
    Ue, Je = uj_exact(k, _mp(X), _mp(G), [mp.mpf(float(v)) for v in s], C)
    Ut = np.array([[float(v) for v in row] for row in Ue])
    Jt = np.array([[float(v) for v in row] for row in Je])
    Uo, Jo = oracle.uj_pairs(X, X, G, s, k)
    assert normwise(Uo, Ut)[0] <= 1e-14
    assert normwise(Jo, Jt)[0] <= 1e-14


@pytest.mark.parametrize("transposed", [True, False])
@pytest.mark.parametrize("k", KERNELS[1:])
def test_oracle_estr_matches_40_digit_evaluation(k, transposed):
    """SFS_t = sum_s zeta(r/sigma_s)/sigma_s^3 (J_t - J_s)^T Gamma_s (or (J_t - J_s) Gamma_s),
    src/FLOWVPM_subfilterscale_models.jl:16-41; static sources contribute nothing."""
    mp.dps = 40
    C = _consts()
    n = 20
    X, G, s = _cloud(n, seed=200 + k)
    rng = np.random.default_rng(7)
    Jv = rng.normal(0, 1.0, (n, 9))
    static = (np.arange(n) % 7 == 3).astype(np.uint8)
    Xm, Gm, Jm = _mp(X), _mp(G), _mp(Jv)
    Se = np.zeros((n, 3))
    for t in range(n):
        acc = [mp.mpf(0)] * 3
        for q in range(n):
            if q == t or static[q]:
                continue
            r = mp.sqrt(sum((Xm[t][i] - Xm[q][i]) ** 2 for i in range(3)))
            sg = mp.mpf(float(s[q]))
            z = zeta(k, r / sg, C) / sg ** 3
            for a in range(3):
                # (J_t - J_s)^T Gamma: sum_i M[i, a] Gamma_i ; M[i, a] = J[3a + i]
                if transposed:
                    acc[a] += z * sum((Jm[t][3 * a + i] - Jm[q][3 * a + i]) * Gm[q][i] for i in range(3))
                else:
                    acc[a] += z * sum((Jm[t][3 * i + a] - Jm[q][3 * i + a]) * Gm[q][i] for i in range(3))
        Se[t] = [float(v) for v in acc]
    So = oracle.estr_pairs(X, Jv, X, G, s, Jv, k, transposed, None, static)
    assert normwise(So, Se)[0] <= 1e-14


@pytest.mark.parametrize("k", [oracle.KERNEL_GAUSSIANERF, oracle.KERNEL_WINCKELMANS])
def test_oracle_uj_adjoint_matches_40_digit_differences(k):
    """d/d(x, Gamma, sigma) of phi = sum Ubar.U + Jbar:J by 40-digit central differences of the
    40-digit forward (h = 1e-15: truncation ~h^2, rounding ~1e-25), against oracle_uj_adjoint."""
    mp.dps = 40
    C = _consts()
    n = 6
    X, G, s = _cloud(n, seed=300 + k, box=0.03)
    rng = np.random.default_rng(9)
    Ub, Jb = rng.normal(size=(n, 3)), rng.normal(size=(n, 9))

    def phi(Xm, Gm, Sm):
        U, J = uj_exact(k, Xm, Gm, Sm, C)
        return sum(U[t][a] * float(Ub[t, a]) for t in range(n) for a in range(3)) + \
            sum(J[t][c] * float(Jb[t, c]) for t in range(n) for c in range(9))

    h = mp.mpf("1e-15")
    Xm, Gm, Sm = _mp(X), _mp(G), [mp.mpf(float(v)) for v in s]
    xb = np.zeros((n, 3)); gb = np.zeros((n, 3)); sb = np.zeros(n)
    for p in range(n):
        for c in range(3):
            for arr, out in ((Xm, xb), (Gm, gb)):
                v = arr[p][c]
                arr[p][c] = v + h; fp = phi(Xm, Gm, Sm)
                arr[p][c] = v - h; fm = phi(Xm, Gm, Sm)
                arr[p][c] = v
                out[p, c] = float((fp - fm) / (2 * h))
        v = Sm[p]
        Sm[p] = v + h; fp = phi(Xm, Gm, Sm)
        Sm[p] = v - h; fm = phi(Xm, Gm, Sm)
        Sm[p] = v
        sb[p] = float((fp - fm) / (2 * h))
    xo, go, so = oracle.uj_adjoint(X, G, s, Ub, Jb, k)
    assert normwise(xo, xb)[0] <= 1e-13
    assert normwise(go, gb)[0] <= 1e-13
    assert normwise(so, sb)[0] <= 1e-13
