"""The oracle against the reference's own known answers (CPU only).

* scripts/check_fmm.jl:39-71 -- closed-form singular velocity and gradient of a
  particle pair (fixture kat_check_fmm.npz);
* src/FLOWVPM_kernel.jl -- each kernel's zeta(rho) = g'(rho) / (4 pi rho^2) and
  dg = g' (the consistency the kernel definitions rely on);
* src/FLOWVPM_gpu_erf.jl -- custom_erf64 against libm erf;
* test/runtests_singlevortexring.jl:124-149 -- the ring self-induced velocity
  within 2% of the analytic Uring (test_oracle_ring_velocity);
* the committed regression fixtures (uj_cloud64.npz, ring_rk3.npz).
"""
import math
import os

import numpy as np
import pytest

import oracle
from helpers import normwise

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _kat_matrix(kat):
    P = np.zeros((46, 2), order="F")
    P[0:3] = kat["X"].T
    P[3:6] = kat["Gamma"].T
    P[6] = kat["sigma"]
    return P


def test_singular_pair_matches_check_fmm_analytic():
    kat = np.load(os.path.join(GOLD, "kat_check_fmm.npz"))
    P = _kat_matrix(kat)
    oracle.uj_direct(P, 2, oracle.KERNEL_SINGULAR, oracle.RESET)
    for i in range(2):
        U = P[9:12, i]
        J = P[15:24, i].reshape(3, 3, order="F")
        assert np.abs(U - kat["U"][i]).max() <= 1e-14 * np.abs(kat["U"][i]).max()
        assert np.abs(J - kat["J"][i]).max() <= 1e-14 * np.abs(kat["J"][i]).max()


def test_gaussianerf_pair_approaches_singular_far_out():
    # rho = 6.7 in this pair: erf kernel differs from singular by ~1e-9 (g = 1 - O(e^-22))
    kat = np.load(os.path.join(GOLD, "kat_check_fmm.npz"))
    P = _kat_matrix(kat)
    oracle.uj_direct(P, 2, oracle.KERNEL_GAUSSIANERF, oracle.RESET)
    for i in range(2):
        assert np.abs(P[9:12, i] - kat["U"][i]).max() <= 1e-8 * np.abs(kat["U"][i]).max()


@pytest.mark.parametrize("x", [0.0, 1e-8, 0.1, 0.5, 0.84, 0.9, 1.2, 1.3, 2.0, 2.8, 3.0, 5.9, 6.1, -0.7, -2.2])
def test_custom_erf64_matches_libm(x):
    assert abs(oracle.erf_ref(x) - math.erf(x)) <= 4e-16


@pytest.mark.parametrize("k", [oracle.KERNEL_GAUSSIAN, oracle.KERNEL_GAUSSIANERF, oracle.KERNEL_WINCKELMANS])
def test_kernel_zeta_is_dg_over_4pi_rho2_and_dg_is_derivative(k):
    for rho in (0.05, 0.3, 1.0, 1.7, 3.0):
        g, dg = oracle.g_dgdr(k, rho)
        assert abs(oracle.zeta(k, rho) - dg / (4 * math.pi * rho * rho)) <= 1e-14 * max(1e-300, oracle.zeta(k, rho))
        h = 1e-5 * rho
        fd = (oracle.g_dgdr(k, rho + h)[0] - oracle.g_dgdr(k, rho - h)[0]) / (2 * h)
        assert abs(fd - dg) <= 1e-7 * abs(dg) + 1e-10  # FD of g ~ 1 has ~eps/h absolute noise


def test_uj_direct_reproduces_cloud_fixture():
    d = np.load(os.path.join(GOLD, "uj_cloud64.npz"))
    for k in range(4):
        P = np.asfortranarray(d["P0"].copy())
        oracle.uj_direct(P, 64, k, int(d["flags"]))
        assert np.abs(P - d[f"P_k{k}"]).max() <= 1e-13 * max(1.0, np.abs(d[f"P_k{k}"]).max())


def test_uj_direct_semantics_resets_statics_and_sfs():
    d = np.load(os.path.join(GOLD, "uj_cloud64.npz"))
    P0 = d["P0"]
    P = d["P_k2"]
    static = P0[42] != 0
    # rows the reference never touches are unchanged
    for rows in (slice(0, 9), slice(27, 39), slice(42, 46)):
        assert np.array_equal(P[rows], P0[rows])
    # reset: non-static vorticity and PSE rows are zeroed; static rows keep old values
    assert np.all(P[12:15, ~static] == 0) and np.all(P[24:27, ~static] == 0)
    assert np.array_equal(P[12:15, static], P0[12:15, static])
    # static targets: U, J accumulate on top of their old values, SFS untouched
    assert np.array_equal(P[39:42, static], P0[39:42, static])
    Q = np.asfortranarray(P0.copy())
    oracle.uj_direct(Q, 64, 2, oracle.RESET)
    assert np.allclose(P[9:24, static], Q[9:24, static])


def test_estr_factored_and_pairwise_agree_with_direct_loop():
    # Estr (transposed) restated literally vs the oracle C loop on a tiny case
    rng = np.random.default_rng(3)
    n = 9
    X = rng.uniform(0, 0.1, (n, 3))
    G = rng.normal(0, 1, (n, 3))
    s = rng.uniform(0.02, 0.04, n)
    J = rng.normal(0, 1, (n, 9))
    st = np.zeros(n, np.uint8)
    st[4] = 1
    S = oracle.estr_pairs(X, J, X, G, s, J, oracle.KERNEL_GAUSSIANERF, True, st, st)
    ref = np.zeros((n, 3))
    for t in range(n):
        if st[t]:
            continue
        for q in range(n):
            if st[q]:
                continue
            r = np.linalg.norm(X[q] - X[t])
            z = oracle.zeta(oracle.KERNEL_GAUSSIANERF, r / s[q]) / s[q] ** 3
            D = (J[t] - J[q]).reshape(3, 3, order="F")   # D[i,j] = d u_i/d x_j difference
            ref[t] += z * (D.T @ G[q])
    assert normwise(S, ref)[0] <= 1e-14


def test_oracle_reproduces_ring_rk3_fixture():
    d = np.load(os.path.join(GOLD, "ring_rk3.npz"))
    P = np.asfortranarray(d["P0"].copy())
    n = P.shape[1]
    prm = oracle.StepParams(kernel=oracle.KERNEL_GAUSSIANERF, transposed=1, f=0.0, g=0.2,
                            relaxation=1, rlxf=0.3)
    for step in range(3):
        assert oracle.rk3_step(P, n, float(d["dt"]), prm, relax=True) == 0
        assert np.abs(P - d["P"][step]).max() <= 1e-12 * max(1.0, np.abs(d["P"][step]).max())


def test_oracle_ring_velocity_matches_reference_test():
    """test/runtests_singlevortexring.jl case "Runge-Kutta time-integration +
    direct UJ": R=1, Nphi=100, nc=0, sigma=0.15R, faux=0.25, Winckelmans,
    cVPM, Pedrizzetti every step, 50 steps over Rtot=2 radii; |err| < 2%."""
    import vpm_gb300.rings as rings
    from vpm_gb300.particlefield import ParticleField, cVPM, winckelmans
    R, Nphi, nc = 1.0, 100, 0
    Rcross = 0.15 * R
    pf = ParticleField(rings.number_particles(Nphi, nc), formulation=cVPM, kernel=winckelmans,
                       UJ=lambda *a, **k: None)
    rings.addvortexring(pf, 1.0, R, 1.0, 0.25 * Rcross, Nphi, nc, Rcross)
    nsteps, Rtot, beta = 50, 2.0, 0.5
    Uref = rings.Uring(1.0, R, Rcross, beta)
    dt = (Rtot / Uref) / nsteps
    P = pf.particles
    n = pf.np
    Z0 = np.zeros(3)  # the ring's placement O, as in the reference test
    prm = oracle.StepParams(kernel=oracle.KERNEL_WINCKELMANS, transposed=1, f=0.0, g=0.0,
                            relaxation=1, rlxf=0.3)
    for i in range(1, nsteps + 1):
        assert oracle.rk3_step(P, n, dt, prm, relax=True) == 0
    Z = rings.calc_rings_weighted(pf, [0, n])[0][0]
    U_vpm = np.linalg.norm(Z - Z0) / (nsteps * dt)
    err = (U_vpm - Uref) / Uref
    assert abs(err) < 0.02, err
