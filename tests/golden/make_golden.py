"""Generate the committed golden fixtures of tests/golden/.

    python tests/golden/make_golden.py

Fixtures:
  kat_check_fmm.npz  Two particles (the `bodies` table of the reference's
                     scripts/check_fmm.jl:94-102: rows x(1:3), sigma(4), Gamma(5:7))
                     with U and J from the closed-form singular Biot-Savart
                     velocity and gradient of that script (:39-71).  Independent
                     of any code in this repository.
  uj_cloud64.npz     64-particle random cloud (5 static) in the reference matrix
                     layout, run through the oracle's UJ_direct with reset,
                     reset_sfs, sfs and the transposed scheme, for each of the
                     four kernels.  Regression fixture for the oracle and the GPU.
  ring_rk3.npz       A 7-per-section ring of 140 particles after 3 rVPM RK3 steps
                     with Pedrizzetti relaxation (oracle), for the time-step parity.

The reference itself (Julia + FastMultipole.jl) cannot run in this build
environment, so uj_cloud64 and ring_rk3 are produced by the oracle
(oracle/vpm_oracle.c); kat_check_fmm pins the oracle to the reference's own
analytic check.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "flowvpm.jl_gb300"))

import oracle  # noqa: E402

BODIES = np.array([[0.4, 0.1], [0.1, -0.5], [-0.3, 0.2], [1 / 8, 1 / 8], [0.3, -0.4], [-0.1, -0.2],
                   [0.08, 0.5]])


def u_analytic(t, s, g):
    """Singular Biot-Savart velocity, scripts/check_fmm.jl:39-47."""
    d = t - s
    n = np.sqrt(d @ d)
    return 1 / 4 / np.pi / n ** 3 * np.array([-d[1] * g[2] + d[2] * g[1], -d[2] * g[0] + d[0] * g[2],
                                              -d[0] * g[1] + d[1] * g[0]])


def duidxj_analytic(t, s, g):
    """Its gradient J[i,j] = du_i/dx_j, scripts/check_fmm.jl:57-71."""
    x, y, z = t - s
    gx, gy, gz = g
    n = np.sqrt(x * x + y * y + z * z)
    xy, yz, xz = x * y, y * z, x * z
    M = np.array([
        [3 * xy * gz - 3 * xz * gy, (2 * y * y - x * x - z * z) * gz - 3 * yz * gy, 3 * yz * gz - (2 * z * z - x * x - y * y) * gy],
        [3 * xz * gx - (2 * x * x - y * y - z * z) * gz, 3 * yz * gx - 3 * xy * gz, (2 * z * z - x * x - y * y) * gx - 3 * xz * gz],
        [(2 * x * x - y * y - z * z) * gy - 3 * xy * gx, 3 * xy * gy - (2 * y * y - x * x - z * z) * gx, 3 * xz * gy - 3 * yz * gx]]) / n ** 5
    return M / 4 / np.pi


def make_kat():
    X = BODIES[0:3].T.copy()
    s = BODIES[3].copy()
    G = BODIES[4:7].T.copy()
    U = np.zeros((2, 3))
    J = np.zeros((2, 3, 3))
    for i in range(2):
        j = 1 - i
        U[i] = u_analytic(X[i], X[j], G[j])
        J[i] = duidxj_analytic(X[i], X[j], G[j])
    np.savez(os.path.join(HERE, "kat_check_fmm.npz"), X=X, sigma=s, Gamma=G, U=U, J=J)


def make_cloud():
    rng = np.random.default_rng(20240601)
    n = 64
    P0 = np.asfortranarray(rng.normal(size=(46, n)))
    P0[0:3] = rng.uniform(0, 0.3, size=(3, n))
    P0[3:6] = rng.normal(0, 1e-3, size=(3, n))
    P0[6] = rng.uniform(0.01, 0.03, size=n)
    P0[42] = 0.0
    P0[42, [3, 17, 30, 41, 63]] = 1.0
    P0[0:3, 10] = P0[0:3, 11]          # a coincident pair (r == 0 but distinct)
    out = {"P0": P0}
    flags = oracle.RESET | oracle.RESET_SFS | oracle.SFS | oracle.TRANSPOSED
    for k in range(4):
        P = P0.copy(order="F")
        oracle.uj_direct(P, n, k, flags)
        out[f"P_k{k}"] = P
    out["flags"] = np.array(flags)
    np.savez(os.path.join(HERE, "uj_cloud64.npz"), **out)


def make_ring():
    import vpm_gb300.rings as rings
    X, G, s, vol = rings.ring_sections(1.0, 1.0, 0.1, 20, 7, 0.05)
    n = X.shape[0]
    P = np.zeros((46, n), order="F")
    P[0:3] = X.T
    P[3:6] = G.T
    P[6] = s
    P[7] = vol
    P0 = P.copy(order="F")
    prm = oracle.StepParams(kernel=oracle.KERNEL_GAUSSIANERF, transposed=1, f=0.0, g=0.2,
                            relaxation=1, rlxf=0.3, sfs=0, viscous=0, erf_mode=0, nthreads=0)
    steps = []
    for _ in range(3):
        rc = oracle.rk3_step(P, n, 0.01, prm, relax=True)
        assert rc == 0
        steps.append(P.copy(order="F"))
    np.savez(os.path.join(HERE, "ring_rk3.npz"), P0=P0, P=np.stack(steps), dt=0.01)


if __name__ == "__main__":
    make_kat()
    make_cloud()
    make_ring()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)), "B")
