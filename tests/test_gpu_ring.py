"""Ring workloads through the drop-in hook: a ParticleField built with
UJ=UJ_gb300 / UJ_gb300_mixed runs the mirrored rVPM RK3 unchanged.

* the reference's own ring test (test/runtests_singlevortexring.jl:124-149):
  ring speed within 2% of the analytic Uring;
* the isolated-ring workload (R=1, Gamma=1, a=0.1, Nphi=200 x 7 per section =
  1400 particles, sigma=a/2, Gaussian-erf, rVPM, Pedrizzetti relaxation every
  step, 10 RK3 steps of dt=0.01): U, J and X after every step against the
  oracle's step (oracle/vpm_oracle.c: oracle_rk3_step);
* the committed ring_rk3 fixture.
"""
import os

import numpy as np
import pytest

import oracle
import vpm_gb300 as vpm
import vpm_gb300.rings as rings
from helpers import normwise

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("UJ", ["fp64", "mixed"])
@pytest.mark.parametrize("nc,formulation", [(0, "cVPM"), (1, "rVPM")])
def test_reference_ring_velocity(UJ, nc, formulation):
    R, Nphi = 1.0, 100
    Rcross = 0.15 * R
    form = vpm.cVPM if formulation == "cVPM" else vpm.rVPM
    pf = vpm.ParticleField(rings.number_particles(Nphi, nc), formulation=form, kernel=vpm.winckelmans,
                           UJ=vpm.UJ_gb300 if UJ == "fp64" else vpm.UJ_gb300_mixed,
                           relaxation=vpm.pedrizzetti)
    rings.addvortexring(pf, 1.0, R, 1.0, 0.25 * Rcross, Nphi, nc, Rcross)
    nsteps, Rtot, beta = 50, 2.0, 0.5
    Uref = rings.Uring(1.0, R, Rcross, beta)
    dt = (Rtot / Uref) / nsteps
    vpm.run_vpm(pf, dt, nsteps)
    Z = rings.calc_rings_weighted(pf, [0, pf.np])[0][0]
    err = (np.linalg.norm(Z) / pf.t - Uref) / Uref
    assert abs(err) < 0.02, err


def _ring1400():
    X, G, s, vol = rings.ring_sections(1.0, 1.0, 0.1, 200, 7, 0.05)
    return X, G, s, vol


@pytest.mark.parametrize("UJ,tol", [("fp64", 1e-11), ("mixed", 2e-5)])
def test_isolated_ring_steps_match_oracle(UJ, tol):
    X, G, s, vol = _ring1400()
    pf = vpm.ParticleField(X.shape[0], kernel=vpm.gaussianerf, relaxation=vpm.pedrizzetti,
                           UJ=vpm.UJ_gb300 if UJ == "fp64" else vpm.UJ_gb300_mixed)
    pf.add_particles(X, G, s, vol=vol)
    n = pf.np
    P = np.asfortranarray(pf.particles.copy())
    prm = oracle.StepParams(kernel=oracle.KERNEL_GAUSSIANERF, transposed=1, f=0.0, g=0.2, relaxation=1,
                            rlxf=0.3)
    worst = {}
    for step in range(10):
        pf.nextstep(0.01, relax=True)
        assert oracle.rk3_step(P, n, 0.01, prm, relax=True) == 0
        for name, rows in (("X", slice(0, 3)), ("Gamma", slice(3, 6)), ("U", slice(9, 12)),
                           ("J", slice(15, 24))):
            e = normwise(pf.particles[rows, :n], P[rows, :n])[0]
            worst[name] = max(worst.get(name, 0.0), e)
            assert e <= tol, (step, name, e)


@pytest.mark.parametrize("UJ,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_golden_ring_fixture(UJ, tol):
    d = np.load(os.path.join(GOLD, "ring_rk3.npz"))
    n = d["P0"].shape[1]
    pf = vpm.ParticleField(n, kernel=vpm.gaussianerf, relaxation=vpm.pedrizzetti,
                           UJ=vpm.UJ_gb300 if UJ == "fp64" else vpm.UJ_gb300_mixed)
    pf.particles[:, :] = d["P0"]
    pf.np = n
    for step in range(3):
        pf.nextstep(float(d["dt"]), relax=True)
        for rows in (slice(0, 3), slice(3, 6), slice(9, 12), slice(15, 24)):
            assert normwise(pf.particles[rows], d["P"][step][rows])[0] <= tol


def test_dynamic_sfs_ring_matches_oracle():
    """Dynamic SFS + core spreading (the leapfrog workload's scheme) on a small
    two-ring field: FP64 GPU steps against the oracle's."""
    X1, G1, s1, v1 = rings.ring_sections(1.0, 1.0, 0.1, 40, 10, 0.05)
    X2, G2, s2, v2 = rings.ring_sections(1.0, 0.7, 0.07, 28, 10, 0.035, O=(0, 0, 0.3))
    X = np.vstack([X1, X2]); G = np.vstack([G1, G2]); s = np.concatenate([s1, s2])
    pf = vpm.ParticleField(X.shape[0], kernel=vpm.gaussianerf, UJ=vpm.UJ_gb300,
                           SFS=vpm.SFS_Cd_twolevel_nobackscatter, viscous=vpm.CoreSpreading(1e-4, 0.05),
                           relaxation=vpm.norelaxation)
    pf.add_particles(X, G, s)
    n = pf.np
    P = np.asfortranarray(pf.particles.copy())
    sfs = pf.SFS
    prm = oracle.StepParams(kernel=oracle.KERNEL_GAUSSIANERF, transposed=1, f=0.0, g=0.2, relaxation=0,
                            sfs=2, alpha=sfs.alpha, sfs_rlxf=sfs.rlxf, minC=sfs.minC, maxC=sfs.maxC,
                            force_positive=1, clip_backscatter=1, viscous=1, nu=1e-4, sgm0=0.05, beta=1.5)
    for step in range(3):
        pf.nextstep(0.005)
        assert oracle.rk3_step(P, n, 0.005, prm, relax=False) == 0
        for rows in (slice(0, 3), slice(3, 6), slice(6, 7), slice(9, 12), slice(15, 24), slice(36, 37),
                     slice(39, 42)):
            assert normwise(pf.particles[rows, :n], P[rows, :n])[0] <= 1e-10, (step, rows)
