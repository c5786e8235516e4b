"""The Python host mirror of the reference's time integration (vpm_gb300.timeintegration)
against the oracle's C restatement of the same step (CPU only).

The mirror is run with `UJ` = the oracle's UJ_direct, so the only difference
between the two sides is the host code around UJ: rungekutta3, relaxation, the
SFS schemes and core spreading must agree to rounding.
"""
import numpy as np
import pytest

import oracle
import vpm_gb300 as vpm
import vpm_gb300.rings as rings
import vpm_gb300.timeintegration as ti


def UJ_oracle(pfield, rbf=False, sfs=False, reset=True, reset_sfs=False, **kw):
    flags = (oracle.RESET if reset else 0) | (oracle.RESET_SFS if reset_sfs else 0) | \
            (oracle.SFS if sfs else 0) | (oracle.TRANSPOSED if pfield.transposed else 0)
    oracle.uj_direct(pfield.particles, pfield.np, pfield.kernel.kid, flags)


def _ring_field(kernel, nphi=16, nper=7, static=False, **kw):
    X, G, s, vol = rings.ring_sections(1.0, 1.0, 0.1, nphi, nper, 0.05)
    n = X.shape[0] + (1 if static else 0)
    pf = vpm.ParticleField(n + 2, kernel=kernel, UJ=UJ_oracle, **kw)
    pf.add_particles(X, G, s, vol=vol)
    if static:
        pf.add_particle([0.0, 0.0, 0.3], [0.0, 0.0, 0.0], 0.05, static=True)
    return pf


CASES = {
    "rvpm_pedrizzetti": dict(kernel=vpm.gaussianerf, relaxation=vpm.pedrizzetti),
    "cvpm_wnklmns_corrected": dict(kernel=vpm.winckelmans, formulation=vpm.cVPM,
                                   relaxation=vpm.correctedpedrizzetti),
    "dynamic_sfs_corespreading": dict(kernel=vpm.gaussianerf, SFS=vpm.SFS_Cd_twolevel_nobackscatter,
                                      viscous=vpm.CoreSpreading(1e-4, 0.05), static=True),
    "constant_sfs_classic": dict(kernel=vpm.gaussianerf, SFS=vpm.SFS_Cs_nobackscatter, transposed=False),
}


def _params(pf, case):
    f = pf.formulation.f
    g = pf.formulation.g
    rl = pf.relaxation
    sfs = pf.SFS
    prm = oracle.StepParams(kernel=pf.kernel.kid, transposed=int(pf.transposed), f=f, g=g,
                            relaxation=0 if rl is ti.relaxation_none else (2 if rl is ti.correctedpedrizzetti else 1),
                            rlxf=rl.rlxf)
    if isinstance(sfs, ti.DynamicSFS):
        prm.sfs, prm.alpha, prm.sfs_rlxf, prm.minC, prm.maxC = 2, sfs.alpha, sfs.rlxf, sfs.minC, sfs.maxC
        prm.force_positive = int(sfs.force_positive)
        prm.clip_backscatter = int(ti.clipping_backscatter in sfs.clippings)
    elif isinstance(sfs, ti.ConstantSFS):
        prm.sfs, prm.Cs = 1, sfs.Cs
        prm.clip_backscatter = int(ti.clipping_backscatter in sfs.clippings)
    if isinstance(pf.viscous, ti.CoreSpreading):
        prm.viscous, prm.nu, prm.sgm0, prm.beta = 1, pf.viscous.nu, pf.viscous.sgm0, pf.viscous.beta
    return prm


@pytest.mark.parametrize("case", sorted(CASES))
def test_mirror_rk3_matches_oracle_step(case):
    kw = dict(CASES[case])
    static = kw.pop("static", False)
    pf = _ring_field(static=static, **kw)
    P = np.asfortranarray(pf.particles.copy())
    prm = _params(pf, case)
    dt = 0.01
    for step in range(3):
        pf.nextstep(dt, relax=True)
        assert oracle.rk3_step(P, pf.np, dt, prm, relax=True) == 0
        n = pf.np
        diff = np.abs(pf.particles[:43, :n] - P[:43, :n]).max()
        assert diff <= 1e-12 * max(1.0, np.abs(P[:43, :n]).max()), (case, step, diff)


def test_dynamic_sfs_sets_coefficients_and_clips():
    pf = _ring_field(kernel=vpm.gaussianerf, SFS=vpm.SFS_Cd_twolevel_nobackscatter)
    pf.nextstep(0.01)
    C = pf.particles[36, :pf.np]
    assert np.all(np.isfinite(C)) and np.all(C >= 0) and np.all(C <= 1)
    G = pf.particles[3:6, :pf.np]
    S = pf.particles[39:42, :pf.np]
    assert np.all(C * (G * S).sum(axis=0) >= 0)   # backscatter clipped


def zeta_oracle(pfield):
    """zeta_direct through the oracle: rows 16:18 of every particle (statics included)."""
    n = pfield.np
    P = pfield.particles
    X = np.ascontiguousarray(P[0:3, :n].T)
    P[15:18, :n] = oracle.zeta_pairs(X, X, np.ascontiguousarray(P[3:6, :n].T), P[6, :n], pfield.kernel.kid).T


def test_corespreading_reset_rebuilds_strengths():
    """The core-size reset of src/FLOWVPM_viscous.jl:194-219: sigma returns to
    sgm0 on the non-static particles, the growth timer restarts, and the RBF
    conjugate gradient leaves strengths whose basis field matches the target
    vorticity to the CG tolerance; the static particle is left alone."""
    pf = _ring_field(kernel=vpm.gaussianerf, static=True, relaxation=vpm.norelaxation,
                     viscous=vpm.CoreSpreading(1e-3, 0.05, beta=1.0001, zeta=zeta_oracle))
    n = pf.np
    st_before = pf.particles[:, n - 1].copy()
    pf.nextstep(0.01)
    P = pf.particles
    assert pf.viscous.t_sgm == 0.0
    assert np.all(P[6, :n - 1] == 0.05)
    assert np.array_equal(P[0:7, n - 1], st_before[0:7])
    # the reference's stopping rule: |b - A x| <= tol |b - A x0| per component, x0 = b vol
    targ = P[33:36, :n - 1].T.copy()
    zeta_oracle(pf)
    W = P[15:18, :n - 1].T.copy()
    P[3:6, :n - 1] = (targ * P[7, :n - 1][:, None]).T
    zeta_oracle(pf)
    r0 = targ - P[15:18, :n - 1].T
    live = (targ ** 2).sum(0) > 1e-12 * (targ ** 2).sum()      # the ring's axial component is zero
    res = np.sqrt(((W - targ) ** 2).sum(0)[live] / (r0 ** 2).sum(0)[live])
    assert live.any() and (res <= 1e-3).all(), res


def test_corespreading_reset_reports_non_convergence():
    pf = _ring_field(kernel=vpm.gaussianerf, relaxation=vpm.norelaxation,
                     viscous=vpm.CoreSpreading(1e-3, 0.05, beta=1.0001, zeta=zeta_oracle, itmax=1, tol=1e-14))
    with pytest.raises(RuntimeError, match="Maximum number of iterations"):
        pf.nextstep(0.01)


def test_add_remove_particles_like_reference():
    pf = vpm.ParticleField(3, UJ=UJ_oracle)
    pf.add_particle([1, 2, 3], [0.1, 0.2, 0.3], 0.5, vol=2.0)
    pf.add_particle([4, 5, 6], [0.4, 0.5, 0.6], 0.7)
    pf.add_particle([7, 8, 9], [0.7, 0.8, 0.9], 0.9)
    with pytest.raises(RuntimeError, match="PARTICLE OVERFLOW"):
        pf.add_particle([0, 0, 0], [0, 0, 0], 1.0)
    pf.remove_particle(0)
    assert pf.np == 2
    assert np.array_equal(pf.X[0], [7, 8, 9])
    with pytest.raises(IndexError):
        pf.remove_particle(5)


def test_nonstandard_kernel_is_rejected():
    from vpm_gb300.uj import _kernel_id
    pf = vpm.ParticleField(2, kernel=vpm.Kernel("custom", 9))
    with pytest.raises(ValueError, match="standard kernels"):
        _kernel_id(pf)
