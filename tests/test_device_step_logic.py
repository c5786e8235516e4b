"""CPU check of the per-particle logic of vpm_gb300.device_step (rVPM RK3,
dynamic SFS, core spreading, relaxation on SoA tensors) against the host
mirror of the reference's step (vpm_gb300.timeintegration).  Both sides take
their pair sums from the oracle, so any difference is in the step logic
itself; the GPU form of the same comparison is tests/test_gpu_device_step.py.
"""
import numpy as np
import pytest
import torch

import oracle
import vpm_gb300 as vpm
from vpm_gb300 import device_step as ds
from vpm_gb300 import workloads
from helpers import normwise


class OracleCtx:
    """Stands in for vpm_gb300.Context: the same two calls, computed by the oracle on CPU tensors."""

    def uj_dev(self, xt, xs, gs, sgs, U, J, kernel, precision):
        Ut, Jt = oracle.uj_pairs(xt.numpy(), xs.numpy(), gs.numpy(), sgs.numpy(), kernel)
        U += torch.from_numpy(Ut)
        J += torch.from_numpy(Jt)

    def estr_dev(self, xt, Jt, xs, gs, sgs, Js, SFS, kernel, precision, transposed=True):
        S = oracle.estr_pairs(xt.numpy(), Jt.numpy(), xs.numpy(), gs.numpy(), sgs.numpy(), Js.numpy(), kernel,
                              transposed)
        SFS += torch.from_numpy(S)


class OracleZetaCtx(OracleCtx):
    def zeta_dev(self, xt, xs, gs, sgs, W, kernel, precision):
        W += torch.from_numpy(oracle.zeta_pairs(xt.numpy(), xs.numpy(), gs.numpy(), sgs.numpy(), kernel))


def UJ_oracle(pfield, rbf=False, sfs=False, reset=True, reset_sfs=False, **kw):
    flags = (oracle.RESET if reset else 0) | (oracle.RESET_SFS if reset_sfs else 0) | \
            (oracle.SFS if sfs else 0) | (oracle.TRANSPOSED if pfield.transposed else 0)
    oracle.uj_direct(pfield.particles, pfield.np, pfield.kernel.kid, flags)


@pytest.mark.parametrize("with_sfs,with_visc", [(True, True), (True, False), (False, False)])
def test_device_step_logic_matches_host_mirror(with_sfs, with_visc):
    X, G, s = workloads.leapfrog_rings(600, nper=10)
    pf = vpm.ParticleField(X.shape[0], kernel=vpm.gaussianerf, UJ=UJ_oracle, relaxation=vpm.pedrizzetti,
                           SFS=vpm.SFS_Cd_twolevel_nobackscatter if with_sfs else vpm.noSFS,
                           viscous=vpm.CoreSpreading(1e-4, 0.05) if with_visc else None)
    pf.add_particles(X, G, s)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    fld = ds.DeviceField(t(X), t(G), t(s), kernel=2, precision=0)
    sfs = ds.DynamicSFSParams() if with_sfs else None
    visc = ds.CoreSpreadingParams(1e-4, 0.05) if with_visc else None
    ctx = OracleCtx()
    n = pf.np
    for step in range(2):
        pf.nextstep(0.005, relax=True)
        ds.rk3_step(fld, 0.005, ctx, sfs=sfs, viscous=visc, relax_rlxf=0.3)
        P = pf.particles
        for name, rows, v in (("X", slice(0, 3), fld.x), ("Gamma", slice(3, 6), fld.gam), ("U", slice(9, 12), fld.U),
                              ("J", slice(15, 24), fld.J)):
            assert normwise(v.numpy(), P[rows, :n].T)[0] <= 1e-13, (step, name)
        assert normwise(fld.sig.numpy(), P[6, :n])[0] <= 1e-14
        if with_sfs:
            assert normwise(fld.SFS.numpy(), P[39:42, :n].T)[0] <= 1e-13
            assert normwise(fld.C.numpy(), P[36:39, :n].T)[0] <= 1e-10
            assert (fld.C[:, 0] >= 0).all()          # force_positive
    if with_visc:
        assert visc.t_sgm == pytest.approx(pf.viscous.t_sgm, abs=1e-15)


def test_core_spreading_reset_needs_volumes():
    X, G, s = workloads.leapfrog_rings(200, nper=10)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    fld = ds.DeviceField(t(X), t(G), t(s), kernel=2, precision=0)
    visc = ds.CoreSpreadingParams(nu=10.0, sgm0=0.05)      # sigma grows past beta within one step
    with pytest.raises(ValueError):
        ds.rk3_step(fld, 0.005, OracleZetaCtx(), viscous=visc)


def test_impulse_matches_numpy():
    X, G, s = workloads.leapfrog_rings(200, nper=10)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    fld = ds.DeviceField(t(X), t(G), t(s))
    Ir = 0.5 * np.cross(X, G).sum(0)
    assert np.abs(ds.impulse(fld).numpy() - Ir).max() <= 1e-13 * np.abs(Ir).max()


def zeta_oracle(pfield):
    """zeta_direct through the oracle: rows 16:18 of every particle."""
    n = pfield.np
    P = pfield.particles
    X = np.ascontiguousarray(P[0:3, :n].T)
    P[15:18, :n] = oracle.zeta_pairs(X, X, np.ascontiguousarray(P[3:6, :n].T), P[6, :n], pfield.kernel.kid).T


def test_core_spreading_reset_matches_host_mirror():
    """A core-size reset (src/FLOWVPM_viscous.jl:194-219): zeta_direct of the
    current strengths becomes the target, sigma returns to sgm0 and the RBF
    conjugate gradient (:314-454) finds new strengths.  beta = 1.0001 makes the
    first step reset."""
    from vpm_gb300 import rings
    X, G, s, vol = rings.ring_sections(1.0, 1.0, 0.1, 40, 7, 0.05)
    n = X.shape[0]
    nu, sgm0 = 1e-3, 0.05
    pf = vpm.ParticleField(n, kernel=vpm.gaussianerf, UJ=UJ_oracle, relaxation=vpm.norelaxation,
                           viscous=vpm.CoreSpreading(nu, sgm0, beta=1.0001, zeta=zeta_oracle))
    pf.add_particles(X, G, s, vol=vol)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    fld = ds.DeviceField(t(X), t(G), t(s), kernel=2, precision=0, vol=t(np.broadcast_to(vol, (n,))))
    visc = ds.CoreSpreadingParams(nu, sgm0, beta=1.0001)
    pf.nextstep(0.01)
    ds.rk3_step(fld, 0.01, OracleZetaCtx(), viscous=visc)
    P = pf.particles
    assert pf.viscous.t_sgm == 0.0 and visc.t_sgm == 0.0
    assert np.all(P[6, :n] == sgm0) and bool((fld.sig == sgm0).all())
    for name, rows, v in (("X", slice(0, 3), fld.x), ("Gamma", slice(3, 6), fld.gam)):
        assert normwise(v.numpy(), P[rows, :n].T)[0] <= 1e-12, name
    # the reference's stopping rule: |b - A x| <= tol |b - A x0| per component, x0 = b vol
    Xn = np.ascontiguousarray(P[0:3, :n].T)
    targ = P[33:36, :n].T
    W = oracle.zeta_pairs(Xn, Xn, np.ascontiguousarray(P[3:6, :n].T), P[6, :n], 2)
    r0 = targ - oracle.zeta_pairs(Xn, Xn, targ * P[7, :n][:, None], P[6, :n], 2)
    live = (targ ** 2).sum(0) > 1e-12 * (targ ** 2).sum()     # the ring's axial component is zero
    res = np.sqrt(((W - targ) ** 2).sum(0)[live] / (r0 ** 2).sum(0)[live])
    assert live.sum() == 2 and (res <= 1e-3).all(), res
