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


    # the per-particle kernels of the step (csrc/step.cu), restated on CPU tensors in the
    # reference's operation order (src/FLOWVPM_timeintegration.jl:463-532,
    # src/FLOWVPM_viscous.jl:175-192, src/FLOWVPM_relaxation.jl:62-81,
    # src/FLOWVPM_subfilterscale.jl:541-673 and :287-296)
    def rk3_stage_dev(self, a, b, dt, Uinf, f, g, zeta0, x, gam, sig, U, J, M, *, SFS=None, C=None, nu=None,
                      transposed=True):
        from vpm_gb300.autodiff import _stretch
        G, s = gam, sig
        Cc = C[:, 0] if C is not None else torch.zeros_like(s)
        S = SFS if SFS is not None else torch.zeros_like(G)
        M[:, 0:3] = a * M[:, 0:3] + dt * (U + torch.tensor(Uinf, dtype=torch.float64))
        x += b * M[:, 0:3]
        MM = _stretch(J, G, transposed)
        Gn2 = (G * G).sum(1)
        s3 = s * s * s
        MM4 = (f + g) / (1 + 3 * f) * (MM * G).sum(1)
        MM4 = MM4 - f / (1 + 3 * f) * (Cc * S[:, 0] * G[:, 0] + Cc * S[:, 1] * G[:, 1] + Cc * S[:, 2] * G[:, 2]) * \
            s3 / zeta0
        pos = Gn2 > 0
        MM4 = torch.where(pos, MM4 / torch.where(pos, Gn2, torch.ones_like(Gn2)), torch.zeros_like(Gn2))
        M[:, 3:6] = a * M[:, 3:6] + dt * (MM - 3 * MM4[:, None] * G - Cc[:, None] * S * s3[:, None] / zeta0)
        M[:, 7] = a * M[:, 7] - dt * (s * MM4)
        G += b * M[:, 3:6]
        s += b * M[:, 7]
        if nu is not None:
            M[:, 6] = a * M[:, 6] + dt * 2 * nu
            sig.copy_(torch.sqrt(sig ** 2 + b * M[:, 6]))

    def relax_dev(self, rlxf, J, gam):
        w = torch.stack([J[:, 5] - J[:, 7], J[:, 6] - J[:, 2], J[:, 1] - J[:, 3]], dim=1)
        nw = torch.sqrt((w * w).sum(1))
        nG = torch.sqrt((gam * gam).sum(1))
        ok = nw != 0
        newg = (1 - rlxf) * gam + rlxf * (nG / torch.where(ok, nw, torch.ones_like(nw)))[:, None] * w
        gam.copy_(torch.where(ok[:, None], newg, gam))

    def dynamic_after_dev(self, alpha, rlxf, minC, maxC, zeta0, G, s, J, SFS, Cp, M, *, force_positive=True,
                          clip_backscatter=True, subtract=False, transposed=True):
        from vpm_gb300.autodiff import _stretch
        if subtract:
            M[:, 0:3] -= _stretch(J, G, transposed)
            M[:, 3:6] -= SFS
        nume = (M[:, 0] * G[:, 0] + M[:, 1] * G[:, 1] + M[:, 2] * G[:, 2]) * (3 * alpha - 2)
        deno = (M[:, 3] * G[:, 0] + M[:, 4] * G[:, 1] + M[:, 5] * G[:, 2]) / (zeta0 / (s * s * s))
        C3 = torch.where(Cp[:, 2] == 0, deno, Cp[:, 2])
        C3 = torch.where(C3 == 0, torch.full_like(C3, ds.EPS), C3)
        nume = rlxf * nume + (1 - rlxf) * Cp[:, 1]
        deno = rlxf * deno + (1 - rlxf) * C3
        ratio = (nume / deno).abs()
        big = ratio > maxC
        deno = torch.where(big & (deno.abs() < C3.abs()), torch.sign(deno) * C3.abs(), deno)
        nume = torch.where(big & ((nume / deno).abs() >= maxC), torch.sign(nume) * deno.abs() * maxC, nume)
        small = (~big) & (ratio < minC)
        nume = torch.where(small, torch.sign(nume) * deno.abs() * minC, nume)
        C1 = nume / deno
        if bool(torch.isnan(C1).any()):
            raise FloatingPointError("NaN in dynamicprocedure_pseudo3level_afterUJ")
        if force_positive:
            C1 = C1 * torch.sign(C1)
        Cp[:, 0] = C1
        Cp[:, 1] = nume
        Cp[:, 2] = deno
        M.zero_()
        if clip_backscatter:
            clip = Cp[:, 0] * (G * SFS).sum(1) < 0
            Cp[:, 0] = torch.where(clip, Cp[:, 0] * 0, Cp[:, 0])


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
