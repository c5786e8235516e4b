"""Device-resident rVPM step (vpm_gb300.device_step) against the host mirror's
rungekutta3 (src/FLOWVPM_timeintegration.jl:388-532) driven by the same UJ
precision:

* two coaxial rings (R=1 and R=0.7, 0.3 apart, 10 particles per section),
  Gaussian-erf, rVPM, the dynamic SFS model SFS_Cd_twolevel_nobackscatter
  (src/FLOWVPM.jl:223), core spreading nu=1e-4 and Pedrizzetti relaxation;
  state, U, J, SFS and the C coefficients after every step;
* the same without SFS/viscosity (the plain ring step);
* the near-field form with theta=0 equals the all-pairs form (random cloud);
* the near-field step with the dynamic SFS model: FP32-comp with the fused
  near-field differences against the FP64 near-field step.
Tolerances are normwise (max|err| / max|ref|).  C is a ratio of two
differences of nearly equal stretching terms (filter widths 1 and 0.999), so
it carries ~1e3 times the state's rounding.
"""
import numpy as np
import pytest

import vpm_gb300 as vpm
from vpm_gb300 import device_step as ds
from vpm_gb300 import workloads
from helpers import normwise

pytestmark = pytest.mark.gpu


def _fields(n_total, kernel, UJ, sfs, viscous, precision):
    import torch
    X, G, s = workloads.leapfrog_rings(n_total, nper=10)
    pf = vpm.ParticleField(X.shape[0], kernel=kernel, UJ=UJ, relaxation=vpm.pedrizzetti,
                           SFS=sfs if sfs is not None else vpm.noSFS,
                           viscous=viscous() if viscous is not None else None)
    pf.add_particles(X, G, s)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    kid = {id(vpm.gaussianerf): vpm._lib.KERNEL_GAUSSIANERF, id(vpm.winckelmans): vpm._lib.KERNEL_WINCKELMANS}
    fld = ds.DeviceField(dev(X), dev(G), dev(s), kernel=kid[id(kernel)], precision=precision)
    return pf, fld


def _compare(pf, fld, tol, tolC, step):
    n = pf.np
    P = pf.particles
    pairs = (("X", slice(0, 3), fld.x), ("Gamma", slice(3, 6), fld.gam), ("U", slice(9, 12), fld.U),
             ("J", slice(15, 24), fld.J), ("SFS", slice(39, 42), fld.SFS))
    for name, rows, t in pairs:
        ref = P[rows, :n].T
        if not np.abs(ref).max() > 0:
            assert not t.abs().max().item() > 0, (step, name)
            continue
        e = normwise(t.cpu().numpy(), ref)[0]
        assert e <= tol, (step, name, e)
    e = normwise(fld.sig.cpu().numpy(), P[6, :n])[0]
    assert e <= tol, (step, "sigma", e)
    if np.abs(P[36:39, :n]).max() > 0:
        e = normwise(fld.C.cpu().numpy(), P[36:39, :n].T)[0]
        assert e <= tolC, (step, "C", e)


@pytest.mark.parametrize("prec,tol,tolC", [(0, 1e-11, 1e-8), (1, 2e-5, 2e-3)])
def test_dynamic_sfs_core_spreading_matches_host_mirror(ctx, prec, tol, tolC):
    """Both precisions of the device step against the FP64 host mirror.  The
    FP32-comp step takes the test-filter differences from vpm_dynamic_diff_dev,
    so its coefficients C follow the FP64 ones (subtracting two FP32-comp
    evaluations instead leaves C with ~1e-2 of noise)."""
    nu, sgm0 = 1e-4, 0.05
    UJ = vpm.UJ_gb300
    pf, fld = _fields(2000, vpm.gaussianerf, UJ, vpm.SFS_Cd_twolevel_nobackscatter,
                      lambda: vpm.CoreSpreading(nu, sgm0), prec)
    sfs = ds.DynamicSFSParams()
    visc = ds.CoreSpreadingParams(nu, sgm0)
    for step in range(3):
        pf.nextstep(0.005, relax=True)
        ds.rk3_step(fld, 0.005, ctx, sfs=sfs, viscous=visc, relax_rlxf=0.3)
        _compare(pf, fld, tol, tolC, step)
    assert abs(visc.t_sgm - pf.viscous.t_sgm) < 1e-15
    assert fld.nt == pf.nt and abs(fld.t - pf.t) < 1e-15


@pytest.mark.parametrize("kernel", ["gaussianerf", "winckelmans"])
def test_plain_ring_step_matches_host_mirror(ctx, kernel):
    k = getattr(vpm, kernel)
    pf, fld = _fields(1400, k, vpm.UJ_gb300, None, None, 0)
    for step in range(3):
        pf.nextstep(0.01, relax=True)
        ds.rk3_step(fld, 0.01, ctx, relax_rlxf=0.3)
        _compare(pf, fld, 1e-11, 1e-8, step)


def test_nearfield_theta_zero_step_equals_all_pairs(ctx):
    """theta = 0 makes every leaf pair near when no two leaves have radius 0
    (0 * r >= 0 + 0 would accept them as far), which holds on a random cloud:
    checked through the pair count.  The near-field sums run in another order
    than the all-pairs ones, so they agree to rounding; the step is taken
    without the dynamic SFS model, whose clipping branches (C bounds, sign,
    backscatter) turn rounding differences into O(1) changes of C on particles
    that sit at a branch.  The SFS term itself is compared directly."""
    import torch
    from helpers import random_cloud
    X, G, s = random_cloud(2500, seed=17, box=0.5)
    dev = lambda v: torch.tensor(np.ascontiguousarray(v), device="cuda", dtype=torch.float64)
    a = ds.DeviceField(dev(X), dev(G), dev(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=0)
    b = ds.DeviceField(dev(X), dev(G), dev(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=0)
    b.leaflist = (64, 0.0)
    U, J = torch.zeros_like(b.U), torch.zeros_like(b.J)
    assert ctx.p2p_leaflist_dev(b.x, b.gam, b.sig, U, J, leaf_size=64, theta=0.0, kernel=2, precision=0)[2] == 2500 ** 2
    va, vb = ds.CoreSpreadingParams(1e-4, 0.05), ds.CoreSpreadingParams(1e-4, 0.05)
    for _ in range(2):
        ds.rk3_step(a, 0.005, ctx, viscous=va, relax_rlxf=0.3)
        ds.rk3_step(b, 0.005, ctx, viscous=vb, relax_rlxf=0.3)
    for name in ("x", "gam", "sig", "U", "J"):
        ta, tb = getattr(a, name), getattr(b, name)
        assert normwise(tb.cpu().numpy(), ta.cpu().numpy())[0] <= 1e-12, name
    ds.uj(a, ctx, sfs=True, reset_sfs=True)
    ds.uj(b, ctx, sfs=True, reset_sfs=True)
    assert normwise(b.SFS.cpu().numpy(), a.SFS.cpu().numpy())[0] <= 1e-12


def test_monitors(ctx):
    import torch
    _, fld = _fields(2000, vpm.gaussianerf, vpm.UJ_gb300, None, None, 0)
    I = ds.impulse(fld).cpu().numpy()
    X, G = fld.x.cpu().numpy(), fld.gam.cpu().numpy()
    Ir = 0.5 * np.cross(X, G).sum(0)
    assert np.abs(I - Ir).max() <= 1e-13 * np.abs(Ir).max()
    ds.uj(fld, ctx)
    E = ds.energy(fld)
    Ur = fld.U.cpu().numpy()
    assert abs(E - 0.5 * (Ur * np.cross(X, G)).sum()) <= 1e-12 * abs(E)
    assert E > 0 and torch.isfinite(fld.J).all()


@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 2e-5)])
def test_core_size_reset_matches_host_mirror(ctx, prec, tol):
    """Core spreading past beta resets: zeta_direct (vpm_zeta / vpm_zeta_dev)
    gives the target vorticity, sigma returns to sgm0, and the RBF conjugate
    gradient rebuilds the strengths -- host mirror and device step alike."""
    import torch
    from vpm_gb300 import rings
    X, G, s, vol = rings.ring_sections(1.0, 1.0, 0.1, 60, 7, 0.05)
    n = X.shape[0]
    nu, sgm0 = 1e-3, 0.05
    zhook = vpm.zeta_gb300 if prec == 0 else vpm.zeta_gb300_mixed
    UJ = vpm.UJ_gb300 if prec == 0 else vpm.UJ_gb300_mixed
    # The planar ring's axial strength is zero up to rounding, and the RBF solve judges each
    # component against its own initial residual, so that component cannot converge:
    # iterror=False lets both sides run all itmax iterations on it instead of raising.
    pf = vpm.ParticleField(n, kernel=vpm.gaussianerf, UJ=UJ, relaxation=vpm.norelaxation,
                           viscous=vpm.CoreSpreading(nu, sgm0, beta=1.0001, zeta=zhook, iterror=False))
    pf.add_particles(X, G, s, vol=vol)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    fld = ds.DeviceField(dev(X), dev(G), dev(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=prec,
                         vol=dev(np.broadcast_to(vol, (n,))))
    visc = ds.CoreSpreadingParams(nu, sgm0, beta=1.0001, iterror=False)
    for step in range(2):
        pf.nextstep(0.01)
        ds.rk3_step(fld, 0.01, ctx, viscous=visc)
        assert pf.viscous.t_sgm == 0.0 and visc.t_sgm == 0.0
        P = pf.particles
        for name, rows, t in (("X", slice(0, 3), fld.x), ("Gamma", slice(3, 6), fld.gam)):
            assert normwise(t.cpu().numpy(), P[rows, :n].T)[0] <= tol, (step, name)
        assert bool((fld.sig == sgm0).all()) and np.all(P[6, :n] == sgm0)


@pytest.mark.parametrize("kernel,alpha", [(2, 0.999), (3, 0.999), (1, 0.999), (2, 0.667)])
def test_dynamic_diff_matches_two_fp64_evaluations(ctx, kernel, alpha):
    """vpm_dynamic_diff_dev against the oracle's two evaluations:
    dJ = J(alpha sigma) - J(sigma), dSFS = SFS(alpha sigma; J_alpha) - SFS(sigma; J)."""
    import torch
    import oracle
    X, G, s = workloads.leapfrog_rings(3000, nper=10)
    n = X.shape[0]
    _, J0 = oracle.uj_pairs(X, X, G, s, kernel)
    _, Ja = oracle.uj_pairs(X, X, G, s * alpha, kernel)
    dJ_ref = Ja - J0
    dS_ref = (oracle.estr_pairs(X, Ja, X, G, s * alpha, Ja, kernel, True) -
              oracle.estr_pairs(X, J0, X, G, s, J0, kernel, True))
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    for prec, tolJ, tolS in ((0, 1e-10, 1e-9), (1, 2e-6, 2e-5)):
        dJ = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
        dS = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
        ctx.dynamic_diff_dev(d(X), d(G), d(s), d(J0), alpha, dJ, dS, kernel, prec)
        eJ = normwise(dJ.cpu().numpy(), dJ_ref)[0]
        eS = normwise(dS.cpu().numpy(), dS_ref)[0]
        assert eJ <= tolJ and eS <= tolS, (prec, eJ, eS)


def test_nearfield_dynamic_sfs_step_follows_fp64(ctx):
    """Near-field state (leaf_size 32, theta 0.4) with the dynamic SFS model: the
    FP32-comp step, whose test-filter differences come from
    vpm_dynamic_diff_leaflist_dev, against the FP64 step that evaluates the
    near field twice and subtracts (the reference's way)."""
    import torch
    X, G, s = workloads.leapfrog_rings(2000, nper=10)
    dev = lambda v: torch.tensor(np.ascontiguousarray(v), device="cuda", dtype=torch.float64)
    flds = []
    for prec in (0, 1):
        f = ds.DeviceField(dev(X), dev(G), dev(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=prec)
        f.leaflist = (32, 0.4)
        flds.append(f)
    p64, p32 = ds.DynamicSFSParams(), ds.DynamicSFSParams()
    for step in range(3):
        ds.rk3_step(flds[0], 0.005, ctx, sfs=p64, relax_rlxf=0.3)
        ds.rk3_step(flds[1], 0.005, ctx, sfs=p32, relax_rlxf=0.3)
        for name, tol in (("x", 2e-5), ("gam", 2e-5), ("sig", 2e-5), ("J", 2e-5), ("SFS", 2e-5), ("C", 2e-3)):
            a, b = getattr(flds[0], name), getattr(flds[1], name)
            e = normwise(b.cpu().numpy(), a.cpu().numpy())[0]
            assert e <= tol, (step, name, e)


def test_nearfield_core_size_reset_theta_zero_equals_all_pairs(ctx):
    """The core-size reset of a near-field state takes zeta_fmm's sum over the
    near lists (vpm_zeta_leaflist_dev); with theta = 0 on a random cloud every
    pair is near, so the reset step equals the all-pairs one to rounding."""
    import torch
    from helpers import random_cloud
    X, G, s = random_cloud(2000, seed=21, box=0.4, sig_lo=0.04, sig_hi=0.05)
    n = X.shape[0]
    dev = lambda v: torch.tensor(np.ascontiguousarray(v), device="cuda", dtype=torch.float64)
    vol = dev(np.full(n, 0.4 ** 3 / n))
    a = ds.DeviceField(dev(X), dev(G), dev(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=0, vol=vol)
    b = ds.DeviceField(dev(X), dev(G), dev(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=0, vol=vol.clone())
    b.leaflist = (64, 0.0)
    va = ds.CoreSpreadingParams(1e-3, 0.045, beta=1.0001, iterror=False)
    vb = ds.CoreSpreadingParams(1e-3, 0.045, beta=1.0001, iterror=False)
    ds.rk3_step(a, 0.01, ctx, viscous=va)
    ds.rk3_step(b, 0.01, ctx, viscous=vb)
    assert va.t_sgm == 0.0 and vb.t_sgm == 0.0     # the reset ran on both
    for name in ("x", "gam", "sig"):
        ta, tb = getattr(a, name), getattr(b, name)
        assert normwise(tb.cpu().numpy(), ta.cpu().numpy())[0] <= 1e-11, name


@pytest.mark.parametrize("transposed", [True, False])
def test_step_kernels_match_their_restatement(ctx, transposed):
    """vpm_rk3_stage_dev, vpm_relax_dev and vpm_dynamic_after_dev against the torch
    restatement of the same arithmetic (the CPU stand-in of tests/test_device_step_logic.py)
    on random states: the same values to FP64 rounding."""
    import torch
    from test_device_step_logic import OracleCtx
    ref = OracleCtx()
    rng = np.random.default_rng(11 + int(transposed))
    n = 3000
    r = lambda *sh: rng.normal(size=sh)
    st = dict(x=r(n, 3), gam=r(n, 3) * 1e-2, sig=rng.uniform(0.01, 0.05, n), U=r(n, 3), J=r(n, 9), SFS=r(n, 3),
              C=r(n, 3) * 1e-3, M=r(n, 9) * 1e-3)
    st["gam"][:7] = 0.0                         # |Gamma| = 0: the stretching split is skipped
    st["C"][::5, 2] = 0.0                       # no earlier denominator
    st["J"][3, 5] = st["J"][3, 7]; st["J"][3, 6] = st["J"][3, 2]; st["J"][3, 1] = st["J"][3, 3]   # w = 0
    cpu = {k: torch.tensor(v) for k, v in st.items()}
    dev = {k: torch.tensor(v, device="cuda") for k, v in st.items()}
    for a, b in ((0.0, 1 / 3), (-5 / 9, 15 / 16), (-153 / 128, 8 / 15)):
        for side, c in ((cpu, ref), (dev, ctx)):
            c.rk3_stage_dev(a, b, 0.01, (0.1, -0.2, 0.3), 0.0, 0.2, 0.8, side["x"], side["gam"], side["sig"],
                            side["U"], side["J"], side["M"], SFS=side["SFS"], C=side["C"], nu=1e-3,
                            transposed=transposed)
    for side, c in ((cpu, ref), (dev, ctx)):
        c.relax_dev(0.3, side["J"], side["gam"])
        side["M"][:, 0:6] += 1e-4
        c.dynamic_after_dev(0.999, 0.005, 0.0, 1.0, 0.8, side["gam"], side["sig"], side["J"], side["SFS"], side["C"],
                            side["M"], subtract=True, transposed=transposed)
    for k in ("x", "gam", "sig", "C", "M"):
        e = normwise(dev[k].cpu().numpy(), cpu[k].numpy())[0]
        assert e <= 1e-13, (k, e)
    assert (dev["M"] == 0).all()


def test_dynamic_after_rejects_bad_bounds(ctx):
    """The reference's error cases of the C bounds (src/FLOWVPM_subfilterscale.jl:549-556)."""
    import torch
    z = lambda k: torch.zeros(10, k, dtype=torch.float64, device="cuda")
    for lo, hi in ((-0.1, 1.0), (0.0, -1.0), (0.5, 0.1)):
        with pytest.raises(vpm._lib.VPMError, match="Invalid C bounds"):
            ctx.dynamic_after_dev(0.999, 0.005, lo, hi, 0.8, z(3), z(1)[:, 0] + 0.05, z(9), z(3), z(3), z(9))


@pytest.mark.parametrize("n", [40000, 200000])
def test_dynamic_diff_fp32comp_follows_fp64_at_scale(ctx, n):
    """vpm_dynamic_diff_dev at the leapfrog workload's sizes (split reductions,
    many source tiles): the FP32-comp differences against FP64's two evaluations."""
    import torch
    X, G, s = workloads.leapfrog_rings(n, nper=10)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    x, g, sg = d(X), d(G), d(s)
    m = x.shape[0]
    U, J = torch.zeros(m, 3, device="cuda", dtype=torch.float64), torch.zeros(m, 9, device="cuda", dtype=torch.float64)
    ctx.uj_dev(x, x, g, sg, U, J, 2, 0)
    out = []
    for prec in (0, 1):
        dJ = torch.zeros(m, 9, device="cuda", dtype=torch.float64)
        dS = torch.zeros(m, 3, device="cuda", dtype=torch.float64)
        ctx.dynamic_diff_dev(x, g, sg, J, 0.999, dJ, dS, 2, prec)
        out.append((dJ.cpu().numpy(), dS.cpu().numpy()))
    eJ = normwise(out[1][0], out[0][0])[0]
    eS = normwise(out[1][1], out[0][1])[0]
    assert eJ <= 2e-6 and eS <= 2e-5, (eJ, eS)


def test_device_step_is_deterministic(ctx):
    """Two FP32-comp steps from the same state (dynamic SFS, core spreading,
    relaxation) give the same bits: the library's work is ordered with the torch
    work around it (it runs on torch's stream, and its own stream is a blocking
    one), and no pair sum depends on scheduling."""
    import torch
    X, G, s = workloads.leapfrog_rings(40000, nper=10)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    outs = []
    for _ in range(2):
        fld = ds.DeviceField(d(X), d(G), d(s), kernel=vpm._lib.KERNEL_GAUSSIANERF, precision=1)
        ds.rk3_step(fld, 0.005, ctx, sfs=ds.DynamicSFSParams(), viscous=ds.CoreSpreadingParams(1e-4, 0.05),
                    relax_rlxf=0.3)
        outs.append([t.clone() for t in (fld.x, fld.gam, fld.sig, fld.C, fld.J, fld.SFS)])
    for a, b in zip(*outs):
        assert torch.equal(a, b)
