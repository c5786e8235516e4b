"""CPU oracle for the UJ hot path -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper over ``oracle/build/libvpm_oracle.so``, a plain-C restatement of
FLOWVPM.jl v4.0.3's UJ_direct (src/FLOWVPM_UJ.jl:21-37, pair math
src/FLOWVPM_fmm.jl:102-168), Estr (src/FLOWVPM_subfilterscale_models.jl:16-92)
and the rVPM RK3 step that consumes them (src/FLOWVPM_timeintegration.jl:388-532).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
use this module, as the checker.  The product library never imports it.

Parity pinning: the reference cannot run here (Julia + FastMultipole.jl are
absent), so the oracle is pinned to the reference's own known-answer checks:
the analytic singular-pair formulas of scripts/check_fmm.jl:39-71 and the
vortex-ring self-induced velocity test of test/runtests_singlevortexring.jl.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "libvpm_oracle.so")

KERNEL_SINGULAR, KERNEL_GAUSSIAN, KERNEL_GAUSSIANERF, KERNEL_WINCKELMANS = 0, 1, 2, 3
RESET, RESET_SFS, SFS, TRANSPOSED = 1, 2, 4, 8
NFIELDS = 46

_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i64 = ctypes.c_int64


class StepParams(ctypes.Structure):
    """Mirror of ``oracle_step_params`` (oracle/vpm_oracle.h)."""
    _fields_ = [
        ("kernel", ctypes.c_int), ("transposed", ctypes.c_int),
        ("f", ctypes.c_double), ("g", ctypes.c_double),
        ("Uinf", ctypes.c_double * 3),
        ("relaxation", ctypes.c_int), ("rlxf", ctypes.c_double),
        ("sfs", ctypes.c_int), ("Cs", ctypes.c_double),
        ("alpha", ctypes.c_double), ("sfs_rlxf", ctypes.c_double),
        ("minC", ctypes.c_double), ("maxC", ctypes.c_double),
        ("force_positive", ctypes.c_int), ("clip_backscatter", ctypes.c_int),
        ("viscous", ctypes.c_int), ("nu", ctypes.c_double), ("sgm0", ctypes.c_double),
        ("beta", ctypes.c_double), ("t_sgm", ctypes.c_double),
        ("erf_mode", ctypes.c_int), ("nthreads", ctypes.c_int),
    ]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle (same flags as oracle/Makefile); returns the library path."""
    src = os.path.join(_HERE, "vpm_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
        subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off",
                        "-std=c99", "-shared", "-o", _LIB_PATH, src, "-lm"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_erf_ref.restype = ctypes.c_double
        L.oracle_erf_ref.argtypes = [ctypes.c_double]
        L.oracle_zeta.restype = ctypes.c_double
        L.oracle_zeta.argtypes = [ctypes.c_int, ctypes.c_double]
        L.oracle_g_dgdr.argtypes = [ctypes.c_int, ctypes.c_double, _dp, _dp]
        L.oracle_uj_direct.restype = ctypes.c_int
        L.oracle_uj_direct.argtypes = [_dp, _i64, _i64, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int]
        L.oracle_uj_pairs.argtypes = [_i64, _i64, _dp, _i64, _dp, _dp, _dp, _dp, _dp,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_estr_pairs.argtypes = [_i64, _i64, _dp, _dp, _u8p, _i64, _dp, _dp, _dp,
                                        _dp, _u8p, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_zeta_pairs.argtypes = [_i64, _i64, _dp, _i64, _dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
        L.oracle_update_particle_states.argtypes = [_dp, _i64, _i64, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, _dp,
                                                    ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_int]
        L.oracle_relax.argtypes = [_dp, _i64, _i64, ctypes.c_double, ctypes.c_int]
        L.oracle_uj_adjoint.argtypes = [_i64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int,
                                        ctypes.c_int]
        L.oracle_g_d1_d2.argtypes = [ctypes.c_int, ctypes.c_double, _dp, _dp, _dp]
        L.oracle_estr_adjoint.argtypes = [_i64, _dp, _dp, _dp, _dp, _u8p, _dp, _dp, _dp, _dp, _dp, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int]
        L.oracle_rk3_step.restype = ctypes.c_int
        L.oracle_rk3_step.argtypes = [_dp, _i64, _i64, ctypes.c_double, ctypes.c_int,
                                      ctypes.POINTER(StepParams)]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def erf_ref(x: float) -> float:
    return lib().oracle_erf_ref(float(x))


def zeta(kernel: int, r: float) -> float:
    return lib().oracle_zeta(int(kernel), float(r))


def g_dgdr(kernel: int, r: float):
    g, dg = ctypes.c_double(), ctypes.c_double()
    lib().oracle_g_dgdr(int(kernel), float(r), ctypes.byref(g), ctypes.byref(dg))
    return g.value, dg.value


def uj_direct(particles: np.ndarray, np_: int, kernel: int, flags: int,
              erf_mode: int = 0, nthreads: int = 0) -> None:
    """UJ_direct on a Fortran-ordered (46, maxparticles) float64 matrix, in place."""
    assert particles.dtype == np.float64 and particles.flags.f_contiguous
    assert particles.shape[0] == NFIELDS
    rc = lib().oracle_uj_direct(_p(particles), NFIELDS, int(np_), int(kernel), int(flags),
                                int(erf_mode), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle_uj_direct failed ({rc})")


def uj_pairs(xt, xs, gs, sgs, kernel: int, targets=None, erf_mode: int = 0,
             compensated: bool = False, nthreads: int = 0):
    """Return (U[nt,3], J[nt,9]) of sources on targets; `targets` = (t0, t1) subset."""
    xt, xs, gs, sgs = _c(xt), _c(xs), _c(gs), _c(sgs)
    nt = xt.shape[0]
    t0, t1 = targets if targets is not None else (0, nt)
    U = np.zeros((nt, 3))
    J = np.zeros((nt, 9))
    lib().oracle_uj_pairs(t0, t1, _p(xt), xs.shape[0], _p(xs), _p(gs), _p(sgs), _p(U), _p(J),
                          int(kernel), int(erf_mode), int(bool(compensated)), int(nthreads))
    return U[t0:t1], J[t0:t1]


def zeta_pairs(xt, xs, gs, sgs, kernel: int, targets=None, nthreads: int = 0):
    """Return W[nt,3] = zeta_direct of the sources on the targets (self pairs included)."""
    xt, xs, gs, sgs = _c(xt), _c(xs), _c(gs), _c(sgs)
    nt = xt.shape[0]
    t0, t1 = targets if targets is not None else (0, nt)
    W = np.zeros((nt, 3))
    lib().oracle_zeta_pairs(t0, t1, _p(xt), xs.shape[0], _p(xs), _p(gs), _p(sgs), _p(W), int(kernel),
                            int(nthreads))
    return W[t0:t1]


def estr_pairs(xt, Jt, xs, gs, sgs, Js, kernel: int, transposed: bool = True,
               static_t=None, static_s=None, targets=None, nthreads: int = 0):
    """Return SFS[nt,3] (Estr of sources on targets)."""
    xt, Jt, xs, gs, sgs, Js = map(_c, (xt, Jt, xs, gs, sgs, Js))
    nt = xt.shape[0]
    t0, t1 = targets if targets is not None else (0, nt)
    st = None if static_t is None else _c(static_t, np.uint8)
    ss = None if static_s is None else _c(static_s, np.uint8)
    S = np.zeros((nt, 3))
    lib().oracle_estr_pairs(t0, t1, _p(xt), _p(Jt),
                            None if st is None else st.ctypes.data_as(_u8p),
                            xs.shape[0], _p(xs), _p(gs), _p(sgs), _p(Js),
                            None if ss is None else ss.ctypes.data_as(_u8p),
                            _p(S), int(kernel), int(bool(transposed)), int(nthreads))
    return S[t0:t1]


def uj_adjoint(x, gam, sig, Ubar, Jbar, kernel: int, nthreads: int = 0):
    """(xbar[n,3], gbar[n,3], sbar[n]) = gradients of sum(Ubar*U) + sum(Jbar*J) for the
    self-induced U, J of one particle set."""
    x, gam, sig, Ubar, Jbar = map(_c, (x, gam, sig, Ubar, Jbar))
    n = x.shape[0]
    xb = np.zeros((n, 3)); gb = np.zeros((n, 3)); sb = np.zeros(n)
    lib().oracle_uj_adjoint(n, _p(x), _p(gam), _p(sig), _p(Ubar), _p(Jbar), _p(xb), _p(gb), _p(sb),
                            int(kernel), int(nthreads))
    return xb, gb, sb


def estr_adjoint(x, gam, sig, J, Sbar, kernel: int, transposed: bool = True, static=None, nthreads: int = 0):
    """(xbar[n,3], gbar[n,3], sbar[n], Jbar[n,9]) = gradients of sum(Sbar * SFS) for the
    self-induced Estr of one particle set (static particles: 0/1 flags, or None)."""
    x, gam, sig, J, Sbar = map(_c, (x, gam, sig, J, Sbar))
    n = x.shape[0]
    st = None if static is None else _c(static, np.uint8)
    xb = np.zeros((n, 3)); gb = np.zeros((n, 3)); sb = np.zeros(n); Jb = np.zeros((n, 9))
    lib().oracle_estr_adjoint(n, _p(x), _p(gam), _p(sig), _p(J), None if st is None else st.ctypes.data_as(_u8p),
                              _p(Sbar), _p(xb), _p(gb), _p(sb), _p(Jb), int(kernel), int(bool(transposed)),
                              int(nthreads))
    return xb, gb, sb, Jb


def g_d1_d2(kernel: int, rho: float):
    g, d1, d2 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib().oracle_g_d1_d2(int(kernel), float(rho), ctypes.byref(g), ctypes.byref(d1), ctypes.byref(d2))
    return g.value, d1.value, d2.value


def update_particle_states(particles, np_, a, b, dt, Uinf, f, g, zeta0, transposed=True):
    U = _c(Uinf)
    lib().oracle_update_particle_states(_p(particles), NFIELDS, int(np_), a, b, dt, _p(U),
                                        f, g, zeta0, int(bool(transposed)))


def relax(particles, np_, rlxf, corrected=False):
    lib().oracle_relax(_p(particles), NFIELDS, int(np_), float(rlxf), int(bool(corrected)))


def rk3_step(particles, np_, dt, params: StepParams, relax: bool = False) -> int:
    return lib().oracle_rk3_step(_p(particles), NFIELDS, int(np_), float(dt), int(bool(relax)),
                                 ctypes.byref(params))
