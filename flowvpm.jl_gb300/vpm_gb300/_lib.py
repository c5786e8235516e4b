"""ctypes binding of libvpm_gb300.so (C ABI declared in include/vpm_gb300.h).

The library is the product path: there is no CPU fallback.  If the shared
library has not been built, or no sm_103 GPU is present, every entry point
raises instead of computing anything.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("VPM_GB300_LIB", os.path.join(PKG_ROOT, "lib", "libvpm_gb300.so"))

# status codes, kernels, precisions and flags of include/vpm_gb300.h
OK, ERR_ARG, ERR_CAPACITY, ERR_CUDA, ERR_NONFINITE, ERR_TIMEOUT, ERR_NODEVICE, ERR_STATE = 0, -1, -2, -3, -4, -5, -6, -7
KERNEL_SINGULAR, KERNEL_GAUSSIAN, KERNEL_GAUSSIANERF, KERNEL_WINCKELMANS = 0, 1, 2, 3
FP64, FP32COMP = 0, 1
RESET, RESET_SFS, SFS, TRANSPOSED, CHECK_FINITE, REUSE_LISTS = 1, 2, 4, 8, 16, 256
DYN_FORCE_POSITIVE, DYN_CLIP_BACKSCATTER, DYN_SUBTRACT = 32, 64, 128
CUDA_STREAM_LEGACY = 1   # cudaStreamLegacy, the legacy default stream's handle
NFIELDS = 46
FLOP_PER_UJ_PAIR = 74
FLOP_PER_ESTR_PAIR = 25
FLOP_PER_UJ_ADJ_PAIR = 186

_STATUS_NAMES = {ERR_ARG: "VPM_ERR_ARG", ERR_CAPACITY: "VPM_ERR_CAPACITY", ERR_CUDA: "VPM_ERR_CUDA",
                 ERR_NONFINITE: "VPM_ERR_NONFINITE", ERR_TIMEOUT: "VPM_ERR_TIMEOUT",
                 ERR_NODEVICE: "VPM_ERR_NODEVICE", ERR_STATE: "VPM_ERR_STATE"}

# Every exported symbol of include/vpm_gb300.h, with (restype, argtypes).
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double
SIGNATURES = {
    "vpm_ctx_create": (_int, [ctypes.POINTER(_vp), _int]),
    "vpm_ctx_destroy": (_int, [_vp]),
    "vpm_last_error": (ctypes.c_char_p, [_vp]),
    "vpm_ctx_set_stream": (_int, [_vp, _vp]),
    "vpm_ctx_set_timeout": (_int, [_vp, _dbl]),
    "vpm_ctx_set_near_capacity": (_int, [_vp, _i64, _i64]),
    "vpm_abi_version": (_int, []),
    "vpm_build_info": (ctypes.c_char_p, []),
    "vpm_launch_count": (_i64, [_vp]),
    "vpm_probe_ffma": (_int, [_vp, _vp]),
    "vpm_probe_dfma": (_int, [_vp, _vp]),
    "vpm_uj": (_int, [_vp, _vp, _i64, _i64, _int, _int, _int]),
    "vpm_uj_cross": (_int, [_vp, _vp, _i64, _i64, _vp, _i64, _i64, _int, _int]),
    "vpm_uj_dev": (_int, [_vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _int, _int]),
    "vpm_estr_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _int, _int, _int]),
    "vpm_uj_dev_noalloc": (_int, [_i64, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _int, _int, _vp]),
    "vpm_uj_adjoint_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _int, _int]),
    "vpm_estr_adjoint_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _int, _int,
                                    _int]),
    "vpm_zeta": (_int, [_vp, _vp, _i64, _i64, _int, _int]),
    "vpm_dynamic_diff_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _dbl, _vp, _vp, _int, _int, _int]),
    "vpm_zeta_dev": (_int, [_vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _int, _int]),
    "vpm_rk3_stage_dev": (_int, [_vp, _i64, _dbl, _dbl, _dbl, _vp, _dbl, _dbl, _dbl, _dbl, _int, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _vp, _vp]),
    "vpm_relax_dev": (_int, [_vp, _i64, _dbl, _vp, _vp]),
    "vpm_dynamic_after_dev": (_int, [_vp, _i64, _dbl, _dbl, _dbl, _dbl, _dbl, _int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpm_zeta_leaflist_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _int, _dbl, _int, _int, _int, _vp]),
    "vpm_dynamic_diff_leaflist_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _dbl, _vp, _vp, _int, _dbl, _int,
                                             _int, _int, _vp]),
    "vpm_p2p_leaflist_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _int, _dbl, _int, _int, _int,
                                    _vp]),
    "vpm_p2p_lists_dev": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp,
                                 _int, _int, _int, _vp]),
    "vpm_leaflist_host": (_int, [_i64, _vp, _int, _dbl, _vp, _vp, _vp, _vp, _vp, _vp]),
    "vpm_leaflist_dev": (_int, [_vp, _i64, _vp, _int, _dbl, _vp, _vp, _vp, _vp, _vp, _vp]),
}


def leaflist_host(x: np.ndarray, leaf_size: int = 64, theta: float = 0.4):
    """The octree leaf-pair lists of vpm_p2p_leaflist_dev (host only):
    (perm, leaf_begin, leaf_end, row, col)."""
    L = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.shape[0]
    sizes = np.zeros(2, dtype=np.int64)
    rc = L.vpm_leaflist_host(n, x.ctypes.data, int(leaf_size), float(theta), None, None, None, None, None,
                             sizes.ctypes.data)
    if rc != OK:
        raise VPMError(rc, L.vpm_last_error(None).decode())
    nl, nc = int(sizes[0]), int(sizes[1])
    perm = np.zeros(n, np.int32); lb = np.zeros(nl, np.int64); le = np.zeros(nl, np.int64)
    row = np.zeros(nl + 1, np.int64); col = np.zeros(nc, np.int32)
    rc = L.vpm_leaflist_host(n, x.ctypes.data, int(leaf_size), float(theta), perm.ctypes.data, lb.ctypes.data,
                             le.ctypes.data, row.ctypes.data, col.ctypes.data, sizes.ctypes.data)
    if rc != OK:
        raise VPMError(rc, L.vpm_last_error(None).decode())
    return perm, lb, le, row, col
NOALLOC_SCRATCH_BYTES = 64 << 20   # VPM_NOALLOC_SCRATCH_BYTES


class VPMError(RuntimeError):
    """A non-zero status returned by libvpm_gb300.so."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None
_lib_lock = threading.Lock()


def load() -> ctypes.CDLL:
    """Load libvpm_gb300.so and declare its signatures; raise if it is missing."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is not built: run `python flowvpm.jl_gb300/build.py` "
                    "(or __graft_entry__.build()); there is no CPU fallback")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (or None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")


class Context:
    """One libvpm_gb300 context (device buffers, a stream, a mutex)."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = ctypes.c_void_p()
        rc = self._L.vpm_ctx_create(ctypes.byref(h), int(device))
        if rc != OK:
            raise VPMError(rc, self._L.vpm_last_error(None).decode())
        self._h = h
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            self._L.vpm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != OK:
            raise VPMError(rc, self._L.vpm_last_error(self._h).decode())

    @property
    def launches(self) -> int:
        return int(self._L.vpm_launch_count(self._h))

    def set_stream(self, stream_handle: int | None):
        self._check(self._L.vpm_ctx_set_stream(self._h, stream_handle))

    def set_timeout(self, seconds: float):
        self._check(self._L.vpm_ctx_set_timeout(self._h, float(seconds)))

    def set_near_capacity(self, frontier_pairs: int, near_pairs: int):
        """Initial traversal capacities of the next near-field list build (grown on overflow)."""
        self._check(self._L.vpm_ctx_set_near_capacity(self._h, int(frontier_pairs), int(near_pairs)))

    # --------------------------------------------------- host-matrix drop-in
    def uj(self, particles: np.ndarray, np_: int, kernel: int, precision: int, flags: int):
        """vpm_uj on a Fortran-ordered (46, maxparticles) float64 matrix, in place."""
        if not (isinstance(particles, np.ndarray) and particles.dtype == np.float64
                and particles.flags.f_contiguous and particles.shape[0] == NFIELDS):
            raise TypeError("particles must be a Fortran-ordered float64 array of shape (46, maxparticles)")
        if np_ > particles.shape[1]:
            raise ValueError(f"np={np_} exceeds maxparticles={particles.shape[1]}")
        self._check(self._L.vpm_uj(self._h, _ptr(particles), NFIELDS, int(np_), int(kernel),
                                   int(precision), int(flags)))

    def zeta(self, particles: np.ndarray, np_: int, kernel: int, precision: int):
        """vpm_zeta (zeta_direct) on a Fortran-ordered (46, maxparticles) matrix: rows 16:18."""
        if not (isinstance(particles, np.ndarray) and particles.dtype == np.float64
                and particles.flags.f_contiguous and particles.shape[0] == NFIELDS):
            raise TypeError("particles must be a Fortran-ordered float64 array of shape (46, maxparticles)")
        if np_ > particles.shape[1]:
            raise ValueError(f"np={np_} exceeds maxparticles={particles.shape[1]}")
        self._check(self._L.vpm_zeta(self._h, _ptr(particles), NFIELDS, int(np_), int(kernel), int(precision)))

    def zeta_dev(self, xt, xs, gs, sgs, W, kernel: int, precision: int):
        """W[nt,3] += sum_s zeta(r/sigma_s)/sigma_s^3 Gamma_s (device tensors)."""
        _check_dev(xt, 3); _check_dev(xs, 3); _check_dev(gs, 3); _check_dev(sgs, 1); _check_dev(W, 3)
        self._torch_stream()
        self._check(self._L.vpm_zeta_dev(self._h, xt.shape[0], _ptr(xt), xs.shape[0], _ptr(xs), _ptr(gs),
                                         _ptr(sgs), _ptr(W), int(kernel), int(precision)))

    def dynamic_diff_dev(self, x, gam, sig, J, alpha: float, dJ, dSFS, kernel: int, precision: int,
                         transposed: bool = True):
        """dJ = J(alpha sigma) - J(sigma), dSFS = SFS(alpha sigma; J + dJ) - SFS(sigma; J) (set, not added)."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(J, 9); _check_dev(dJ, 9)
        _check_dev(dSFS, 3)
        self._torch_stream()
        self._check(self._L.vpm_dynamic_diff_dev(self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(J),
                                                 float(alpha), _ptr(dJ), _ptr(dSFS), int(kernel), int(precision),
                                                 TRANSPOSED if transposed else 0))

    # ------------------------------------------- per-particle work of a step
    def rk3_stage_dev(self, a: float, b: float, dt: float, Uinf, f: float, g: float, zeta0: float, x, gam, sig,
                      U, J, M, *, SFS=None, C=None, nu: float | None = None, transposed: bool = True):
        """One stage of update_particle_states (+ core spreading with nu) on device tensors, in place."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(U, 3); _check_dev(J, 9)
        _check_dev(M, 9)
        if SFS is not None:
            _check_dev(SFS, 3); _check_dev(C, 3)
        ui = (ctypes.c_double * 3)(*[float(v) for v in Uinf])
        self._torch_stream()
        self._check(self._L.vpm_rk3_stage_dev(self._h, x.shape[0], float(a), float(b), float(dt), ui, float(f),
                                              float(g), float(zeta0), -1.0 if nu is None else float(nu),
                                              TRANSPOSED if transposed else 0, _ptr(x), _ptr(gam), _ptr(sig),
                                              _ptr(U), _ptr(J), _ptr(SFS), _ptr(C), _ptr(M)))

    def relax_dev(self, rlxf: float, J, gam):
        """relax_pedrizzetti on device tensors, gam in place."""
        _check_dev(J, 9); _check_dev(gam, 3)
        self._torch_stream()
        self._check(self._L.vpm_relax_dev(self._h, gam.shape[0], float(rlxf), _ptr(J), _ptr(gam)))

    def dynamic_after_dev(self, alpha: float, rlxf: float, minC: float, maxC: float, zeta0: float, gam, sig, J,
                          SFS, C, M, *, force_positive: bool = True, clip_backscatter: bool = True,
                          subtract: bool = False, transposed: bool = True):
        """dynamicprocedure_pseudo3level_afterUJ (+ clipping_backscatter) on device tensors: C and M in place.
        A NaN coefficient raises FloatingPointError, as the reference's error()."""
        _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(J, 9); _check_dev(SFS, 3); _check_dev(C, 3)
        _check_dev(M, 9)
        flags = ((TRANSPOSED if transposed else 0) | (DYN_FORCE_POSITIVE if force_positive else 0) |
                 (DYN_CLIP_BACKSCATTER if clip_backscatter else 0) | (DYN_SUBTRACT if subtract else 0))
        self._torch_stream()
        rc = self._L.vpm_dynamic_after_dev(self._h, gam.shape[0], float(alpha), float(rlxf), float(minC),
                                           float(maxC), float(zeta0), flags, _ptr(gam), _ptr(sig), _ptr(J),
                                           _ptr(SFS), _ptr(C), _ptr(M))
        if rc == ERR_NONFINITE:
            raise FloatingPointError("NaN in dynamicprocedure_pseudo3level_afterUJ")
        self._check(rc)

    def zeta_leaflist_dev(self, x, gam, sig, W, *, leaf_size: int = 64, theta: float = 0.4,
                          kernel: int = KERNEL_GAUSSIANERF, precision: int = FP64, reuse: bool = False):
        """zeta_fmm's near-field sum, W[n,3] += (CUDA float64 tensors); returns
        (leaves, leaf pairs, particle pairs).  reuse: VPM_REUSE_LISTS."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(W, 3)
        self._torch_stream()
        stats = np.zeros(3, dtype=np.int64)
        self._check(self._L.vpm_zeta_leaflist_dev(self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(W),
                                                  int(leaf_size), float(theta), int(kernel), int(precision),
                                                  REUSE_LISTS if reuse else 0, stats.ctypes.data))
        return tuple(int(v) for v in stats)

    def dynamic_diff_leaflist_dev(self, x, gam, sig, J, alpha: float, dJ, dSFS, *, leaf_size: int = 64,
                                  theta: float = 0.4, kernel: int = KERNEL_GAUSSIANERF, precision: int = FP32COMP,
                                  transposed: bool = True, static=None, reuse: bool = False):
        """dynamic_diff_dev over the near field of p2p_leaflist_dev (same leaf_size, theta; J the
        near-field J at sigma); dJ, dSFS set.  Returns (leaves, leaf pairs, particle pairs)."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(J, 9); _check_dev(dJ, 9)
        _check_dev(dSFS, 3)
        self._torch_stream()
        stats = np.zeros(3, dtype=np.int64)
        self._check(self._L.vpm_dynamic_diff_leaflist_dev(
            self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(static), _ptr(J), float(alpha), _ptr(dJ),
            _ptr(dSFS), int(leaf_size), float(theta), int(kernel), int(precision),
            (TRANSPOSED if transposed else 0) | (REUSE_LISTS if reuse else 0), stats.ctypes.data))
        return tuple(int(v) for v in stats)

    def uj_cross(self, src: np.ndarray, ns: int, tgt: np.ndarray, nt: int, kernel: int, precision: int):
        for m in (src, tgt):
            if not (isinstance(m, np.ndarray) and m.dtype == np.float64 and m.flags.f_contiguous
                    and m.shape[0] == NFIELDS):
                raise TypeError("matrices must be Fortran-ordered float64 arrays of shape (46, n)")
        self._check(self._L.vpm_uj_cross(self._h, _ptr(src), NFIELDS, int(ns), _ptr(tgt), NFIELDS,
                                         int(nt), int(kernel), int(precision)))

    # --------------------------------------------------- device-pointer API
    def _torch_stream(self):
        """Run on torch's current stream.  torch reports its default stream (the legacy
        default stream) as handle 0, which vpm_ctx_set_stream reads as "the context's own
        stream": pass cudaStreamLegacy (handle 1) for it instead."""
        import torch
        h = torch.cuda.current_stream().cuda_stream
        self.set_stream(h if h else CUDA_STREAM_LEGACY)

    def uj_dev(self, xt, xs, gs, sgs, U, J, kernel: int, precision: int):
        """U += and J += on CUDA float64 tensors x[n,3], gamma[n,3], sigma[n], U[n,3], J[n,9]."""
        _check_dev(xt, 3); _check_dev(xs, 3); _check_dev(gs, 3); _check_dev(sgs, 1)
        _check_dev(U, 3); _check_dev(J, 9)
        self._torch_stream()
        self._check(self._L.vpm_uj_dev(self._h, xt.shape[0], _ptr(xt), xs.shape[0], _ptr(xs), _ptr(gs),
                                       _ptr(sgs), _ptr(U), _ptr(J), int(kernel), int(precision)))

    def uj_adjoint_dev(self, x, gam, sig, Ubar, Jbar, xbar, gbar, sbar, kernel: int, precision: int = FP64):
        """xbar += dL/dx, gbar += dL/dGamma, sbar += dL/dsigma for dL/dU = Ubar, dL/dJ = Jbar."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(Ubar, 3); _check_dev(Jbar, 9)
        _check_dev(xbar, 3); _check_dev(gbar, 3); _check_dev(sbar, 1)
        self._torch_stream()
        self._check(self._L.vpm_uj_adjoint_dev(self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(Ubar),
                                               _ptr(Jbar), _ptr(xbar), _ptr(gbar), _ptr(sbar), int(kernel),
                                               int(precision)))

    def estr_adjoint_dev(self, x, gam, sig, J, Sbar, xbar, gbar, sbar, Jbar, kernel: int, precision: int = FP64,
                         transposed: bool = True, static=None):
        """vpm_estr_adjoint_dev: += dL/dx, dL/dGamma, dL/dsigma, dL/dJ of sum(Sbar * SFS)."""
        for t, c in ((x, 3), (gam, 3), (sig, 1), (J, 9), (Sbar, 3), (xbar, 3), (gbar, 3), (sbar, 1), (Jbar, 9)):
            _check_dev(t, c)
        self._torch_stream()
        self._check(self._L.vpm_estr_adjoint_dev(self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(J),
                                                 _ptr(static), _ptr(Sbar), _ptr(xbar), _ptr(gbar), _ptr(sbar),
                                                 _ptr(Jbar), int(kernel), int(precision),
                                                 TRANSPOSED if transposed else 0))

    def p2p_leaflist_dev(self, x, gam, sig, U, J, sfs_out=None, *, leaf_size: int = 64, theta: float = 0.4,
                         kernel: int = KERNEL_GAUSSIANERF, precision: int = FP32COMP, sfs: bool = False,
                         transposed: bool = True, static=None, reuse: bool = False):
        """Near-field P2P (UJ, and Estr into sfs_out with sfs=True) over octree leaf pairs;
        returns (leaves, leaf pairs, particle pairs)."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(U, 3); _check_dev(J, 9)
        if sfs:
            _check_dev(sfs_out, 3)
        self._torch_stream()
        stats = np.zeros(3, dtype=np.int64)
        flags = (SFS if sfs else 0) | (TRANSPOSED if transposed else 0) | (REUSE_LISTS if reuse else 0)
        self._check(self._L.vpm_p2p_leaflist_dev(self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(static),
                                                 _ptr(U), _ptr(J), _ptr(sfs_out) if sfs else None, int(leaf_size),
                                                 float(theta), int(kernel), int(precision), flags,
                                                 stats.ctypes.data))
        return tuple(int(v) for v in stats)

    def p2p_lists_dev(self, x, gam, sig, U, J, lists, sfs_out=None, *, kernel: int = KERNEL_GAUSSIANERF,
                      precision: int = FP32COMP, sfs: bool = False, transposed: bool = True, static=None):
        """Near-field P2P over caller-supplied host lists (perm, leaf_begin, leaf_end, row, col);
        returns (leaves, leaf pairs, particle pairs)."""
        _check_dev(x, 3); _check_dev(gam, 3); _check_dev(sig, 1); _check_dev(U, 3); _check_dev(J, 9)
        if sfs:
            _check_dev(sfs_out, 3)
        perm, lb, le, row, col = (np.ascontiguousarray(lists[0], np.int32), np.ascontiguousarray(lists[1], np.int64),
                                  np.ascontiguousarray(lists[2], np.int64), np.ascontiguousarray(lists[3], np.int64),
                                  np.ascontiguousarray(lists[4], np.int32))
        self._torch_stream()
        stats = np.zeros(3, dtype=np.int64)
        flags = (SFS if sfs else 0) | (TRANSPOSED if transposed else 0)
        self._check(self._L.vpm_p2p_lists_dev(self._h, x.shape[0], _ptr(x), _ptr(gam), _ptr(sig), _ptr(static),
                                              _ptr(U), _ptr(J), _ptr(sfs_out) if sfs else None, perm.ctypes.data,
                                              lb.shape[0], lb.ctypes.data, le.ctypes.data, row.ctypes.data,
                                              col.ctypes.data if col.size else None, int(kernel), int(precision),
                                              flags, stats.ctypes.data))
        return tuple(int(v) for v in stats)

    def leaflist_dev(self, x, leaf_size: int = 64, theta: float = 0.4):
        """The leaf-pair lists built on the GPU from device positions x[n,3]:
        (perm, leaf_begin, leaf_end, row, col, particle pairs)."""
        _check_dev(x, 3)
        self._torch_stream()
        n = x.shape[0]
        sizes = np.zeros(3, dtype=np.int64)
        self._check(self._L.vpm_leaflist_dev(self._h, n, _ptr(x), int(leaf_size), float(theta), None, None, None,
                                             None, None, sizes.ctypes.data))
        nl, nc = int(sizes[0]), int(sizes[1])
        perm = np.zeros(n, np.int32); lb = np.zeros(nl, np.int64); le = np.zeros(nl, np.int64)
        row = np.zeros(nl + 1, np.int64); col = np.zeros(max(nc, 1), np.int32)
        self._check(self._L.vpm_leaflist_dev(self._h, n, _ptr(x), int(leaf_size), float(theta), perm.ctypes.data,
                                             lb.ctypes.data, le.ctypes.data, row.ctypes.data, col.ctypes.data,
                                             sizes.ctypes.data))
        return perm, lb, le, row, col[:nc], int(sizes[2])

    def estr_dev(self, xt, Jt, xs, gs, sgs, Js, SFS, kernel: int, precision: int, transposed: bool = True,
                 static_t=None, static_s=None):
        _check_dev(xt, 3); _check_dev(Jt, 9); _check_dev(xs, 3); _check_dev(gs, 3); _check_dev(sgs, 1)
        _check_dev(Js, 9); _check_dev(SFS, 3)
        self._torch_stream()
        self._check(self._L.vpm_estr_dev(self._h, xt.shape[0], _ptr(xt), _ptr(Jt), _ptr(static_t),
                                         xs.shape[0], _ptr(xs), _ptr(gs), _ptr(sgs), _ptr(Js),
                                         _ptr(static_s), _ptr(SFS), int(kernel), int(precision),
                                         TRANSPOSED if transposed else 0))


def _check_dev(t, ncol: int):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise TypeError("expected a contiguous float64 CUDA tensor")
    if ncol > 1 and (t.dim() != 2 or t.shape[1] != ncol):
        raise TypeError(f"expected shape [n, {ncol}], got {tuple(t.shape)}")


_default_ctx: Context | None = None


def default_context() -> Context:
    """A process-wide context on CUDA device 0 (created on first use)."""
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
