"""The C ABI library loads and exports every symbol include/vpm_gb300.h declares
(CPU only: no compute calls), and the FP32 regular-form math of
csrc/vpm_math.cuh is checked against the reference formula in float64.
"""
import math
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vpm_gb300.h")
MATH = os.path.join(ROOT, "flowvpm.jl_gb300", "csrc", "vpm_math.cuh")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\**\s+\**(vpm_[a-z_0-9]+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    import vpm_gb300._lib as L
    if not os.path.exists(L.LIB_PATH):
        try:
            subprocess.run(["python", os.path.join(ROOT, "flowvpm.jl_gb300", "build.py")], check=True,
                           capture_output=True)
        except (OSError, subprocess.CalledProcessError) as e:
            pytest.skip(f"library not built and nvcc build failed: {e}")
    return L.load()


def test_header_declares_expected_entry_points():
    fns = header_functions()
    for f in ("vpm_ctx_create", "vpm_ctx_destroy", "vpm_last_error", "vpm_uj", "vpm_uj_cross",
              "vpm_uj_dev", "vpm_estr_dev"):
        assert f in fns


def test_library_exports_every_declared_symbol(lib):
    import vpm_gb300._lib as L
    for f in header_functions():
        assert hasattr(lib, f), f"libvpm_gb300.so does not export {f}"
        assert f in L.SIGNATURES, f"{f} has no ctypes signature in vpm_gb300._lib"


def test_work_constants_agree():
    """The flop-per-pair constants of the header are the ones the Python binding and the bench use."""
    import importlib.util
    import vpm_gb300._lib as L
    src = open(HEADER).read()
    defs = {k: int(v) for k, v in re.findall(r"#define\s+VPM_(FLOP_PER_\w+)\s+(\d+)", src)}
    assert defs == {"FLOP_PER_UJ_PAIR": 74, "FLOP_PER_ESTR_PAIR": 25, "FLOP_PER_UJ_ADJ_PAIR": 186}
    for k, v in defs.items():
        assert getattr(L, k) == v, k
    spec = importlib.util.spec_from_file_location("bench_consts", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.FLOP_PER_PAIR == defs["FLOP_PER_UJ_PAIR"]
    assert bench.FLOP_PER_ADJ_PAIR == defs["FLOP_PER_UJ_ADJ_PAIR"]


def test_abi_version_and_build_info(lib):
    assert lib.vpm_abi_version() == 1
    assert b"sm_103a" in lib.vpm_build_info()


def test_context_creation_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import vpm_gb300
    with pytest.raises(vpm_gb300.VPMError) as ei:
        vpm_gb300.Context(0)
    assert ei.value.code == vpm_gb300._lib.ERR_NODEVICE


def test_null_context_is_an_argument_error(lib):
    assert lib.vpm_uj(None, None, 46, 0, 2, 0, 1) == -1
    assert lib.vpm_ctx_create(None, 0) == -1
    assert lib.vpm_ctx_destroy(None) == 0


# ----------------------------------------------------------- FP32 math design
def _coeffs(name):
    src = open(MATH).read()
    body = re.search(name + r"\(float \w\)\s*\{(.*?)return", src, flags=re.S).group(1)
    nums = re.findall(r"([-+]?\d[\d.]*e?[-+]?\d*)f", body)
    return [float(x) for x in nums]  # highest degree first


def _horner(c, s):
    p = c[0]
    for a in c[1:]:
        p = p * s + a
    return p


def _gerf_exact(s):
    from scipy.special import erf
    rho = np.sqrt(s)
    c2 = math.sqrt(2 / math.pi)
    g = erf(rho / math.sqrt(2)) - c2 * rho * np.exp(-s / 2)
    G = g / rho ** 3
    H = (c2 * np.exp(-s / 2) - 3 * G) / s
    return G, H


def _kummer(s, first, terms=300):
    """sum_m s^m / (2m + first)!! in double (positive terms)."""
    out = np.zeros_like(s)
    t = np.full_like(s, 1.0 / math.prod(range(first, 0, -2)))
    for m in range(terms):
        out += t
        t = t * s / (2 * m + first + 2)
    return out


def _body(path, head, stop):
    src = open(path).read()
    i = src.index(head)
    return src[i:src.index(stop, i)]


def _poly(body, var):
    c0 = re.search(r"float p = ([-+\d.e]+)f;", body).group(1)
    rest = re.findall(r"p = fmaf\(p, " + var + r", ([-+\d.e]+)f\);", body)
    return [float(c0)] + [float(x) for x in rest]   # highest degree first


def _erfcx_fit():
    body = _body(MATH, "float gerf_G_erfcx(", "return fmaf")
    A, B = (float(v) for v in re.search(r"w = fmaf\(([-+\d.e]+)f, t, ([-+\d.e]+)f\)", body).groups())
    return A, B, _poly(body, "w")


def test_gaussianerf_positive_series():
    """gerf_GQ below s = 2: G = c2 e (1/3 + s S2), -H/3 = c2 e S2 with
    S2 = sum s^m/(2m+5)!! (Kummer's series of erf), against the erf closed form."""
    pytest.importorskip("scipy")
    s = np.linspace(0.05, 2.0, 60)
    G, H = _gerf_exact(s)
    S2 = _horner(_poly(_body(MATH, "if (s < S_SERIES) {", "const float ce"), "s"), s)
    ce = math.sqrt(2 / math.pi) * np.exp(-s / 2)
    assert np.abs(ce * (1 / 3 + s * S2) / G - 1).max() < 2e-9
    assert np.abs(-3 * ce * S2 / H - 1).max() < 2e-9


def test_gaussianerf_erfcx_fit():
    """gerf_G_erfcx for s >= 2: g = 1 - e (erfcx(rho/sqrt2) + c2 rho), erfcx from
    the degree-7 fit in w = A t + B, t = 1/(1 + rho/2), rho capped at 10."""
    pytest.importorskip("scipy")
    A, B, c = _erfcx_fit()
    s = np.concatenate([np.linspace(2.0, 50.0, 2000), np.linspace(50.0, 400.0, 200)])
    rho = np.sqrt(s)
    t = 1 / (1 + 0.5 * np.minimum(rho, 10.0))
    h = _horner(c, A * t + B) * t + math.sqrt(2 / math.pi) * rho
    G = (1 - np.exp(-s / 2) * h) / rho ** 3
    Gx, _ = _gerf_exact(s)
    assert np.abs(G / Gx - 1).max() < 2e-8


def test_gaussianerf_fp32_design_error():
    """The whole gerf_GQ evaluated with FP32 rounding after every operation
    (correctly rounded exp, rsqrt and reciprocal): worst relative error of G and
    Q over 0 < s <= 120 within 5e-7 and 1.2e-6 -- the bound of the closed
    form with a correctly rounded erf, set by the FP32 rounding of s^-1.5."""
    r = lambda x: np.asarray(x, np.float64).astype(np.float32).astype(np.float64)
    fma = lambda a, b, c: r(np.asarray(a) * np.asarray(b) + np.asarray(c))
    mul = lambda a, b: r(np.asarray(a) * np.asarray(b))
    c2 = math.sqrt(2 / math.pi)
    cs = _poly(_body(MATH, "if (s < S_SERIES) {", "const float ce"), "s")
    A, B, cw = _erfcx_fit()
    s = r(np.concatenate([np.linspace(1e-4, 2.0, 4001), np.linspace(2.0, 120.0, 40001)]))
    e = r(np.exp(-s / 2))
    p = np.full_like(s, r(cs[0]))
    for a in cs[1:]:
        p = fma(p, s, r(a))
    Gs, Qs = mul(mul(c2, e), fma(s, p, 1 / 3)), mul(mul(c2, e), p)
    rs = r(1 / np.sqrt(s))
    rs2 = mul(rs, rs)
    rho = mul(s, rs)
    t = r(1 / fma(0.5, np.minimum(rho, 10.0), 1.0))
    w = fma(A, t, B)
    q = np.full_like(s, r(cw[0]))
    for a in cw[1:]:
        q = fma(q, w, r(a))
    h = fma(c2, rho, mul(q, t))
    Gm = mul(mul(fma(-e, h, 1.0), rs), rs2)
    Qm = mul(fma(-c2 / 3, e, Gm), rs2)
    G, Q = np.where(s < 2, Gs, Gm), np.where(s < 2, Qs, Qm)
    Ge = c2 * np.exp(-s / 2) * _kummer(s, 3)
    Qe = c2 * np.exp(-s / 2) * _kummer(s, 5)
    assert np.abs(G / Ge - 1).max() < 5e-7
    assert np.abs(Q / Qe - 1).max() < 1.2e-6


def test_adjoint_S3_series():
    """The adjoint's K(s) = 15 c2 e S3(s), S3 = sum s^m/(2m+7)!!, below s = 6,
    against K = (15 G - c2 e (5 + s))/s^2 from the erf closed form."""
    pytest.importorskip("scipy")
    adj = os.path.join(ROOT, "flowvpm.jl_gb300", "csrc", "adjoint.cu")
    c = _poly(_body(adj, "float gerf_S3_series(", "return p;"), "s")
    s = np.linspace(0.5, 6.0, 40)
    G, _ = _gerf_exact(s)
    e = math.sqrt(2 / math.pi) * np.exp(-s / 2)
    K = (15 * G - e * (5 + s)) / s ** 2
    assert np.abs(15 * e * _horner(c, s) / K - 1).max() < 1e-8


def test_gaussian_series_coefficients():
    t = np.linspace(0.01, 1.0, 30)
    e = np.exp(-t)
    assert np.abs(_horner(_coeffs("gaus_G_series"), t) / ((1 - e) / t) - 1).max() < 1e-9
    assert np.abs(_horner(_coeffs("gaus_H_series"), t) / ((t * e - 1 + e) / t ** 2) - 1).max() < 1e-9


def test_far_field_cutoffs_are_below_fp32_resolution():
    # Gaussian-erf: for s > 50 the singular form differs by < 2e-9 relative
    src = open(MATH).read()
    s_far = float(re.search(r"S_FAR_GERF = ([\d.]+)f", src).group(1))
    G, H = _gerf_exact(np.array([s_far]))
    assert abs(G[0] * s_far ** 1.5 - 1) < 2e-9 and abs(H[0] / (-3 * s_far ** -2.5) - 1) < 2e-9
    # Gaussian: for s > 8 (t = rho^3 > 22.6)
    t = 8.0 ** 1.5
    e = math.exp(-t)
    assert abs((1 - e) - 1) < 1e-9 and abs(3 * (t * e - 1 + e) / -3 - 1) < 1e-8


def test_dynamic_ratio_series():
    """dyn_math.cuh's e^x - 1 and log(1 + x) series (used for |x| <= 1/8 in the
    dynamic procedure's weight ratio) against numpy: < 1e-10 relative."""
    dyn = os.path.join(ROOT, "flowvpm.jl_gb300", "csrc", "dyn_math.cuh")
    x = np.linspace(-0.125, 0.125, 4001)
    x = x[x != 0]
    for head, ref in (("float expm1_small(", np.expm1), ("float log1p_small(", np.log1p)):
        body = _body(dyn, head, "return p * x")
        c = [float(re.search(r"float p = ([-+\d.e]+)f;", body).group(1))]
        c += [float(v) for v in re.findall(r"p = fmaf\(p, x, ([-+\d.e]+)f\);", body)]
        assert np.abs(_horner(c, x) * x / ref(x) - 1).max() < 1e-10, head
