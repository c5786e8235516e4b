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
    import ctypes
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


def test_gaussianerf_series_coefficients():
    s = np.linspace(0.05, 2.0, 40)
    G, H = _gerf_exact(s)
    Gs = _horner(_coeffs("gerf_G_series"), s)
    Hs = _horner(_coeffs("gerf_H_series"), s)
    assert np.abs(Gs / G - 1).max() < 2e-8
    assert np.abs(Hs / H - 1).max() < 2e-8


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
