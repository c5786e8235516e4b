"""Build libvpm_gb300.so (the GB300 UJ library) in-tree with nvcc for sm_103a.

    python flowvpm.jl_gb300/build.py [--verbose-ptxas]

Objects go to flowvpm.jl_gb300/_build/, the library to flowvpm.jl_gb300/lib/.
Translation units compile in parallel; the whole build takes well under a
minute.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libvpm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["uj.cu", "estr.cu", "order.cu", "adjoint.cu", "estr_adjoint.cu", "dynamic.cu", "nearfield.cu", "leaflist.cu", "step.cu", "tree.cpp",
           "abi.cu", "noalloc.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvpm_gb300.so")


def _needs(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, ptxas_verbose: bool = False, defines=(), lib: str = LIB,
          objdir: str = OBJ) -> str:
    """Compile (if stale) and link; `defines` are extra -D options (tuning
    variants), `lib`/`objdir` redirect the outputs."""
    os.makedirs(objdir, exist_ok=True)
    os.makedirs(os.path.dirname(os.path.abspath(lib)), exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "vpm_gb300.h"))
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "--expt-relaxed-constexpr"]
    if ptxas_verbose:
        flags += ["-Xptxas", "-v"]
    flags += ["-D" + d for d in defines]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or ptxas_verbose or defines or _needs(o, [s] + headers):
            jobs.append([cc] + flags + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True, errors="replace"), jobs))
    for cmd, r in zip(jobs, results):
        if ptxas_verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if force or jobs or not os.path.exists(lib):
        r = subprocess.run([cc] + ARCH + ["-shared", "-o", lib] + objs, capture_output=True, text=True,
                           errors="replace")
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("nvcc link of libvpm_gb300.so failed")
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    ap.add_argument("--define", action="append", default=[], help="extra -D for a tuning variant")
    ap.add_argument("--lib", default=LIB, help="output library path (default: lib/libvpm_gb300.so)")
    ap.add_argument("--objdir", default=OBJ)
    a = ap.parse_args()
    print(build(force=a.force, ptxas_verbose=a.verbose_ptxas, defines=a.define, lib=a.lib, objdir=a.objdir))
