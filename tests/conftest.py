"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a GB300 (sm_103a) and the built libvpm_gb300.so; the
rest run on any CPU and use only the oracle, the host mirror and the library's
export table.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "flowvpm.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def ctx():
    """A libvpm_gb300 context on device 0 (GPU tests only)."""
    import vpm_gb300
    c = vpm_gb300.Context(0)
    yield c
    c.close()
