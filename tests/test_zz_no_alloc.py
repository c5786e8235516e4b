"""vpm_uj_dev_noalloc -- the UJ entry point for callers that cannot allocate
device memory (their memory belongs to another allocator, or they must not
allocate once running).  It keeps its scratch in a static 64 MiB device array
instead of cudaMalloc'ed buffers; its results must equal those of the
allocating entry point vpm_uj_dev bit for bit, call after call, and the
oracle within the parity tolerance.

Named test_zz_* so pytest collects it last.  It creates its own inputs and
needs nothing from other test files, so it passes alone in a fresh process and
after the rest of the suite.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64, FP32COMP = 0, 1
TOL = {FP64: 1e-12, FP32COMP: 1e-6}


def _cloud(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(0, 0.3, (n, 3)), rng.normal(0, 1e-3, (n, 3)), rng.uniform(0.01, 0.03, n))


def _noalloc(L, xt, xs, gs, sgs, U, J, kernel, precision, stream):
    return L.vpm_uj_dev_noalloc(xt.shape[0], xt.data_ptr(), xs.shape[0], xs.data_ptr(), gs.data_ptr(),
                                sgs.data_ptr(), U.data_ptr(), J.data_ptr(), kernel, precision, stream)


def _normwise(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("precision", [FP64, FP32COMP])
@pytest.mark.parametrize("kernel", [2, 3])
@pytest.mark.parametrize("n", [3000, 40000])
def test_noalloc_matches_allocating_entry_point_twice(kernel, precision, n):
    """Both entry points run the same kernels with the same source-split rule
    (the split depends only on the sizes and the SM count), so the results are
    bit for bit equal, on the first call and on the second, which reuses the
    static scratch the first one left behind."""
    import torch
    import vpm_gb300
    L = vpm_gb300.load()
    ctx = vpm_gb300.Context(0)
    X, G, s = _cloud(n, seed=n + kernel)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    x, g, sg = d(X), d(G), d(s)
    Uref = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    Jref = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    ctx.uj_dev(x, x, g, sg, Uref, Jref, kernel, precision)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        U = torch.zeros_like(Uref)
        J = torch.zeros_like(Jref)
        rc = _noalloc(L, x, x, g, sg, U, J, kernel, precision, stream)
        assert rc == 0, L.vpm_last_error(None).decode()
        assert torch.equal(U, Uref), call
        assert torch.equal(J, Jref), call
    ctx.close()


@pytest.mark.parametrize("precision", [FP64, FP32COMP])
def test_noalloc_matches_the_oracle(precision):
    """One comparison against the FP64 CPU oracle (the reference's pair loop,
    src/FLOWVPM_fmm.jl:102-168), within the tolerance of the other parity tests."""
    import torch
    import oracle
    import vpm_gb300
    L = vpm_gb300.load()
    n = 2500
    X, G, s = _cloud(n, seed=11)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    x, g, sg = d(X), d(G), d(s)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    assert _noalloc(L, x, x, g, sg, U, J, 2, precision, torch.cuda.current_stream().cuda_stream) == 0
    Ur, Jr = oracle.uj_pairs(X, X, G, s, 2)
    assert np.abs(U.cpu().numpy() - Ur).max() / np.abs(Ur).max() <= TOL[precision]
    assert np.abs(J.cpu().numpy() - Jr).max() / np.abs(Jr).max() <= TOL[precision]


def test_noalloc_cross_targets_and_accumulation():
    import torch
    import vpm_gb300
    L = vpm_gb300.load()
    ctx = vpm_gb300.Context(0)
    Xs, Gs, ss = _cloud(5000, seed=1)
    Xt, _, _ = _cloud(777, seed=2)
    d = lambda a: torch.tensor(a, device="cuda", dtype=torch.float64).contiguous()
    xs, gs, sg, xt = d(Xs), d(Gs), d(ss), d(Xt)
    Uref = torch.ones(777, 3, device="cuda", dtype=torch.float64)
    Jref = torch.ones(777, 9, device="cuda", dtype=torch.float64)
    ctx.uj_dev(xt, xs, gs, sg, Uref, Jref, 2, FP32COMP)
    U = torch.ones_like(Uref)
    J = torch.ones_like(Jref)
    for _ in range(2):
        assert _noalloc(L, xt, xs, gs, sg, U, J, 2, FP32COMP, torch.cuda.current_stream().cuda_stream) == 0
    # the second call accumulated on top of the first (+= semantics, like vpm_uj_dev)
    assert _normwise(U - 1.0, 2.0 * (Uref - 1.0)) <= 1e-6
    assert _normwise(J - 1.0, 2.0 * (Jref - 1.0)) <= 1e-6
    ctx.close()


def test_noalloc_rejects_problems_beyond_the_static_scratch():
    import torch
    import vpm_gb300
    L = vpm_gb300.load()
    n = 1 << 21   # needs well over 64 MiB of scratch
    x = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    s = torch.ones(n, device="cuda", dtype=torch.float64)
    U = torch.zeros(n, 3, device="cuda", dtype=torch.float64)
    J = torch.zeros(n, 9, device="cuda", dtype=torch.float64)
    rc = _noalloc(L, x, x, x, s, U, J, 2, FP32COMP, None)
    assert rc == vpm_gb300._lib.ERR_CAPACITY
    msg = L.vpm_last_error(None).decode()
    assert "scratch" in msg and str(vpm_gb300._lib.NOALLOC_SCRATCH_BYTES) in msg
    # host pointers are rejected, nothing runs
    h = np.zeros((4, 3))
    rc = L.vpm_uj_dev_noalloc(4, h.ctypes.data, 4, h.ctypes.data, h.ctypes.data, h.ctypes.data,
                              h.ctypes.data, h.ctypes.data, 2, FP64, None)
    assert rc == vpm_gb300._lib.ERR_ARG
