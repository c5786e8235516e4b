"""Shared input generators and error metrics for the tests."""
import numpy as np

NFIELDS = 46


def random_cloud(n, seed=0, gamma_std=1e-3, sig_lo=0.01, sig_hi=0.03, box=1.0):
    """The random-cloud workload: X ~ U[0,box]^3, Gamma ~ N(0, gamma_std) i.i.d.,
    sigma ~ U[sig_lo, sig_hi] (numpy PCG64, seeded)."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(0.0, box, size=(n, 3))
    G = rng.normal(0.0, gamma_std, size=(n, 3))
    s = rng.uniform(sig_lo, sig_hi, size=n)
    return X, G, s


def matrix_of(X, G, s, static=None, extra=0, seed=None):
    """Fortran-ordered (46, n+extra) particle matrix with X, Gamma, sigma (and
    optional static flags); other rows random when `seed` is given, so resets
    and accumulation are visible."""
    n = X.shape[0]
    P = np.zeros((NFIELDS, n + extra), order="F")
    if seed is not None:
        rng = np.random.default_rng(seed)
        P[:, :n] = rng.normal(size=(NFIELDS, n))
    P[0:3, :n] = X.T
    P[3:6, :n] = G.T
    P[6, :n] = s
    P[42, :n] = 0.0 if static is None else np.asarray(static, dtype=float)
    return P


def normwise(err_ref, ref):
    """(max |err| / max |ref|, ||err||_2 / ||ref||_2) over all entries."""
    err = np.asarray(err_ref, dtype=float) - np.asarray(ref, dtype=float)
    ref = np.asarray(ref, dtype=float)
    mx = np.abs(ref).max()
    nrm = np.linalg.norm(ref)
    return (np.abs(err).max() / mx if mx > 0 else np.abs(err).max(),
            np.linalg.norm(err) / nrm if nrm > 0 else np.linalg.norm(err))
