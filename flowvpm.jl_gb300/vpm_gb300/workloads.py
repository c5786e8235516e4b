"""Seeded synthetic particle sets for the UJ workloads (the reference names no
public dataset; all inputs are generated here).

* random_cloud      -- X ~ U[0,1]^3, Gamma ~ N(0, 1e-3) i.i.d., sigma ~ U[0.01, 0.03]
* isolated_ring     -- R=1, Gamma=1, a=0.1R, Nphi=200 x 7 per section, sigma=a/2
* leapfrog_rings    -- rings R=1 and R=0.7, 0.3R apart axially, Gamma=1 each,
                       a=0.1R, 10 per section, sigma=a/2 (~200k particles)
* rollout_ring      -- the isolated ring at Nphi=1000 x 32 per section (32k)
* jet_cloud         -- particles uniform in a cylinder (radius 0.5, length 4)
                       with Gamma = vol * omega(x), omega = curl A of a seeded
                       random Fourier field A with a Gaussian spectrum (so omega
                       is solenoidal), sigma = 0.02

Every function returns (X[n,3], Gamma[n,3], sigma[n]) as float64 numpy arrays.
"""
from __future__ import annotations

import math

import numpy as np

from . import rings


def random_cloud(n: int, seed: int = 0, gamma_std: float = 1e-3, sig_lo: float = 0.01, sig_hi: float = 0.03):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 1.0, (n, 3)), rng.normal(0.0, gamma_std, (n, 3)), rng.uniform(sig_lo, sig_hi, n)


def isolated_ring(nphi: int = 200, nper: int = 7, R: float = 1.0, circulation: float = 1.0):
    a = 0.1 * R
    X, G, s, _ = rings.ring_sections(circulation, R, a, nphi, nper, a / 2)
    return X, G, s


def rollout_ring(nphi: int = 1000, nper: int = 32):
    return isolated_ring(nphi, nper)


def leapfrog_rings(total: int = 200_000, nper: int = 10):
    """Two coaxial rings (R=1 at z=0 and R=0.7 at z=0.3), equal section counts."""
    nphi = max(1, total // (2 * nper))
    X1, G1, s1, _ = rings.ring_sections(1.0, 1.0, 0.1, nphi, nper, 0.05)
    X2, G2, s2, _ = rings.ring_sections(1.0, 0.7, 0.07, nphi, nper, 0.035, O=(0.0, 0.0, 0.3))
    return np.vstack([X1, X2]), np.vstack([G1, G2]), np.concatenate([s1, s2])


def jet_cloud(n: int = 1 << 20, seed: int = 0, radius: float = 0.5, length: float = 4.0, sigma: float = 0.02,
              modes: int = 64, k0: float = 8.0, amp: float = 1.0):
    """Uniform particles in the cylinder r <= radius, 0 <= z <= length, with
    Gamma_p = vol * curl A(x_p),  A(x) = sum_m a_m cos(k_m . x + phi_m),
    k_m ~ N(0, k0^2 I) (Gaussian spectrum), a_m ~ N(0, amp^2 I) / sqrt(modes)."""
    rng = np.random.default_rng(seed)
    r = radius * np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * math.pi, n)
    X = np.stack([r * np.cos(th), r * np.sin(th), rng.uniform(0, length, n)], axis=1)
    k = rng.normal(0, k0, (modes, 3))
    a = rng.normal(0, amp, (modes, 3)) / math.sqrt(modes)
    phi = rng.uniform(0, 2 * math.pi, modes)
    kxa = np.cross(k, a)                                   # curl of a cos(k.x+phi) = -(k x a) sin(k.x+phi)
    W = np.zeros((n, 3))
    for c in range(0, n, 1 << 16):                         # chunked to bound memory
        ph = X[c:c + (1 << 16)] @ k.T + phi                # [chunk, modes]
        W[c:c + (1 << 16)] = -np.sin(ph) @ kxa
    vol = math.pi * radius * radius * length / n
    return X, vol * W, np.full(n, sigma)
