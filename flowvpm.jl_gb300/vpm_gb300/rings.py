"""Vortex-ring particle generators and ring diagnostics.

* `addvortexring` restates examples/vortexrings/vortexrings_functions.jl:73-227
  for circular rings (aspect ratio 1).  For a circle the reference's elliptic
  arc length is a*phi and its cell volumes, integrated there with HCubature to
  rtol 1e-8, have the closed form
      vol = dphi * [R (r2^2 - r1^2)/2 (th2 - th1) + (r2^3 - r1^3)/3 (sin th2 - sin th1)],
  which is used here.  Particle counts are Nphi*(1 + 8*sum(1:nc)).
* `ring_sections` is this library's generator for n particles per cross
  section (7, 10, 32, ...), which the reference's layered generator cannot
  produce: cross-section points on a sunflower (Vogel) spiral of equal-area
  cells, each particle carrying omega * cell volume along the ring tangent,
  omega = circulation / (pi a^2).
* `Uring` (vortexrings_functions.jl:47) and `calc_rings_weighted`
  (:275-315) are the reference's analytic ring speed and strength-weighted ring
  centroid / radius.
* `analytic_coaxialrings` restates the reference's reference solution for
  coaxial rings (examples/vortexrings/vortexrings_postprocessing.jl:110-320):
  the thin-ring ODEs of Borisov, Kilin & Mamaev (2013), "The dynamics of vortex
  rings: leapfrogging, choreographies and the stability problem", integrated
  by forward Euler with its step, its one-sided differences of the stream
  function and its elliptic integrals K(k), E(k) of parameter k^2.
"""
from __future__ import annotations

import math

import numpy as np

from .particlefield import ParticleField


def Uring(circulation: float, R: float, Rcross: float, beta: float) -> float:
    """Analytic self-induced velocity of an inviscid ring."""
    return circulation / (4 * math.pi * R) * (math.log(8 * R / Rcross) - beta)


def number_particles(Nphi: int, nc: int, extra_nc: int = 0) -> int:
    return int(Nphi * (1 + 8 * sum(range(1, nc + extra_nc + 1))))


def _frame(phic: float):
    """Ring-centre point and local axes of a circular ring of unit radius at angle phic."""
    T = np.array([math.cos(phic), -math.sin(phic), 0.0])
    T = -T / np.linalg.norm(T)                       # flip so +circulation travels +Z
    zvec = np.array([0.0, 0.0, 1.0])
    return T, np.cross(zvec, T), zvec


def addvortexring(pfield: ParticleField, circulation: float, R: float, AR: float, Rcross: float,
                  Nphi: int, nc: int, sigma: float, *, extra_nc: int = 0, O=(0.0, 0.0, 0.0), Oaxis=None):
    """Add a circular vortex ring the way the reference's addvortexring does (AR == 1 only)."""
    if AR < 1:
        raise ValueError(f"Invalid aspect ratio AR < 1 (AR = {AR})")
    if AR != 1:
        raise NotImplementedError("only circular rings (AR = 1) are restated")
    O = np.asarray(O, dtype=np.float64)
    Oaxis = np.eye(3) if Oaxis is None else np.asarray(Oaxis, dtype=np.float64)
    rl = Rcross / (2 * nc + 1)
    dphi = 2 * math.pi / Nphi
    omega = circulation / (math.pi * Rcross ** 2)
    Xs, Gs, sg, vols, circs = [], [], [], [], []

    def vol(r1, t1, r2, t2):
        return dphi * (R * (r2 ** 2 - r1 ** 2) / 2 * (t2 - t1) + (r2 ** 3 - r1 ** 3) / 3 * (math.sin(t2) - math.sin(t1)))

    def length(r, th):
        return (R + r * math.cos(th)) * dphi

    for N in range(Nphi):
        phic = 2 * math.pi * (N + 0.5) / Nphi
        Xc = np.array([R * math.sin(phic), R * math.cos(phic), 0.0])
        T, ax2, ax3 = _frame(phic)
        for n in range(nc + extra_nc + 1):
            if n == 0:
                v = vol(0.0, 0.0, rl, 2 * math.pi)
                G = omega * v * T
                Xs.append(Xc); Gs.append(G); vols.append(v)
                circs.append(np.linalg.norm(G) / length(0.0, 0.0))
            else:
                rc = (1 + 12 * n * n) / (6 * n) * rl
                r1, r2 = (2 * n - 1) * rl, (2 * n + 1) * rl
                ncells = 8 * n
                dth = 2 * math.pi / ncells
                for j in range(ncells):
                    t1, t2 = dth * j, dth * (j + 1)
                    tc = (t1 + t2) / 2
                    v = vol(r1, t1, r2, t2)
                    X = Xc + rc * math.cos(tc) * ax2 + rc * math.sin(tc) * ax3
                    G = omega * v * T if n <= nc else np.finfo(float).eps * T
                    Xs.append(X); Gs.append(G); vols.append(v)
                    circs.append(np.linalg.norm(G) / length(rc, tc))
    X = np.array(Xs) @ Oaxis.T + O
    G = np.array(Gs) @ Oaxis.T
    pfield.add_particles(X, G, np.full(len(Xs), sigma), vol=np.array(vols), circulation=np.array(circs))


def ring_sections(circulation: float, R: float, a: float, Nphi: int, n_per_section: int, sigma: float,
                  O=(0.0, 0.0, 0.0)):
    """Particles (X[n,3], Gamma[n,3], sigma[n], vol[n]) of a circular ring in the z=O_z plane,
    n_per_section particles per cross section on an equal-area sunflower spiral."""
    golden = math.pi * (3 - math.sqrt(5))
    k = np.arange(n_per_section)
    rk = a * np.sqrt((k + 0.5) / n_per_section)
    tk = k * golden
    dphi = 2 * math.pi / Nphi
    omega = circulation / (math.pi * a * a)
    cell_area = math.pi * a * a / n_per_section
    phic = 2 * math.pi * (np.arange(Nphi) + 0.5) / Nphi
    Xc = np.stack([R * np.sin(phic), R * np.cos(phic), np.zeros(Nphi)], axis=1)      # [Nphi,3]
    T = np.stack([-np.cos(phic), np.sin(phic), np.zeros(Nphi)], axis=1)                # tangent
    radial = np.stack([np.sin(phic), np.cos(phic), np.zeros(Nphi)], axis=1)            # outward
    zhat = np.array([0.0, 0.0, 1.0])
    X = (Xc[:, None, :] + (rk * np.cos(tk))[None, :, None] * radial[:, None, :]
         + (rk * np.sin(tk))[None, :, None] * zhat[None, None, :])
    vol = np.broadcast_to(cell_area * (R + rk * np.cos(tk)) * dphi, (Nphi, n_per_section))  # Pappus
    G = omega * vol[:, :, None] * T[:, None, :]
    X = X.reshape(-1, 3) + np.asarray(O, dtype=np.float64)
    return X, G.reshape(-1, 3), np.full(X.shape[0], float(sigma)), vol.reshape(-1)


def calc_rings_weighted(pfield: ParticleField, intervals):
    """Strength-weighted centroid, ring radius and core size of each ring,
    examples/vortexrings/vortexrings_functions.jl:275-315.  intervals = [0, n1, n1+n2, ...]."""
    out = []
    X = pfield.X
    G = pfield.Gamma
    s = pfield.sigma
    for ri in range(len(intervals) - 1):
        sl = slice(intervals[ri], intervals[ri + 1])
        nG = np.sqrt((G[sl] ** 2).sum(axis=1))
        tot = nG.sum()
        Z = (X[sl] * nG[:, None]).sum(axis=0) / tot
        Rr = (nG * np.sqrt(((X[sl] - Z) ** 2).sum(axis=1))).sum() / tot
        sg = (nG * s[sl]).sum() / tot
        out.append((Z, Rr, sg))
    return out


def _stream_G(z, r, zt, rt):
    """Stokes stream function of a thin ring of unit circulation at (zt, rt),
    evaluated at (z, r) (vortexrings_postprocessing.jl:308-314)."""
    from scipy.special import ellipe, ellipk
    k = math.sqrt(4 * r * rt / ((z - zt) ** 2 + (r + rt) ** 2))
    return math.sqrt(r * rt) / (2 * math.pi) * ((2 / k - k) * ellipk(k * k) - 2 / k * ellipe(k * k))


def analytic_coaxialrings(Gammas, Rs, Zs, As, Deltas, *, tend: float, dtmax: float = 1e-3,
                          dynamica: bool = True):
    """Radii and centroids of coaxial thin rings at time tend (and every step):
    dZ_i/dt = Gamma_i/(4 pi R_i) (ln(8 R_i/a_i) - 1/2 + Delta_i) + 1/R_i sum_j Gamma_j dG/dR_i,
    dR_i/dt = -1/R_i sum_j Gamma_j dG/dZ_i,   da_i/dt = -a_i/(2 R_i) dR_i/dt (dynamica),
    by forward Euler with step dtmax/10 and the last step cut to end at tend;
    dG/d. by forward differences with h = 1e-5.  Returns (t, R[nt, nrings], Z[nt, nrings])."""
    h = 1e-5
    nr = len(Rs)
    R = np.array(Rs, dtype=np.float64)
    Z = np.array(Zs, dtype=np.float64)
    a = np.array(As, dtype=np.float64)
    Gam = np.array(Gammas, dtype=np.float64)
    Dl = np.array(Deltas, dtype=np.float64)
    dt = dtmax / 10
    t = list(np.arange(0.0, tend + dt / 2, dt))      # the range (0 : dt : tend)
    if t[-1] > tend:
        t.pop()
    if t[-1] != tend:
        t.append(tend)
    Rh, Zh = [R.copy()], [Z.copy()]
    for k in range(1, len(t)):
        step = t[k] - t[k - 1]
        dR = np.zeros(nr)
        dZ = Gam / (4 * math.pi * R) * (np.log(8 * R / a) - 0.5 + Dl)
        for i in range(nr):
            for j in range(nr):
                if i == j:
                    continue
                g0 = _stream_G(Z[i], R[i], Z[j], R[j])
                dGdZ = (_stream_G(Z[i] + h, R[i], Z[j], R[j]) - g0) / h
                dGdR = (_stream_G(Z[i], R[i] + h, Z[j], R[j]) - g0) / h
                dR[i] -= 1 / R[i] * Gam[j] * dGdZ
                dZ[i] += 1 / R[i] * Gam[j] * dGdR
        da = -a / (2 * R) * dR if dynamica else np.zeros(nr)
        R = R + dR * step
        Z = Z + dZ * step
        a = a + da * step
        Rh.append(R.copy())
        Zh.append(Z.copy())
    return np.array(t), np.array(Rh), np.array(Zh)
