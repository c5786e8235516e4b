"""Generates the coefficients of the Gaussian-erf pair functions in vpm_math.cuh
(gerf_GQ).  Run by hand (numpy + scipy); its output is pasted into the header.

The Gaussian-erf kernel's g(rho) = erf(rho/sqrt2) - sqrt(2/pi) rho e^{-rho^2/2}
(src/FLOWVPM_kernel.jl:45-84) enters the pair term through, with s = rho^2,

    G(s) = g/rho^3,        -H(s)/3 = (G - c2 e/3)/s,      c2 = sqrt(2/pi), e = e^{-s/2}.

Two forms cover s >= 0 with one exponential:

* s < 2 -- Kummer's series erf(x) = (2/sqrt pi) e^{-x^2} sum_n 2^n x^{2n+1}/(2n+1)!!
  turns both into series of positive terms (no cancellation at small s):
      G = c2 e (1/3 + s S2(s)),   -H/3 = c2 e S2(s),   S2(s) = sum_m s^m/(2m+5)!!;
  ten terms reach 2e-9 of S2 at s = 2.
* s >= 2 -- g = 1 - e (erfcx(rho/sqrt2) + c2 rho), erfcx(x) = e^{x^2} erfc(x) being
  smooth there; erfcx(rho/sqrt2) (1 + rho/2) is fitted by a degree-7 polynomial in
  w = A t + B, t = 1/(1 + rho/2), over rho in [sqrt2, 10] (relative least squares on
  Chebyshev nodes).  Beyond rho = 10 the caller caps rho, since e < 2e-22 there and
  G equals its singular form s^-1.5.

The printed check is the worst relative error of the fit itself (double precision).
"""
import numpy as np
from scipy.special import erfcx

K = 0.5
DEG = 7
RHO_LO, RHO_HI = np.sqrt(2.0), 10.0


def fit():
    n = 4000
    x = np.cos(np.pi * (np.arange(n) + 0.5) / n)
    tlo, thi = 1 / (1 + K * RHO_HI), 1 / (1 + K * RHO_LO)
    t = tlo + (thi - tlo) * (x + 1) / 2
    rho = (1 / t - 1) / K
    y = erfcx(rho / np.sqrt(2)) * (1 + K * rho)
    tc, th = (thi + tlo) / 2, (thi - tlo) / 2
    V = np.vander((t - tc) / th, DEG + 1, increasing=True)
    c, *_ = np.linalg.lstsq(V / y[:, None], np.ones_like(y), rcond=None)
    return c, 1 / th, -tc / th


def main():
    c, A, B = fit()
    rho = np.linspace(RHO_LO, RHO_HI, 100001)
    t = 1 / (1 + K * rho)
    err = np.abs(np.polyval(c[::-1], A * t + B) * t / erfcx(rho / np.sqrt(2)) - 1).max()
    print(f"// w = {float(A)!r} t + {float(B)!r}; fit error {err:.2e}")
    for a in c[::-1]:
        print(f"    {float(a)!r}f,")
    d = 15.0
    print("// S2 series: 1/(2m+5)!!")
    for m in range(10):
        print(f"    {1.0 / d!r}f,")
        d *= 2 * m + 7


if __name__ == "__main__":
    main()
