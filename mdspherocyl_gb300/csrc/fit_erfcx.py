"""Coefficients of the erfc approximation in k_real.cu.

erfc(x) = exp(-x^2) * t * Q(t) with t = 1 / (1 + x/2).  Q is a degree-9
polynomial in t fitted to erfcx(x) / t by least squares weighted for
relative error, on Chebyshev nodes of the t interval that covers
0 <= x <= 9.5 (above x = 9.35, exp(-x^2) underflows FP32).  Prints the
FP32 coefficients (constant term first) and the largest relative error of
t * Q(t) against scipy's erfcx over that range.

    python mdspherocyl_gb300/csrc/fit_erfcx.py
"""
import numpy as np
from numpy.polynomial import Chebyshev, Polynomial
from scipy.special import erfcx

P, DEG, XMAX = 0.5, 9, 9.5


def q_exact(t):
    x = (1.0 / t - 1.0) / P
    return erfcx(x) / t


def main():
    tmin = 1.0 / (1.0 + P * XMAX)
    t = np.cos(np.linspace(0.0, np.pi, 8000)) * 0.5 * (1 - tmin) + 0.5 * (1 + tmin)
    q = q_exact(t)
    fit = Chebyshev.fit(t, q, DEG, domain=[tmin, 1.0], w=1.0 / q)
    coef = fit.convert(kind=Polynomial, domain=[-1, 1], window=[-1, 1]).coef.astype(np.float32)
    x = np.linspace(0.0, XMAX, 500001)
    tx = 1.0 / (1.0 + P * x)
    rel = np.abs(np.polyval(coef.astype(np.float64)[::-1], tx) / q_exact(tx) - 1.0).max()
    for k, c in enumerate(coef):
        print(f"kQ{k} = {c:.9e}f")
    print(f"max relative error on 0 <= x <= {XMAX}: {rel:.2e}")


if __name__ == "__main__":
    main()
