"""Derives the polynomial coefficients of ptmath.cuh (portable FP32 sin, cos, asin).

The renderer evaluates the reference's sphere sampling (sin/cos/acos) with
these polynomials instead of the platform math library, so that the GPU and
the CPU oracle compute bit-identical paths. Method: least-squares fit in
float64 on Chebyshev nodes of the reduced interval (an approximation of the
minimax polynomial), coefficients rounded to FP32, evaluated by Horner's rule.

  sin(r) = r + r^3 * S(r^2),   cos(r) = 1 + r^2 * C(r^2),   |r| <= pi/4
  asin(x) = x + x^3 * A(x^2),  |x| <= 1/2

Run: python devilray_gb300/csrc/ptmath_coefficients.py
"""
from __future__ import annotations

import numpy as np


def cheb_nodes(a: float, b: float, n: int) -> np.ndarray:
    k = np.arange(n)
    return 0.5 * (a + b) + 0.5 * (b - a) * np.cos((2 * k + 1) * np.pi / (2 * n))


def fit(f_rest, lo: float, hi: float, degree: int, n: int = 4000) -> np.ndarray:
    """Coefficients c_0..c_degree of a polynomial in t = x^2 approximating f_rest(x)."""
    x = cheb_nodes(lo, hi, n)
    t = x * x
    y = f_rest(x)
    # relative weighting keeps the error uniform in ulps
    w = 1.0 / np.maximum(np.abs(y), 1e-300)
    A = np.vander(t, degree + 1, increasing=True) * w[:, None]
    c, *_ = np.linalg.lstsq(A, y * w, rcond=None)
    return c


def main():
    q = np.pi / 4
    # sin: (sin(r) - r) / r^3 as a polynomial in r^2
    S = fit(lambda x: (np.sin(x) - x) / x ** 3, 1e-4, q, 3)
    # cos: (cos(r) - 1) / r^2
    Cc = fit(lambda x: (np.cos(x) - 1.0) / x ** 2, 1e-4, q, 4)
    # asin: (asin(x) - x) / x^3
    A = fit(lambda x: (np.arcsin(x) - x) / x ** 3, 1e-4, 0.5, 6)
    for name, c in (("S", S), ("C", Cc), ("A", A)):
        print(name, ", ".join("%.9gf" % np.float32(v) for v in c))
    # Cody-Waite split of pi/2: hi part with 12 significant bits (k*hi exact)
    hi = np.float32(np.floor(np.pi / 2 * 2 ** 11) / 2 ** 11)
    mid = np.float32(np.pi / 2 - float(hi))
    lo = np.float32(np.pi / 2 - float(hi) - float(mid))
    print("PIO2", "%.9gf %.9gf %.9gf" % (hi, mid, lo))


if __name__ == "__main__":
    main()
