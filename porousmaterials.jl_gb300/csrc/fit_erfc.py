"""Derives the erfc approximation used by the Ewald real-space pair term (pmgb_kernels.cu).

erfc(x) = t * exp(-x^2) * Q(y),  t = 1 / (1 + x/2),  y = (t - t_mid) / t_half,
with Q a degree-7 polynomial fitted by Chebyshev least squares (relative weight) to
erfcx(x) / t over x in [0, 4] (t in [1/3, 1]).  The change of variable t follows the
classic erfc parameterisation of Numerical Recipes (erfcc); the fit and coefficients are
our own.  In FP32 with exact t the fit has max relative error 3.3e-7 on [0, 3.2] and
mean relative bias below 1e-8.  Run to print the constants pasted into the kernel.
"""
import numpy as np
from numpy.polynomial import chebyshev as Ch
from scipy.special import erfc, erfcx

X_MAX = 4.0
T_LO = 1.0 / (1.0 + X_MAX / 2.0)
T_MID = (1.0 + T_LO) / 2.0
T_HALF = (1.0 - T_LO) / 2.0
DEG = 7


def coefficients(deg: int = DEG) -> np.ndarray:
    n = 4000
    c = np.cos(np.pi * (np.arange(n) + 0.5) / n)           # Chebyshev nodes in y
    t = c * T_HALF + T_MID
    g = erfcx(2.0 * (1.0 / t - 1.0)) / t
    return Ch.cheb2poly(Ch.chebfit(c, g, deg, w=1.0 / g))  # monomial coefficients in y


def evaluate32(q: np.ndarray, x: np.ndarray) -> np.ndarray:
    x = x.astype(np.float32)
    t = (np.float32(1.0) / (np.float32(1.0) + np.float32(0.5) * x)).astype(np.float32)
    y = ((t - np.float32(T_MID)) * np.float32(1.0 / T_HALF)).astype(np.float32)
    h = np.zeros_like(y)
    for ck in q.astype(np.float32)[::-1]:
        h = (h * y + ck).astype(np.float32)
    return h.astype(np.float64) * t * np.exp(-x.astype(np.float64) ** 2)


if __name__ == "__main__":
    q = coefficients()
    xs = np.linspace(0.0, 3.2, 320001)
    rel = evaluate32(q, xs) / erfc(xs.astype(np.float32).astype(np.float64)) - 1.0
    print(f"t_mid = {np.float32(T_MID)!r}, 1/t_half = {np.float32(1.0 / T_HALF)!r}")
    print("coefficients (y^0 .. y^7):", ", ".join(f"{np.float32(c)!r}f" for c in q))
    print(f"max rel {np.abs(rel).max():.2e}, mean rel {rel.mean():+.2e}")
