"""Ewald-sum set-up (host side).

Mirrors determine_ewald_params (src/electrostatics.jl:123-141), required_kreps (:157-175),
precompute_kvec_wts (:198-232) and setup_Ewald_sum (:256-272).  The roots of the two
precision conditions are found by bisection to machine precision, as a bracketing
fzero does.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .crystal import Box

EPS0 = 8.854187817e-12 / (1.602176565e-19 ** 2) / 1.0e10 * 1.3806488e-23  # e²/(Å K), electrostatics.jl:6
FOUR_PI_EPS0 = 4.0 * math.pi * EPS0


@dataclass
class EwaldParams:
    kreps: tuple[int, int, int]
    alpha: float
    sr_cutoff_r: float
    kvec_abc: np.ndarray  # (n_k, 3) int32
    kvec_wt: np.ndarray   # (n_k,) float64

    @property
    def n_kvecs(self) -> int:
        return int(self.kvec_wt.shape[0])


def _bisect(f, lo: float, hi: float) -> float:
    flo = f(lo)
    for _ in range(2000):
        mid = 0.5 * (lo + hi)
        if mid <= lo or mid >= hi:
            break
        fm = f(mid)
        if fm == 0.0:
            return mid
        if (fm > 0.0) == (flo > 0.0):
            lo, flo = mid, fm
        else:
            hi = mid
    return 0.5 * (lo + hi)


def determine_ewald_params(sr_cutoff_r: float, eps: float) -> tuple[float, float]:
    alpha = _bisect(lambda a: math.erfc(sr_cutoff_r * a) / sr_cutoff_r - eps, 0.0, 25.0)

    def lr(k2):
        if k2 == 0.0:
            return math.inf
        return 2.0 * math.exp(-k2 / (4.0 * alpha * alpha)) / k2 - eps

    return alpha, _bisect(lr, 0.0, 100.0)


def required_kreps(box: Box, max_mag_k_sqrd: float) -> tuple[int, int, int]:
    kreps = [0, 0, 0]
    for abc in range(3):
        n = 0
        while True:
            n += 1
            k = box.reciprocal_lattice[abc, :] * n
            if float(np.dot(k, k)) > max_mag_k_sqrd:
                kreps[abc] = n - 1
                break
    return kreps[0], kreps[1], kreps[2]


def precompute_kvec_wts(kreps, box: Box, alpha: float, max_mag_k_sqrd: float = math.inf):
    """k-vectors of the half space (ka >= 0 with the tie rules) with |k|² < max and their
    weights 2 exp(-k²/4α²) / k² / ε₀ / Ω."""
    ka = np.arange(0, kreps[0] + 1)
    kb = np.arange(-kreps[1], kreps[1] + 1)
    kc = np.arange(-kreps[2], kreps[2] + 1)
    A, B, Cc = np.meshgrid(ka, kb, kc, indexing="ij")  # kc fastest, then kb, then ka
    abc = np.stack([A.ravel(), B.ravel(), Cc.ravel()], axis=1)
    keep = ~((abc[:, 0] == 0) & (abc[:, 1] == 0) & (abc[:, 2] == 0))
    keep &= ~((abc[:, 0] == 0) & (abc[:, 1] < 0))
    keep &= ~((abc[:, 0] == 0) & (abc[:, 1] == 0) & (abc[:, 2] < 0))
    abc = abc[keep]
    k = abc.astype(np.float64) @ box.reciprocal_lattice  # rows: transpose(recip) * n
    k2 = np.einsum("ij,ij->i", k, k)
    sel = k2 < max_mag_k_sqrd
    abc, k2 = abc[sel], k2[sel]
    wt = 2.0 * np.exp(-k2 / (4.0 * alpha * alpha)) / k2 / EPS0 / box.Omega
    return np.ascontiguousarray(abc, dtype=np.int32), np.ascontiguousarray(wt, dtype=np.float64)


def setup_Ewald_sum(box: Box, sr_cutoff_r: float, eps: float = 1e-6, verbose: bool = False) -> EwaldParams:
    """setup_Ewald_sum (src/electrostatics.jl:256-272) through the library's native set-up
    (pmgb_ewald_setup): the steps of determine_ewald_params, required_kreps and
    precompute_kvec_wts above, in C++, so that a screening loop does not pay interpreter time per
    framework.  The library is loaded for this host-only call; no device work is done."""
    import ctypes as C

    from ._lib import PMGBError, lib

    L = lib()
    f = np.ascontiguousarray(box.f_to_c.T.reshape(-1))  # column-major
    fp = f.ctypes.data_as(C.POINTER(C.c_double))
    n = C.c_int64(0)
    rc = L.pmgb_ewald_setup(fp, float(sr_cutoff_r), float(eps), 0, None, None, None, C.byref(n), None, None)
    if rc != 0:
        raise PMGBError(rc, "pmgb_ewald_setup: the box must be non-singular, the cutoff positive and the precision "
                            "in (0, 1)")
    abc = np.zeros((n.value, 3), dtype=np.int32)
    wt = np.zeros(n.value, dtype=np.float64)
    alpha, kr = C.c_double(0.0), (C.c_int32 * 3)()
    rc = L.pmgb_ewald_setup(fp, float(sr_cutoff_r), float(eps), n.value, C.byref(alpha), None, kr, C.byref(n),
                            abc.ctypes.data_as(C.POINTER(C.c_int32)), wt.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise PMGBError(rc, "pmgb_ewald_setup failed")
    kreps = (int(kr[0]), int(kr[1]), int(kr[2]))
    ep = EwaldParams(kreps, float(alpha.value), float(sr_cutoff_r), abc, wt)
    if verbose:
        print("\tEwald summation parameters:")
        print(f"\t\tk-replication factors: {kreps[0]} {kreps[1]} {kreps[2]}")
        print(f"\t\tEwald convergence param. α = {ep.alpha:f}")
        print(f"\t\tshort-range cutoff radius (Å): {sr_cutoff_r:f}")
        print(f"\t\t{ep.n_kvecs} kvectors")
        print(f"\t\t(calculated with specified precision {eps:e})")
    return ep
