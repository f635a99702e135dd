"""Seeded synthetic frameworks and guests for the benchmark workloads.

No public benchmark suite exists for this path; the workloads are defined by their
shapes: cell, atom count and species mix (Zn:O:C:H = 32:104:192:96), positions uniform
with a 1.2 Å minimum-image separation, N(0, 0.4) charges shifted to neutrality, UFF-like
Lorentz-Berthelot parameters, CH4 / CO2 / Xe guests.
"""
from __future__ import annotations

import math

import numpy as np

from .crystal import Atoms, Box, Charges, Crystal
from .forcefield import LJForceField
from .molecule import molecule_from_sites

SPECIES_MIX = {"Zn": 32, "O": 104, "C": 192, "H": 96}
UFF_LIKE = {  # species: (sigma Å, epsilon K)
    "Zn": (2.46, 62.4), "O": (3.12, 30.19), "C": (3.43, 52.83), "H": (2.57, 22.14),
    "CH4": (3.73, 148.0), "C_CO2": (2.80, 27.0), "O_CO2": (3.05, 79.0), "Xe": (4.10, 221.0),
}


def forcefield(r_cutoff: float = 12.5) -> LJForceField:
    return LJForceField(dict(UFF_LIKE), r_cutoff=r_cutoff, name="UFF_like")


def species_counts(n_atoms: int) -> dict:
    total = sum(SPECIES_MIX.values())
    raw = {s: n_atoms * c / total for s, c in SPECIES_MIX.items()}
    counts = {s: int(round(v)) for s, v in raw.items()}
    # fix rounding so the counts add up to n_atoms (largest remainders first)
    diff = n_atoms - sum(counts.values())
    order = sorted(raw, key=lambda s: raw[s] - math.floor(raw[s]), reverse=(diff > 0))
    for s in order[:abs(diff)]:
        counts[s] += 1 if diff > 0 else -1
    return counts


def _place(box: Box, n: int, rng: np.random.Generator, min_sep: float = 1.2, max_tries: int = 200000) -> np.ndarray:
    """n fractional positions, uniform, every minimum-image pair at least min_sep apart."""
    # cell list in fractional space with cells at least min_sep wide along each axis
    widths = box.Omega / np.array([np.linalg.norm(np.cross(box.f_to_c[:, (i + 1) % 3], box.f_to_c[:, (i + 2) % 3]))
                                   for i in range(3)])
    nc = np.maximum(1, np.floor(widths / min_sep).astype(int))
    cells: dict = {}
    pts = np.zeros((n, 3))
    k = 0
    tries = 0
    while k < n:
        tries += 1
        if tries > max_tries + 50 * n:
            raise RuntimeError("could not place atoms with the requested separation")
        x = rng.random(3)
        c = tuple((x * nc).astype(int) % nc)
        ok = True
        for d0 in (-1, 0, 1):
            for d1 in (-1, 0, 1):
                for d2 in (-1, 0, 1):
                    cc = ((c[0] + d0) % nc[0], (c[1] + d1) % nc[1], (c[2] + d2) % nc[2])
                    for j in cells.get(cc, ()):
                        d = pts[j] - x
                        d -= np.round(d)
                        if np.dot(box.f_to_c @ d, box.f_to_c @ d) < min_sep * min_sep:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            pts[k] = x
            cells.setdefault(c, []).append(k)
            k += 1
    return pts


def framework(name: str, box: Box, n_atoms: int, seed: int, charged: bool, q_sigma: float = 0.4) -> Crystal:
    rng = np.random.default_rng(seed)
    counts = species_counts(n_atoms)
    species = [s for s, c in counts.items() for _ in range(c)]
    rng.shuffle(species)
    xf = _place(box, n_atoms, rng)
    if charged:
        q = rng.normal(0.0, q_sigma, n_atoms)
        q -= q.mean()
        charges = Charges(q, xf.copy())
    else:
        charges = Charges(np.zeros(0), np.zeros((0, 3)))
    return Crystal(name, box, Atoms(species, xf), charges, True, {"seed": seed})


def ch4():
    return molecule_from_sites("CH4", ["CH4"], [[0.0, 0.0, 0.0]])


def xe():
    return molecule_from_sites("Xe", ["Xe"], [[0.0, 0.0, 0.0]])


def co2():
    x = [[0.0, 0.0, 0.0], [-1.16, 0.0, 0.0], [1.16, 0.0, 0.0]]
    return molecule_from_sites("CO2", ["C_CO2", "O_CO2", "O_CO2"], x, [0.70, -0.35, -0.35], x)


def config0(seed: int = 1000) -> Crystal:
    """Cubic a = 25.832 Å, 424 uncharged atoms."""
    d = math.pi / 2
    return framework("synthetic_c0", Box(25.832, 25.832, 25.832, d, d, d), 424, seed, charged=False)


def config1(seed: int = 1001) -> Crystal:
    """Triclinic 13.2 / 18.9 / 9.8 Å, β = 102°, 600 charged atoms (replicated 2x2x3 for a 12.5 Å cutoff)."""
    d = math.pi / 2
    return framework("synthetic_c1", Box(13.2, 18.9, 9.8, d, math.radians(102.0), d), 600, seed, charged=True)


def config1_porous(seed: int = 1101, n_atoms: int = 150) -> Crystal:
    """The config1 cell with a quarter of the atoms: open enough for CO2 to bind, so the
    Boltzmann-weighted averages are not dominated by a single insertion."""
    d = math.pi / 2
    return framework("synthetic_c1_porous", Box(13.2, 18.9, 9.8, d, math.radians(102.0), d), n_atoms, seed,
                     charged=True)


def config4(seed: int = 1004) -> Crystal:
    """Orthorhombic 52 Å cube, 20,000 charged atoms."""
    d = math.pi / 2
    return framework("synthetic_c4", Box(52.0, 52.0, 52.0, d, d, d), 20000, seed, charged=True)


def batch_frameworks(n: int = 512, seed: int = 1003):
    """Frameworks of uneven size: atoms log-uniform 50-5000, lengths U(8, 40) Å, angles U(80, 110)°,
    neutralised N(0, 0.4) charges."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        for _ in range(100):
            a, b, c = rng.uniform(8.0, 40.0, 3)
            al, be, ga = np.radians(rng.uniform(80.0, 110.0, 3))
            arg = 1 - math.cos(al) ** 2 - math.cos(be) ** 2 - math.cos(ga) ** 2 + 2 * math.cos(al) * math.cos(be) * math.cos(ga)
            if arg > 0.05:
                break
        box = Box(a, b, c, al, be, ga)
        n_atoms = int(round(math.exp(rng.uniform(math.log(50), math.log(5000)))))
        # keep the packing physical: at most one atom per 7 Å³
        n_atoms = max(1, min(n_atoms, int(box.Omega / 7.0)))
        out.append(framework(f"batch_{i:03d}", box, n_atoms, int(rng.integers(1 << 31)), charged=True))
    return out
