"""Lennard-Jones force field and supercell replication factors (host side).

Mirrors LJForceField (src/forcefield.jl:12-22, constructor :46-100 with the
Lorentz-Berthelot, Kong and geometric mixing rules), replication_factors (:120-162) and
forcefield_coverage (:180-191).
"""
from __future__ import annotations

import csv
import io
import math
import warnings
from pathlib import Path

import numpy as np

from .crystal import Box, Crystal
from .paths import rc

MIXING_RULES = ("lorentz-berthelot", "kong", "geometric")


class LJForceField:
    """Pure (σ, ε) per species and the mixed ε / σ² tables."""

    def __init__(self, forcefield: str | Path | dict, r_cutoff: float = 14.0,
                 mixing_rules: str = "Lorentz-Berthelot", name: str | None = None):
        if mixing_rules.lower() not in MIXING_RULES:
            raise ValueError(f"{mixing_rules} mixing rules not implemented...")
        self.mixing_rules = mixing_rules
        if isinstance(forcefield, dict):
            pure = dict(forcefield)
            self.name = name or "custom"
        else:
            path = Path(forcefield)
            if path.suffix != ".csv":
                path = Path(rc["paths"]["forcefields"]) / (str(forcefield) + ".csv")
            self.name = name or path.stem
            pure = _read_ff_csv(path)
        self.pure_sigma = {k: float(v[0]) for k, v in pure.items()}
        self.pure_epsilon = {k: float(v[1]) for k, v in pure.items()}
        self.r2_cutoff = float(r_cutoff) ** 2
        self.epsilon: dict[str, dict[str, float]] = {}
        self.sigma2: dict[str, dict[str, float]] = {}
        for a in self.pure_sigma:
            self.epsilon[a] = {}
            self.sigma2[a] = {}
            for b in self.pure_sigma:
                e, s2 = _mix(self.pure_epsilon[a], self.pure_sigma[a], self.pure_epsilon[b], self.pure_sigma[b],
                             mixing_rules.lower())
                self.epsilon[a][b] = e
                self.sigma2[a][b] = s2

    @property
    def r_cutoff(self) -> float:
        return math.sqrt(self.r2_cutoff)

    def tables(self, species: list[str]):
        """(ε, σ²) as dense n x n arrays over `species` (errors on a missing species)."""
        missing = [s for s in species if s not in self.pure_sigma]
        if missing:
            raise KeyError(f"species {sorted(set(missing))} missing from the {self.name} force field")
        n = len(species)
        eps = np.zeros((n, n))
        sig2 = np.zeros((n, n))
        for i, a in enumerate(species):
            for j, b in enumerate(species):
                eps[i, j] = self.epsilon[a][b]
                sig2[i, j] = self.sigma2[a][b]
        return eps, sig2

    def __repr__(self):
        return f"LJForceField({self.name!r}, {len(self.pure_sigma)} species, r_cutoff={self.r_cutoff:g} Å)"


def _mix(ei, si, ej, sj, rule):
    if rule == "lorentz-berthelot":
        return math.sqrt(ei * ej), ((si + sj) / 2.0) ** 2
    if rule == "kong":
        e6i, e6j = ei * si ** 6, ej * sj ** 6
        e12i, e12j = e6i * si ** 6, e6j * sj ** 6
        e6 = math.sqrt(e6i * e6j)
        e12 = ((e12i ** (1 / 13) + e12j ** (1 / 13)) / 2) ** 13
        if e12 == 0.0:
            return 0.0, ((si + sj) / 2.0) ** 2
        return e6 ** 2 / e12, (e12 / e6) ** (1 / 3) if e6 > 0 else ((si + sj) / 2.0) ** 2
    return math.sqrt(ei * ej), si * sj


def _read_ff_csv(path: Path) -> dict:
    text = "\n".join(ln for ln in path.read_text().splitlines() if not ln.lstrip().startswith("#"))
    reader = csv.DictReader(io.StringIO(text))
    pure = {}
    for row in reader:
        row = {k.strip().strip('"'): v for k, v in row.items()}
        atom = row["atom"].strip().strip('"')
        if atom in pure:
            raise ValueError(f"Atom {atom} listed at least twice in {path}.")
        pure[atom] = (float(row["sigma(A)"]), float(row["epsilon(K)"]))
    return pure


def replication_factors(box_or_crystal, r_cutoff) -> tuple[int, int, int]:
    """Smallest supercell whose perpendicular half-widths reach r_cutoff
    (src/forcefield.jl:120-158).  r_cutoff may be an LJForceField."""
    box: Box = box_or_crystal.box if isinstance(box_or_crystal, Crystal) else box_or_crystal
    rcut = r_cutoff.r_cutoff if isinstance(r_cutoff, LJForceField) else float(r_cutoff)
    f = box.f_to_c
    a, b, c = f[:, 0].copy(), f[:, 1].copy(), f[:, 2].copy()
    n_ab, n_ac, n_bc = np.cross(a, b), np.cross(a, c), np.cross(b, c)
    rep = [1, 1, 1]

    def center():
        return 0.5 * a + 0.5 * b + 0.5 * c

    c0 = center()
    while abs(np.dot(n_bc, c0)) / np.linalg.norm(n_bc) < rcut:
        rep[0] += 1
        a += f[:, 0]
        c0 = center()
    while abs(np.dot(n_ac, c0)) / np.linalg.norm(n_ac) < rcut:
        rep[1] += 1
        b += f[:, 1]
        c0 = center()
    while abs(np.dot(n_ab, c0)) / np.linalg.norm(n_ab) < rcut:
        rep[2] += 1
        c += f[:, 2]
        c0 = center()
    return rep[0], rep[1], rep[2]


def forcefield_coverage(obj, ljff: LJForceField) -> bool:
    species = obj.atoms.species if hasattr(obj, "atoms") else obj.species
    ok = True
    for s in sorted(set(species)):
        if s not in ljff.pure_epsilon:
            warnings.warn(f"\t{s} missing from {ljff.name} force field.")
            ok = False
    return ok
