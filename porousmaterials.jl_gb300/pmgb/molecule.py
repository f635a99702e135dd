"""Rigid guest molecules (host side).

Mirrors Molecule (src/molecule.jl:10-15; constructor :56-91 reading atoms.csv /
charges.csv), Frac/Cart conversion (:100-109), translate_to! (:171-183),
random_rotation_matrix (:233-246) and needs_rotations (src/mc_helpers.jl:8).
Coordinates are (n, 3) arrays; `frac` tells whether they are fractional.
"""
from __future__ import annotations

import copy
import csv
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .crystal import Box
from .masses import atomic_mass
from .paths import rc


@dataclass
class Molecule:
    species: str
    atom_species: list[str]
    atom_x: np.ndarray    # (n_atoms, 3)
    charge_q: np.ndarray  # (n_charges,)
    charge_x: np.ndarray  # (n_charges, 3)
    com: np.ndarray       # (3,)
    frac: bool = False

    @property
    def n_atoms(self) -> int:
        return len(self.atom_species)

    @property
    def n_charges(self) -> int:
        return int(self.charge_q.shape[0])

    @property
    def charges(self):
        return _ChargesView(self.charge_q)

    def copy(self) -> "Molecule":
        return copy.deepcopy(self)


class _ChargesView:
    def __init__(self, q):
        self.q = q
        self.n = int(q.shape[0])


def center_of_mass(atom_species, atom_x, masses=None) -> np.ndarray:
    m = np.array([atomic_mass(s, masses) for s in atom_species]) if atom_species else np.zeros(0)
    if m.size == 0:
        return np.zeros(3)
    if m.sum() == 0.0:
        return atom_x.mean(axis=0)
    return (m[:, None] * atom_x).sum(axis=0) / m.sum()


def read_molecule(species: str, path: str | Path | None = None, check_neutrality: bool = True,
                  masses: dict | None = None) -> Molecule:
    root = Path(path) if path is not None else Path(rc["paths"]["molecules"])
    d = root / species
    atoms, ax = [], []
    with open(d / "atoms.csv") as f:
        for row in csv.DictReader(f):
            atoms.append(row["atom"].strip())
            ax.append([float(row["x"]), float(row["y"]), float(row["z"])])
    qs, qx = [], []
    with open(d / "charges.csv") as f:
        for row in csv.DictReader(f):
            qs.append(float(row["q"]))
            qx.append([float(row["x"]), float(row["y"]), float(row["z"])])
    ax = np.array(ax, dtype=np.float64).reshape(-1, 3)
    qx = np.array(qx, dtype=np.float64).reshape(-1, 3)
    q = np.array(qs, dtype=np.float64)
    if check_neutrality and q.size and abs(q.sum()) > 1e-4:
        raise ValueError(f"Molecule {species} is not charge neutral! Pass check_neutrality=False to ignore")
    return Molecule(species, atoms, ax, q, qx, center_of_mass(atoms, ax, masses), False)


def molecule_from_sites(species: str, atom_species, atom_x, charge_q=(), charge_x=(), masses=None) -> Molecule:
    ax = np.array(atom_x, dtype=np.float64).reshape(-1, 3)
    q = np.array(charge_q, dtype=np.float64).reshape(-1)
    qx = np.array(charge_x, dtype=np.float64).reshape(-1, 3)
    return Molecule(species, list(atom_species), ax, q, qx, center_of_mass(list(atom_species), ax, masses), False)


def Frac(molecule: Molecule, box: Box) -> Molecule:
    if molecule.frac:
        return molecule.copy()
    m = molecule.copy()
    m.atom_x = (box.c_to_f @ m.atom_x.T).T.copy()
    m.charge_x = (box.c_to_f @ m.charge_x.T).T.copy() if m.n_charges else m.charge_x
    m.com = box.c_to_f @ m.com
    m.frac = True
    return m


def Cart(molecule: Molecule, box: Box) -> Molecule:
    if not molecule.frac:
        return molecule.copy()
    m = molecule.copy()
    m.atom_x = (box.f_to_c @ m.atom_x.T).T.copy()
    m.charge_x = (box.f_to_c @ m.charge_x.T).T.copy() if m.n_charges else m.charge_x
    m.com = box.f_to_c @ m.com
    m.frac = False
    return m


def translate_to(molecule: Molecule, x) -> None:
    """Move the centre of mass to x (same coordinate kind as the molecule), in place."""
    dx = np.asarray(x, dtype=np.float64) - molecule.com
    molecule.atom_x = molecule.atom_x + dx
    if molecule.n_charges:
        molecule.charge_x = molecule.charge_x + dx
    molecule.com = molecule.com + dx


def needs_rotations(molecule: Molecule) -> bool:
    return molecule.n_atoms + molecule.n_charges > 1


def has_charges(molecule: Molecule) -> bool:
    return molecule.n_charges > 0


def random_rotation_matrix(rng: np.random.Generator | None = None) -> np.ndarray:
    """Uniform random rotation by Arvo's method (src/molecule.jl:233-244)."""
    rng = rng or np.random.default_rng()
    u1, u2, u3 = rng.random(3)
    t = 2.0 * math.pi * u1
    rz = np.array([[math.cos(t), math.sin(t), 0.0], [-math.sin(t), math.cos(t), 0.0], [0.0, 0.0, 1.0]])
    p = 2.0 * math.pi * u2
    v = np.array([math.cos(p) * math.sqrt(u3), math.sin(p) * math.sqrt(u3), math.sqrt(1.0 - u3)])
    h = np.eye(3) - 2.0 * np.outer(v, v)
    return -h @ rz


def body_offsets(molecule: Molecule, box: Box | None = None):
    """Cartesian offsets of the LJ sites and charges from the centre of mass."""
    m = Cart(molecule, box) if molecule.frac else molecule
    return m.atom_x - m.com, (m.charge_x - m.com if m.n_charges else np.zeros((0, 3)))
