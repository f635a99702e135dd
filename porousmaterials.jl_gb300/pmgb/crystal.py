"""Crystal geometry on the host: Box, Crystal, a P1 CIF reader, replicate, density.

These mirror the parts of Xtals.jl 0.4 that PorousMaterials.jl re-exports and uses on the
Widom / energy-grid path (src/PorousMaterials.jl:7-9; call sites src/henry.jl:41,86,89,96,
src/grid.jl:295,328,332): a Box built from (a, b, c, α, β, γ) with an upper-triangular
f_to_c whose columns are the lattice vectors, the reciprocal lattice 2π inv(f_to_c)
(rows), fractional-coordinate replication, and the P1 check.

Coordinates are numpy arrays of shape (n, 3): row k holds the xyz of atom k, which is the
same memory order as Julia's 3 x n column-major `coords.xf`.
"""
from __future__ import annotations

import math
import re
import shlex
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .masses import atomic_mass


class Box:
    """Unit-cell (or supercell) geometry."""

    def __init__(self, a: float, b: float, c: float, alpha: float, beta: float, gamma: float):
        ca, cb, cg, sg = math.cos(alpha), math.cos(beta), math.cos(gamma), math.sin(gamma)
        omega = a * b * c * math.sqrt(1.0 - ca * ca - cb * cb - cg * cg + 2.0 * ca * cb * cg)
        f_to_c = np.array([[a, b * cg, c * cb],
                           [0.0, b * sg, c * (ca - cb * cg) / sg],
                           [0.0, 0.0, omega / (a * b * sg)]])
        self._set(a, b, c, alpha, beta, gamma, omega, f_to_c)

    def _set(self, a, b, c, alpha, beta, gamma, omega, f_to_c):
        self.a, self.b, self.c = float(a), float(b), float(c)
        self.alpha, self.beta, self.gamma = float(alpha), float(beta), float(gamma)
        self.Omega = float(omega)
        self.f_to_c = np.ascontiguousarray(f_to_c, dtype=np.float64)
        self.c_to_f = np.linalg.inv(self.f_to_c)
        self.reciprocal_lattice = 2.0 * math.pi * self.c_to_f

    @classmethod
    def from_f_to_c(cls, f_to_c) -> "Box":
        """Box from its lattice vectors (columns of f_to_c)."""
        f = np.asarray(f_to_c, dtype=np.float64)
        av, bv, cv = f[:, 0], f[:, 1], f[:, 2]
        a, b, c = (float(np.linalg.norm(v)) for v in (av, bv, cv))
        alpha = math.acos(float(np.dot(bv, cv)) / (b * c))
        beta = math.acos(float(np.dot(av, cv)) / (a * c))
        gamma = math.acos(float(np.dot(av, bv)) / (a * b))
        box = cls.__new__(cls)
        box._set(a, b, c, alpha, beta, gamma, abs(float(np.linalg.det(f))), f)
        return box

    def __repr__(self):
        return (f"Box(a={self.a:.4f}, b={self.b:.4f}, c={self.c:.4f}, α={math.degrees(self.alpha):.3f}°, "
                f"β={math.degrees(self.beta):.3f}°, γ={math.degrees(self.gamma):.3f}°, Ω={self.Omega:.3f} Å³)")

    def isapprox(self, other: "Box", rtol: float = 1e-8) -> bool:
        return bool(np.allclose(self.f_to_c, other.f_to_c, rtol=rtol, atol=1e-10))


def replicate_box(box: Box, repfactors) -> Box:
    ra, rb, rc = (int(r) for r in repfactors)
    return Box(box.a * ra, box.b * rb, box.c * rc, box.alpha, box.beta, box.gamma)


@dataclass
class Atoms:
    species: list[str]
    xf: np.ndarray  # (n, 3) fractional

    @property
    def n(self) -> int:
        return len(self.species)


@dataclass
class Charges:
    q: np.ndarray   # (n,)
    xf: np.ndarray  # (n, 3) fractional

    @property
    def n(self) -> int:
        return int(self.q.shape[0])


@dataclass
class Crystal:
    name: str
    box: Box
    atoms: Atoms
    charges: Charges
    symmetry_is_p1: bool = True
    meta: dict = field(default_factory=dict)


def has_charges(obj) -> bool:
    """True iff the crystal (or molecule) carries point charges (Xtals has_charges,
    src/molecule.jl:322 for molecules)."""
    return obj.charges.n > 0


def assert_P1_symmetry(crystal: Crystal) -> None:
    if not crystal.symmetry_is_p1:
        raise ValueError(f"the crystal {crystal.name} is not in P1 symmetry; convert it to P1 first")


def net_charge(crystal: Crystal) -> float:
    return float(np.sum(crystal.charges.q))


# ---------------------------------------------------------------------------
# CIF reading (P1)
# ---------------------------------------------------------------------------
_NUM = re.compile(r"^([-+]?[0-9]*\.?[0-9]+(?:[eE][-+]?[0-9]+)?)")


def _cif_float(tok: str) -> float:
    m = _NUM.match(tok.strip().strip("'\""))
    if not m:
        raise ValueError(f"not a number in CIF: {tok!r}")
    return float(m.group(1))


def _tokenize(line: str) -> list[str]:
    try:
        return shlex.split(line, posix=True)
    except ValueError:
        return line.split()


def read_cif(path: str | Path, species_col=("_atom_site_type_symbol", "_atom_site_label"),
             wrap_coords: bool = True, include_zero_charges: bool = True,
             check_neutrality: bool = True, net_charge_tol: float = 1e-3) -> Crystal:
    """Read a CIF in P1 (or whose symmetry operations are the identity only).  A bare file name
    that does not exist where it is given is looked up in rc["paths"]["crystals"], as Xtals'
    Crystal(filename) does."""
    from .paths import rc

    path = Path(path)
    if not path.exists() and not path.is_absolute() and rc["paths"].get("crystals"):
        path = Path(rc["paths"]["crystals"]) / path
    text = path.read_text()
    lines = [ln.split("#", 1)[0].rstrip() if not ln.lstrip().startswith(";") else ln for ln in text.splitlines()]
    scalars: dict[str, str] = {}
    loops: list[tuple[list[str], list[list[str]]]] = []
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        if not ln:
            i += 1
            continue
        if ln.lower().startswith("loop_"):
            i += 1
            heads = []
            while i < len(lines) and lines[i].strip().startswith("_"):
                heads.append(lines[i].strip().split()[0])
                i += 1
            rows = []
            while i < len(lines):
                s = lines[i].strip()
                if not s:
                    i += 1
                    if rows:
                        break
                    continue
                if s.startswith("_") or s.lower().startswith("loop_") or s.lower().startswith("data_"):
                    break
                toks = _tokenize(s)
                # a row may wrap over several lines
                while len(toks) < len(heads) and i + 1 < len(lines) and lines[i + 1].strip() and \
                        not lines[i + 1].strip().startswith("_"):
                    i += 1
                    toks += _tokenize(lines[i].strip())
                rows.append(toks)
                i += 1
            loops.append((heads, rows))
            continue
        if ln.startswith("_"):
            parts = ln.split(None, 1)
            if len(parts) == 2:
                scalars[parts[0]] = parts[1].strip()
            i += 1
            continue
        i += 1

    a = _cif_float(scalars["_cell_length_a"])
    b = _cif_float(scalars["_cell_length_b"])
    c = _cif_float(scalars["_cell_length_c"])
    al = math.radians(_cif_float(scalars["_cell_angle_alpha"]))
    be = math.radians(_cif_float(scalars["_cell_angle_beta"]))
    ga = math.radians(_cif_float(scalars["_cell_angle_gamma"]))
    box = Box(a, b, c, al, be, ga)

    # symmetry: P1 if the H-M symbol says so, or every listed operation is the identity
    p1 = True
    hm = None
    for key in ("_symmetry_space_group_name_H-M", "_space_group_name_H-M_alt"):
        if key in scalars:
            hm = scalars[key].strip("'\"").replace(" ", "").upper()
    ops = []
    for heads, rows in loops:
        for key in ("_symmetry_equiv_pos_as_xyz", "_space_group_symop_operation_xyz"):
            if key in heads:
                col = heads.index(key)
                ops += ["".join(r[col:]).replace(" ", "").replace("'", "").lower() for r in rows if len(r) > col]
    if ops:
        p1 = all(op in ("x,y,z", "+x,+y,+z") for op in ops)
    elif hm is not None:
        p1 = hm in ("P1",)

    site = None
    for heads, rows in loops:
        if any(h.startswith("_atom_site_fract") or h.startswith("_atom_site_Cartn") for h in heads):
            site = (heads, rows)
            break
    if site is None:
        raise ValueError(f"{path.name}: no _atom_site loop")
    heads, rows = site
    scol = next((heads.index(k) for k in species_col if k in heads), None)
    if scol is None:
        raise ValueError(f"{path.name}: no species column among {species_col}")
    frac = "_atom_site_fract_x" in heads
    cols = [heads.index(k) for k in (("_atom_site_fract_x", "_atom_site_fract_y", "_atom_site_fract_z") if frac
                                    else ("_atom_site_Cartn_x", "_atom_site_Cartn_y", "_atom_site_Cartn_z"))]
    qcol = heads.index("_atom_site_charge") if "_atom_site_charge" in heads else None
    species, xyz, qs = [], [], []
    for r in rows:
        if len(r) < len(heads):
            continue
        species.append(r[scol])
        xyz.append([_cif_float(r[k]) for k in cols])
        if qcol is not None:
            qs.append(_cif_float(r[qcol]))
    xyz = np.array(xyz, dtype=np.float64).reshape(-1, 3)
    xf = xyz if frac else (box.c_to_f @ xyz.T).T
    if wrap_coords:
        xf = np.mod(xf, 1.0)
    xf = np.ascontiguousarray(xf)
    if qcol is not None:
        q = np.array(qs, dtype=np.float64)
        keep = np.ones(len(q), dtype=bool) if include_zero_charges else (q != 0.0)
        charges = Charges(q[keep].copy(), np.ascontiguousarray(xf[keep]))
    else:
        charges = Charges(np.zeros(0), np.zeros((0, 3)))
    cr = Crystal(path.name, box, Atoms(species, xf), charges, p1)
    if check_neutrality and charges.n > 0 and abs(net_charge(cr)) > net_charge_tol:
        raise ValueError(f"{path.name} is not charge neutral (net charge {net_charge(cr):.6g})")
    return cr


Crystal.from_cif = staticmethod(read_cif)  # type: ignore[attr-defined]


def strip_numbers_from_atom_labels(crystal: Crystal) -> None:
    """'Zn1' -> 'Zn' in place (Xtals strip_numbers_from_atom_labels!)."""
    crystal.atoms.species = [re.sub(r"[0-9]+$", "", re.sub(r"[^A-Za-z_0-9]", "", s)) or s
                             for s in crystal.atoms.species]


def replicate(crystal: Crystal, repfactors) -> Crystal:
    """Supercell of ra x rb x rc unit cells with fractional coordinates rescaled into the
    supercell (Xtals.replicate; src/henry.jl:86)."""
    assert_P1_symmetry(crystal)
    rep = np.array([int(r) for r in repfactors], dtype=np.int64)
    if np.any(rep < 1):
        raise ValueError(f"replication factors must be >= 1, got {tuple(rep)}")
    shifts = np.array([(i, j, k) for i in range(rep[0]) for j in range(rep[1]) for k in range(rep[2])],
                      dtype=np.float64)

    def rep_xf(xf):
        if xf.shape[0] == 0:
            return np.zeros((0, 3))
        out = (xf[None, :, :] + shifts[:, None, :]) / rep[None, None, :]
        return np.ascontiguousarray(out.reshape(-1, 3))

    n_img = shifts.shape[0]
    atoms = Atoms(list(crystal.atoms.species) * n_img, rep_xf(crystal.atoms.xf))
    charges = Charges(np.tile(crystal.charges.q, n_img), rep_xf(crystal.charges.xf))
    return Crystal(crystal.name, replicate_box(crystal.box, rep), atoms, charges, True, dict(crystal.meta))


def crystal_density(crystal: Crystal, masses: dict | None = None) -> float:
    """Mass density in kg/m³ (Xtals crystal_density; used at src/henry.jl:96,143).  The mass is
    summed per species (one table lookup per species, not per atom)."""
    from collections import Counter

    total = sum(atomic_mass(s, masses) * n for s, n in Counter(crystal.atoms.species).items())
    return total / crystal.box.Omega * 1660.5390666


def Frac_point(x, box: Box) -> np.ndarray:
    return box.c_to_f @ np.asarray(x, dtype=np.float64)


def Cart_point(xf, box: Box) -> np.ndarray:
    return box.f_to_c @ np.asarray(xf, dtype=np.float64)
