"""Energy grids: Grid, energy_grid on the GPU, grid index helpers, .cube I/O.

Mirrors Grid (src/grid.jl:12-18), xf_to_id / id_to_xf (:34-61), required_n_pts (:115-123),
write_cube / read_cube (:139-264), energy_grid (:291-362; single-site probes) and the
accessibility lookup (:778-836).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .crystal import Box, Crystal, assert_P1_symmetry, replicate
from .forcefield import LJForceField, replication_factors
from .molecule import Frac, Molecule, needs_rotations
from .paths import rc
from .system import GPUSystem

KJ_PER_MOL_FACTOR = 8.314 / 1000.0  # the factor energy_grid applies (src/grid.jl:358)


@dataclass
class Grid:
    box: Box
    n_pts: tuple
    data: np.ndarray
    units: str
    origin: np.ndarray

    def isapprox(self, other: "Grid", atol: float = 1e-6) -> bool:
        return (np.allclose(self.box.f_to_c, other.box.f_to_c, rtol=1e-5, atol=atol)
                and tuple(self.n_pts) == tuple(other.n_pts)
                and self.units == other.units and np.allclose(self.origin, other.origin, atol=atol)
                and np.allclose(self.data, other.data, atol=atol))


def required_n_pts(box: Box, dx: float) -> tuple[int, int, int]:
    norms = [float(np.linalg.norm(box.f_to_c[:, i])) for i in range(3)]
    return tuple(math.ceil(n / dx) + 1 for n in norms)


def xf_to_id(n_pts, xf) -> list[int]:
    """1-based voxel index of xf with periodic wrap (src/grid.jl:34-44)."""
    vid = [math.floor(x * n) + 1 for x, n in zip(xf, n_pts)]
    for k in range(3):
        if vid[k] <= 0:
            vid[k] += n_pts[k]
        elif vid[k] > n_pts[k]:
            vid[k] -= n_pts[k]
    return vid


def id_to_xf(vid, n_pts) -> np.ndarray:
    return np.array([(vid[k] - 1.0) / (n_pts[k] - 1.0) for k in range(3)])


def _arg_nearest_neighbor(n_pts, xf) -> list[int]:
    return [1 + int(np.round(x * (n - 1))) for x, n in zip(xf, n_pts)]


def _apply_pbc_to_index(vid: list[int], n_pts) -> None:
    for k in range(3):
        if vid[k] == 0:
            vid[k] = n_pts[k]
        if vid[k] == n_pts[k] + 1:
            vid[k] = 1


def accessible(grid: Grid, xf, repfactors=None) -> bool:
    """Inaccessible iff the nearest node and all 26 neighbours are inaccessible (grid.jl:813-836)."""
    if repfactors is not None:
        xf = np.mod(np.asarray(xf) * np.asarray(repfactors), 1.0)
    nn = _arg_nearest_neighbor(grid.n_pts, xf)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                vid = [nn[0] + i, nn[1] + j, nn[2] + k]
                _apply_pbc_to_index(vid, grid.n_pts)
                if grid.data[vid[0] - 1, vid[1] - 1, vid[2] - 1]:
                    return True
    return False


def _units(units) -> str:
    u = str(units).lstrip(":")
    if u not in ("kJ_mol", "K"):
        raise ValueError("Pass :kJ_mol or :K for units of kJ/mol or K, respectively.")
    return u


def energy_grid(crystal: Crystal, molecule: Molecule, ljforcefield: LJForceField, *, resolution=1.0,
                n_rotations: int = 1000, temperature: float = float("nan"), units="kJ_mol", center: bool = False,
                verbose: bool = True) -> Grid:
    """Potential energy of a single-site probe on a regular fractional grid of the unit
    cell (endpoints included), in kJ/mol (×8.314/1000) or K; FP32 data."""
    assert_P1_symmetry(crystal)
    units = _units(units)
    n_pts = tuple(int(v) for v in resolution) if isinstance(resolution, (tuple, list)) else \
        required_n_pts(crystal.box, float(resolution))
    if needs_rotations(molecule):
        if math.isnan(temperature):
            raise ValueError("Must pass temperature (K) for Boltzmann weighted rotations.")
        raise NotImplementedError("energy grids of multi-site probes (rotational Boltzmann averages) are not "
                                  "supported by this build")
    origin = crystal.box.f_to_c @ np.array([-0.5, -0.5, -0.5]) if center else np.zeros(3)
    if verbose:
        print(f"Computing energy grid of {molecule.species} in {crystal.name}")
        print(f"\tRegular grid (in fractional space) of {n_pts[0]} by {n_pts[1]} by {n_pts[2]} points "
              f"superimposed over the unit cell.")
    box = crystal.box
    fmol = Frac(molecule, box)
    repfactors = replication_factors(box, ljforcefield)
    sc = replicate(crystal, repfactors)
    system = GPUSystem(sc, Frac(molecule, sc.box), ljforcefield, None)
    data = system.energy_grid(n_pts, repfactors, KJ_PER_MOL_FACTOR if units == "kJ_mol" else 1.0)
    del fmol
    return Grid(box, n_pts, np.ascontiguousarray(data), units, origin)


def write_cube(grid: Grid, filename: str, verbose: bool = True, length_units: str = "Angstrom") -> Path:
    assert length_units in ("Angstrom", "Bohr")
    d = Path(rc["paths"]["grids"])
    d.mkdir(parents=True, exist_ok=True)
    if ".cube" not in filename:
        filename += ".cube"
    path = d / filename
    with open(path, "w") as f:
        f.write(f"Units of data: {grid.units}\nLoop order: x, y, z\n")
        f.write(f"{0} {grid.origin[0]:f} {grid.origin[1]:f} {grid.origin[2]:f}\n")
        for k in range(3):
            v = grid.box.f_to_c[:, k] / (grid.n_pts[k] - 1)
            if length_units == "Bohr":
                v = 1.88973 * v
            f.write(f"{grid.n_pts[k]} {v[0]:f} {v[1]:f} {v[2]:f}\n")
        for i in range(grid.n_pts[0]):
            for j in range(grid.n_pts[1]):
                for k in range(grid.n_pts[2]):
                    f.write(f"{grid.data[i, j, k]:e} ")
                    if (k + 1) % 6 == 0:
                        f.write("\n")
                f.write("\n")
    if verbose:
        print(f"\tSee {path}")
    return path


def read_cube(filename: str, has_units: bool = True) -> Grid:
    if ".cube" not in filename:
        filename += ".cube"
    path = Path(rc["paths"]["grids"]) / filename
    with open(path) as f:
        line = f.readline()
        units = line.split()[3] if has_units else "missing"
        f.readline()
        parts = f.readline().split()
        n_atoms = int(parts[0])
        origin = np.array([float(p) for p in parts[1:4]])
        box_lines = [f.readline().split() for _ in range(3)]
        n_pts = tuple(int(b[0]) for b in box_lines)
        f_to_c = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                f_to_c[j, i] = float(box_lines[i][j + 1])
        for k in range(3):
            f_to_c[:, k] *= n_pts[k] - 1.0
        for _ in range(n_atoms):
            f.readline()
        vals = [float(t) for t in f.read().split()]
    data = np.array(vals).reshape(n_pts)
    return Grid(Box.from_f_to_c(f_to_c), n_pts, data, units, origin)
