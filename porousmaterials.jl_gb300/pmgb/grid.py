"""Energy grids: Grid, energy_grid on the GPU, grid index helpers, .cube I/O.

Mirrors Grid (src/grid.jl:12-18), xf_to_id / id_to_xf (:34-61), required_n_pts (:115-123),
write_cube / read_cube (:139-264), energy_grid (:291-362; single-site probes) and the
accessibility lookup (:778-836).
"""
from __future__ import annotations

import math
import secrets
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
                verbose: bool = True, seed: int | None = None) -> Grid:
    """Potential energy of a probe on a regular fractional grid of the unit cell (endpoints
    included), in kJ/mol (×8.314/1000) or K; FP32 data (src/grid.jl:291-362).  A single-site
    probe gets its van der Waals energy; a probe that needs rotations gets -T log⟨e^{-U/T}⟩ over
    n_rotations random orientations at `temperature`, with the Ewald energy included when crystal
    and probe are charged (pmgb_energy_grid_rotational; `seed` fixes the orientations)."""
    assert_P1_symmetry(crystal)
    units = _units(units)
    n_pts = tuple(int(v) for v in resolution) if isinstance(resolution, (tuple, list)) else \
        required_n_pts(crystal.box, float(resolution))
    rotations = needs_rotations(molecule)
    if rotations and math.isnan(temperature):
        raise ValueError("Must pass temperature (K) for Boltzmann weighted rotations.")
    origin = crystal.box.f_to_c @ np.array([-0.5, -0.5, -0.5]) if center else np.zeros(3)
    if verbose:
        print(f"Computing energy grid of {molecule.species} in {crystal.name}")
        print(f"\tRegular grid (in fractional space) of {n_pts[0]} by {n_pts[1]} by {n_pts[2]} points "
              f"superimposed over the unit cell.")
        if rotations:
            print(f"\t{n_rotations} molecule rotations per grid point with temperature {temperature:f} K.")
    box = crystal.box
    repfactors = replication_factors(box, ljforcefield)
    sc = replicate(crystal, repfactors)
    factor = KJ_PER_MOL_FACTOR if units == "kJ_mol" else 1.0
    if rotations:
        from .crystal import has_charges
        from .ewald import setup_Ewald_sum

        charged = has_charges(sc) and molecule.n_charges > 0
        ep = setup_Ewald_sum(sc.box, ljforcefield.r_cutoff, verbose=verbose and charged) if charged else None
        system = GPUSystem(sc, Frac(molecule, sc.box), ljforcefield, ep)
        if seed is None:
            seed = secrets.randbits(63)
        data = system.energy_grid_rotational(n_pts, repfactors, n_rotations, temperature, seed, factor)
    else:
        system = GPUSystem(sc, Frac(molecule, sc.box), ljforcefield, None)
        data = system.energy_grid(n_pts, repfactors, factor)
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


# ---------------------------------------------------------------------------- accessibility
def _segment_grid(data: np.ndarray, energy_tol: float) -> tuple[np.ndarray, int]:
    """Flood fill (src/grid.jl:383-456): label the 26-connected regions of points with energy
    below energy_tol (1, 2, ... in the reference's scan order), -1 elsewhere.  The grid's
    faces are not wrapped here: connections across the unit-cell faces are the graph's job."""
    from scipy import ndimage

    accessible_pts = data < energy_tol
    labels, n = ndimage.label(accessible_pts, structure=np.ones((3, 3, 3), dtype=bool))
    # renumber in the reference's scan order (i slowest, k fastest: the array's C order)
    order = np.zeros(n + 1, dtype=np.int64)
    first = {}
    flat = labels.reshape(-1)
    nz = np.flatnonzero(flat)
    _, idx = np.unique(flat[nz], return_index=True)
    for new, lab in enumerate(flat[nz][np.sort(idx)], start=1):
        first[int(lab)] = new
    for lab, new in first.items():
        order[lab] = new
    seg = np.where(labels > 0, order[labels], -1)
    return seg, n


def _segment_connections(seg: np.ndarray) -> list[tuple[int, int, tuple[int, int, int]]]:
    """Directed segment connections across the unit-cell faces (src/grid.jl:490-545): the end
    plane and the first plane of each axis are the same points (endpoints included), each
    connection noted once with its reverse."""
    conns: list[tuple[int, int, tuple[int, int, int]]] = []
    seen = set()

    def note(a: int, b: int, d: tuple[int, int, int]):
        if a == -1 or b == -1:
            return
        if (a, b, d) in seen:
            return
        seen.add((a, b, d))
        conns.append((a, b, d))
        rev = (b, a, (-d[0], -d[1], -d[2]))
        seen.add(rev)
        conns.append(rev)

    n1, n2, n3 = seg.shape
    for i in range(n1):
        for j in range(n2):
            note(int(seg[i, j, -1]), int(seg[i, j, 0]), (0, 0, 1))
    for j in range(n2):
        for k in range(n3):
            note(int(seg[-1, j, k]), int(seg[0, j, k]), (1, 0, 0))
    for i in range(n1):
        for k in range(n3):
            note(int(seg[i, -1, k]), int(seg[i, 0, k]), (0, 1, 0))
    return conns


def _simple_cycles(adj: dict[int, list[int]]):
    """All simple cycles of a directed graph (Johnson's algorithm, 1975), each as a vertex list
    starting at its smallest vertex."""
    def scc_of(nodes: set[int]) -> list[set[int]]:
        index, low, onstack, stack, out = {}, {}, set(), [], []
        counter = [0]
        for root in sorted(nodes):
            if root in index:
                continue
            work = [(root, iter(adj.get(root, ())))]
            index[root] = low[root] = counter[0]
            counter[0] += 1
            stack.append(root)
            onstack.add(root)
            while work:
                v, it = work[-1]
                advanced = False
                for w in it:
                    if w not in nodes:
                        continue
                    if w not in index:
                        index[w] = low[w] = counter[0]
                        counter[0] += 1
                        stack.append(w)
                        onstack.add(w)
                        work.append((w, iter(adj.get(w, ()))))
                        advanced = True
                        break
                    if w in onstack:
                        low[v] = min(low[v], index[w])
                if advanced:
                    continue
                work.pop()
                if work:
                    low[work[-1][0]] = min(low[work[-1][0]], low[v])
                if low[v] == index[v]:
                    comp = set()
                    while True:
                        w = stack.pop()
                        onstack.discard(w)
                        comp.add(w)
                        if w == v:
                            break
                    out.append(comp)
        return out

    remaining = set(adj) | {w for ws in adj.values() for w in ws}
    while remaining:
        comps = [c for c in scc_of(remaining) if len(c) > 1 or any(v in adj.get(v, ()) for v in c)]
        if not comps:
            break
        s = min(min(c) for c in comps)
        comp = next(c for c in comps if s in c)
        blocked, bmap, path = {s}, {}, [s]
        stack = [(s, iter([w for w in adj.get(s, ()) if w in comp]))]
        closed = [False]
        while stack:
            v, it = stack[-1]
            nxt = next(it, None)
            if nxt is not None:
                if nxt == s:
                    yield list(path)
                    closed[-1] = True
                elif nxt not in blocked:
                    path.append(nxt)
                    blocked.add(nxt)
                    stack.append((nxt, iter([w for w in adj.get(nxt, ()) if w in comp])))
                    closed.append(False)
                continue
            stack.pop()
            done = closed.pop()
            if done:
                # unblock v and everything waiting on it
                todo = [v]
                while todo:
                    u = todo.pop()
                    if u in blocked:
                        blocked.discard(u)
                        todo.extend(bmap.pop(u, ()))
            else:
                for w in adj.get(v, ()):
                    if w in comp:
                        bmap.setdefault(w, set()).add(v)
            path.pop()
            if closed:
                closed[-1] = closed[-1] or done
        remaining.discard(s)


def _classify_segments(n_segments: int, conns) -> np.ndarray:
    """1 for segments on a simple cycle of the segment graph that ends in another unit cell
    (src/grid.jl:548-616), 0 otherwise.  As in the reference, each connection is a vertex of
    its own carrying the face it crosses."""
    adj: dict[int, list[int]] = {v: [] for v in range(1, n_segments + 1)}
    direction: dict[int, tuple[int, int, int]] = {}
    for a, b, d in conns:
        c = n_segments + 1 + len(direction)
        direction[c] = d
        adj.setdefault(a, []).append(c)
        adj[c] = [b]
    cls = np.zeros(n_segments + 1, dtype=np.int64)
    for cyc in _simple_cycles(adj):
        cell = np.zeros(3, dtype=np.int64)
        for v in cyc:
            if v in direction:
                cell += direction[v]
        if np.any(cell != 0):
            for v in cyc:
                if v not in direction:
                    cls[v] = 1
    # the reference then marks segments with a direct edge into an accessible one; every
    # segment edge runs through a connection vertex, so that step adds nothing
    return cls[1:]


def compute_accessibility_grid(crystal: Crystal, probe: Molecule, forcefield: LJForceField, *,
                               resolution=1.0, energy_tol: float = 10.0, energy_units="kJ_mol",
                               verbose: bool = True, write_b4_after_grids: bool = True,
                               block_inaccessible_pockets: bool = True):
    """(accessibility Grid of Bool, nb_segments_blocked, porosity) of src/grid.jl:689-774: the
    probe's energy grid (on the GPU), points below energy_tol occupiable, and with
    block_inaccessible_pockets the occupiable regions that do not connect to their own images
    in another unit cell blocked.  porosity is a float without blocking, else a dict with
    'b4_blocking' and 'after_blocking'."""
    assert_P1_symmetry(crystal)
    units = _units(energy_units)
    if verbose:
        print(f"Computing accessibility grid of {crystal.name} using {energy_tol:f} {units} potential energy tol "
              f"and {probe.species} probe...")
    grid = energy_grid(crystal, probe, forcefield, resolution=resolution, verbose=verbose, units=units)
    data = np.asarray(grid.data, dtype=np.float64)
    if not block_inaccessible_pockets:
        acc = Grid(grid.box, grid.n_pts, data < energy_tol, "accessibility", grid.origin)
        return acc, 0, float(np.mean(acc.data))
    seg, n_segments = _segment_grid(data, energy_tol)
    if verbose:
        print(f"Found {n_segments} segments")
    name = crystal.name.replace(".cif", "").replace(".cssr", "")
    ffname = forcefield.name.replace(".csv", "")
    if write_b4_after_grids:
        write_cube(Grid(grid.box, grid.n_pts, np.where(seg != -1, 1, -1), "Segment_No", grid.origin),
                   f"{probe.species}_in_{name}_{ffname}_b4_pocket_blocking.cube", verbose=verbose)
    cls = _classify_segments(n_segments, _segment_connections(seg))
    for s in range(1, n_segments + 1):
        if cls[s - 1] == 0:
            seg[seg == s] = -1
    out = np.where(seg != -1, 1, -1)
    if write_b4_after_grids:
        write_cube(Grid(grid.box, grid.n_pts, out, "Segment_No", grid.origin),
                   f"{probe.species}_in_{name}_{ffname}_after_pocket_blocking.cube", verbose=verbose)
    nb_blocked = int(np.sum(cls == 0))
    acc = Grid(grid.box, grid.n_pts, out == 1, "accessibility", grid.origin)
    porosity = {"b4_blocking": float(np.mean(data < energy_tol)), "after_blocking": float(np.mean(acc.data))}
    if verbose and nb_blocked:
        print(f"\t{nb_blocked} pockets in {crystal.name} were found to be inaccessible to {probe.species} "
              f"and blocked.")
    return acc, nb_blocked, porosity
