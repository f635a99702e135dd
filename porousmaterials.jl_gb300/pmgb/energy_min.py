"""Energy minimisation of a guest's centre of mass (src/energy_min.jl).

find_energy_minimum_gridsearch: the GPU energy grid and its lowest point (energy_min.jl:75-85).
find_energy_minimum: local minimisation of the guest-host van der Waals energy over the
centre of mass (energy_min.jl:19-58).  The reference runs Nelder-Mead on energies alone; here
each step gets the energy and its gradient from the GPU adjoint (pmgb_energies_grad: dU/dx of
the rigid guest) and L-BFGS uses both.  Orientation is not optimised, as in the reference.
"""
from __future__ import annotations

import warnings

import numpy as np

from .crystal import Crystal, has_charges, replicate
from .forcefield import LJForceField, replication_factors
from .grid import energy_grid, id_to_xf
from .molecule import Frac, Molecule, needs_rotations, translate_to
from ._lib import Context
from .system import GPUSystem

K_TO_KJ = 8.314 / 1000.0  # energy_min.jl:49 (the grid factor, not R)


MAX_CANDIDATES = 65536  # grid points re-evaluated in FP64 before the argmin, at most


def _visited_coordinate(values, repeat: int, n_cycles: int, start_atom: float, start_com: float):
    """Coordinates at which the reference's energy_grid loop places a one-atom probe along one axis.

    The loop (src/grid.jl:331-333) calls translate_to!(molecule, Frac(xf ./ repfactors)), which adds
    d = target - com to the atom and to the centre of mass (src/molecule.jl:147-151,176-179): each
    value of this axis is targeted `repeat` times in a row, the sequence of values `n_cycles` times.
    A repeated target is reached exactly on its second step (target - com is then exact), after which
    further steps change nothing.  Returns f(cycle, m, r) -> the atom's coordinate after the r-th
    step (0-based) at value m of that cycle."""
    n = len(values)
    steps = min(repeat, 2)
    table, seen = [], {}
    atom, com = float(start_atom), float(start_com)
    for cyc in range(n_cycles):
        key = (atom, com)
        if key in seen:                       # from here on the cycles repeat
            first = seen[key]
            period = cyc - first
            break
        seen[key] = cyc
        rows = []
        for m in range(n):
            row = []
            for _ in range(steps):
                d = values[m] - com
                atom, com = atom + d, com + d
                row.append(atom)
            rows.append(row)
        table.append(rows)
    else:
        first, period = 0, max(len(table), 1)

    def at(cycle: int, m: int, r: int) -> float:
        c = cycle if cycle < len(table) else first + (cycle - first) % period
        return table[c][m][min(r, steps - 1)]

    return at


def reference_grid_positions(n_pts, repfactors, start_atom_xf, start_com_xf, ids) -> np.ndarray:
    """Fractional coordinates (supercell) at which the reference's energy_grid evaluates the grid
    points `ids` ((i, j, k), 0-based) for a one-atom probe that starts at start_atom_xf with its
    centre of mass at start_com_xf, replaying the loop's order (k fastest, src/grid.jl:331) and its
    FP64 translate_to! steps.  The targets are (i/(n-1), j/(n-1), k/(n-1)) ./ repfactors."""
    n0, n1, n2 = (int(n) for n in n_pts)
    axes = []
    for a, (n, rep, rpt, cyc) in enumerate(((n0, repfactors[0], n1 * n2, 1), (n1, repfactors[1], n2, n0),
                                             (n2, repfactors[2], 1, n0 * n1))):
        vals = [(m / (n - 1.0) if n > 1 else 0.0) / float(rep) for m in range(n)]
        axes.append(_visited_coordinate(vals, rpt, cyc, start_atom_xf[a], start_com_xf[a]))
    out = np.empty((len(ids), 3))
    for t, (i, j, k) in enumerate(ids):
        out[t, 0] = axes[0](0, i, j * n2 + k)
        out[t, 1] = axes[1](i, j, k)
        out[t, 2] = axes[2](i * n1 + j, k, 0)
    return out


def find_energy_minimum_gridsearch(crystal: Crystal, molecule: Molecule, ljforcefield: LJForceField, *,
                                   resolution=1.0, n_pts=None):
    """(molecule at the lowest grid point (fractional), that energy in kJ/mol).  n_pts is the
    keyword the reference's test passes (test/energy_min.jl:20); resolution is the function's.

    The GPU grid (every point within 1e-5 relative or 1e-4 K of FP64) selects the candidates: every
    point within twice that tolerance of the grid's minimum.  Those are re-evaluated in FP64 in the
    reference's own operation order at the positions the reference's grid loop gives the probe
    (pmgb_vdw_energy_ordered, reference_grid_positions), and the minimum is the first in
    column-major order, as Julia's findmin over the reference's FP64 grid.  Points whose energies
    are equal in exact arithmetic (inversion images) are thereby told apart as the reference's
    rounding tells them apart."""
    res = n_pts if n_pts is not None else resolution
    grid = energy_grid(crystal, molecule, ljforcefield, resolution=res, verbose=False, units="kJ_mol")
    data = np.asarray(grid.data)
    flat = data.ravel(order="F")
    fin = np.isfinite(flat)
    rep = replication_factors(crystal.box, ljforcefield)
    fmol = Frac(molecule, crystal.box)          # the probe in unit-cell fractions (src/grid.jl:325)
    if fmol.n_atoms != 1:
        raise ValueError("find_energy_minimum_gridsearch: a one-atom probe is required (the grid of a "
                         "probe that needs rotations takes a temperature)")
    if fin.any():
        lo = float(flat[fin].min())
        tol = max(1e-5 * abs(lo), 1e-4 * K_TO_KJ)
        cand = np.flatnonzero(fin & (flat <= lo + 2.0 * tol))
    else:
        cand = np.arange(flat.size)
    cand = cand[:MAX_CANDIDATES]                                   # column-major order
    ids = [tuple(int(v) for v in np.unravel_index(int(c), data.shape, order="F")) for c in cand]
    sc = replicate(crystal, rep)
    sites = reference_grid_positions(grid.n_pts, rep, np.asarray(fmol.atom_x)[0], np.asarray(fmol.com), ids)
    species = sorted(set(sc.atoms.species) | set(fmol.atom_species))
    sid = {s: i for i, s in enumerate(species)}
    eps, sig2 = ljforcefield.tables(species)
    ctx = Context.default(0)
    e_k = ctx.vdw_energy_ordered(sc.box.f_to_c, sc.atoms.xf, [sid[s] for s in sc.atoms.species], eps, sig2,
                                 ljforcefield.r2_cutoff, [sid[fmol.atom_species[0]]], sites[:, None, :])
    e = e_k * 8.314 / 1000.0                    # as the reference converts its grid (src/grid.jl:357)
    best = int(np.argmin(e))                    # first of the minima, in column-major order
    xf = id_to_xf(tuple(v + 1 for v in ids[best]), grid.n_pts)
    mol = Frac(molecule, crystal.box)
    translate_to(mol, xf)
    return mol, float(e[best])


def find_energy_minimum(crystal: Crystal, molecule: Molecule, ljforcefield: LJForceField, *, gtol: float = 1e-9,
                        max_iter: int = 500):
    """(molecule at the local minimum of the guest-host vdW energy (fractional, unit cell),
    minimum energy in kJ/mol), starting from the molecule's current centre of mass."""
    from scipy.optimize import minimize

    if needs_rotations(molecule):
        warnings.warn("needs rotations. does not optimize over configurations, only over center of mass")
    if molecule.n_charges > 0 and has_charges(crystal):
        raise ValueError("cannot handle electrostatics")
    rep = replication_factors(crystal.box, ljforcefield)
    sc = replicate(crystal, rep)
    fmol = Frac(molecule, crystal.box)                    # the guest in the unit cell
    xf0 = np.asarray(fmol.com, dtype=np.float64) / np.asarray(rep)   # supercell fraction
    system = GPUSystem(sc, Frac(molecule, sc.box), ljforcefield, None)
    ax, _ = _offsets(system)
    f_to_c = sc.box.f_to_c

    def energy_and_grad(xf):
        xf = np.mod(xf, 1.0)
        sites = (xf[None, :] + ax)[None, :, :]
        e, g = system.energies_grad(sites)
        u = float(e[0, 0])
        if not np.isfinite(u):
            return 1e30, np.zeros(3)
        # dU/dxf = f_to_c^T dU/dx (Cartesian gradient of the rigid guest)
        return u * K_TO_KJ, (f_to_c.T @ g[0].astype(np.float64)) * K_TO_KJ

    res = minimize(energy_and_grad, xf0, jac=True, method="L-BFGS-B",
                   options={"gtol": gtol, "maxiter": max_iter, "ftol": 1e-15})
    xf_min = np.mod(np.mod(res.x, 1.0) * np.asarray(rep), 1.0)
    mol = Frac(molecule, crystal.box)
    translate_to(mol, xf_min)
    return mol, float(res.fun)


def _offsets(system: GPUSystem):
    """Fractional offsets of the guest's LJ sites from its centre of mass in the system's box."""
    from .molecule import body_offsets

    ax, qx = body_offsets(system.molecule, system.crystal.box)
    c_to_f = system.crystal.box.c_to_f
    return np.asarray(ax) @ c_to_f.T, np.asarray(qx) @ c_to_f.T if len(qx) else qx
