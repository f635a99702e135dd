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
from .system import GPUSystem

K_TO_KJ = 8.314 / 1000.0  # energy_min.jl:49 (the grid factor, not R)


N_CANDIDATES = 16  # lowest grid points re-evaluated at full precision before the argmin


def find_energy_minimum_gridsearch(crystal: Crystal, molecule: Molecule, ljforcefield: LJForceField, *,
                                   resolution=1.0, n_pts=None):
    """(molecule at the lowest grid point (fractional), that energy in kJ/mol).  n_pts is the
    keyword the reference's test passes (test/energy_min.jl:20); resolution is the function's.

    The grid holds FP32 values; the lowest N_CANDIDATES points are re-evaluated in double-float
    (pmgb_energies, FP64-grade) and the minimum is taken over those values, the first in
    column-major order on a tie, as Julia's findmin over an FP64 grid."""
    res = n_pts if n_pts is not None else resolution
    grid = energy_grid(crystal, molecule, ljforcefield, resolution=res, verbose=False, units="kJ_mol")
    data = np.asarray(grid.data)
    flat = data.ravel(order="F")
    k = min(N_CANDIDATES, flat.size)
    cand = np.sort(np.argpartition(flat, k - 1)[:k])           # column-major order
    ids = [np.unravel_index(int(c), data.shape, order="F") for c in cand]
    xfs = np.array([id_to_xf(tuple(int(i) + 1 for i in idx), grid.n_pts) for idx in ids])
    rep = replication_factors(crystal.box, ljforcefield)
    sc = replicate(crystal, rep)
    system = GPUSystem(sc, Frac(molecule, sc.box), ljforcefield, None)
    ax, _ = _offsets(system)
    sites = (np.mod(xfs, 1.0) / np.asarray(rep))[:, None, :] + ax[None, :, :]
    e = system.energies(sites)[:, 0] * K_TO_KJ
    best = int(np.argmin(np.where(np.isfinite(e), e, np.inf)))
    mol = Frac(molecule, crystal.box)
    translate_to(mol, xfs[best])
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
