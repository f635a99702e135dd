"""Single-configuration guest-host energies on the GPU.

Drop-ins for vdw_energy(crystal, molecule, ljff) (src/vdw_energetics.jl:62-64 -> 25-47)
and electrostatic_potential_energy(crystal, molecule, eparams, eikr)
(src/electrostatics.jl:331-342 -> _ϕ :347-388).  As in the reference, `crystal` is
already replicated for the cutoff and `molecule` holds coordinates in that crystal's
box.  Batched forms take many configurations in one launch.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .crystal import Crystal
from .ewald import EwaldParams
from .forcefield import LJForceField
from .molecule import Frac, Molecule
from .system import GPUSystem


@dataclass
class PotentialEnergy:
    """(vdw, es) energy pair in K (src/energy_utilities.jl:4-16)."""
    vdw: float = 0.0
    es: float = 0.0

    def sum(self) -> float:
        return self.vdw + self.es

    def __add__(self, o):
        return PotentialEnergy(self.vdw + o.vdw, self.es + o.es)

    def __sub__(self, o):
        return PotentialEnergy(self.vdw - o.vdw, self.es - o.es)

    def __mul__(self, a: float):
        return PotentialEnergy(a * self.vdw, a * self.es)

    __rmul__ = __mul__

    def __truediv__(self, a: float):
        return PotentialEnergy(self.vdw / a, self.es / a)

    def isapprox(self, o, atol: float = 1e-6) -> bool:
        return abs(self.vdw - o.vdw) <= atol and abs(self.es - o.es) <= atol


@dataclass
class EwaldSum:
    """Short- and long-range parts of an Ewald potential energy (src/electrostatics.jl:9-16)."""
    sr: float = 0.0
    lr: float = 0.0


def total(e) -> float:
    if isinstance(e, EwaldSum):
        return e.sr + e.lr
    if isinstance(e, PotentialEnergy):
        return e.sum()
    return float(e)


class Eikr:
    """Accepted for signature compatibility; the GPU keeps S(k) instead of per-call e^{ik·r}."""

    def __init__(self, *args, **kwargs):
        pass


_cache: dict = {}


def _system(crystal: Crystal, molecule: Molecule, ljff: LJForceField | None, eparams: EwaldParams | None):
    key = (id(crystal), id(ljff), id(eparams), tuple(molecule.atom_species), molecule.n_charges,
           tuple(np.round(molecule.charge_q, 12)))
    hit = _cache.get(key)
    if hit is None:
        if len(_cache) > 8:
            _cache.clear()
        # the entry keeps its key objects alive so that their ids cannot be reused
        hit = (GPUSystem(crystal, molecule, ljff, eparams), (crystal, ljff, eparams))
        _cache[key] = hit
    return hit[0]


def _frac(molecule: Molecule, crystal: Crystal) -> Molecule:
    return molecule if molecule.frac else Frac(molecule, crystal.box)


def guest_host_energies(crystal: Crystal, molecules, ljff: LJForceField | None, eparams: EwaldParams | None = None):
    """(n, 3) array of (U_vdw, U_es sr, U_es lr) for a list of molecule configurations."""
    mols = [_frac(m, crystal) for m in molecules]
    sys_ = _system(crystal, mols[0], ljff, eparams)
    if sys_.charged and sys_.eparams is None:
        raise ValueError("framework and guest are charged: pass eparams (setup_Ewald_sum)")
    ax = np.stack([m.atom_x for m in mols]) if mols[0].n_atoms else np.zeros((len(mols), 0, 3))
    qx = np.stack([m.charge_x for m in mols]) if mols[0].n_charges else None
    return sys_.energies(sys_.site_coords(ax, qx))


def vdw_energy(crystal: Crystal, molecule: Molecule, ljff: LJForceField) -> float:
    m = _frac(molecule, crystal)
    if m.n_atoms == 0:
        return 0.0
    lj_only = Molecule(m.species, m.atom_species, m.atom_x, np.zeros(0), np.zeros((0, 3)), m.com, True)
    return float(guest_host_energies(crystal, [lj_only], ljff)[0, 0])


def electrostatic_potential_energy(crystal: Crystal, molecule: Molecule, eparams: EwaldParams,
                                   eikr: Eikr | None = None) -> EwaldSum:
    m = _frac(molecule, crystal)
    if m.n_charges == 0 or crystal.charges.n == 0:
        return EwaldSum(0.0, 0.0)
    q_only = Molecule(m.species, [], np.zeros((0, 3)), m.charge_q, m.charge_x, m.com, True)
    e = guest_host_energies(crystal, [q_only], None, eparams)[0]
    return EwaldSum(float(e[1]), float(e[2]))
