"""henry_coefficient: Widom insertions on the GPU behind the reference's signature.

Mirrors src/henry.jl:34-181 (set-up, block statistics, result keys and units) with the
insertion loop of _conduct_Widom_insertions (:185-265) replaced by one libpmgb launch.
Differences from the reference, by design:
  * insertion poses come from Philox4x32-10 keyed by (seed, insertion index) instead of
    Julia's global RNG, so a run is reproducible from `seed`;
  * each insertion applies a fresh uniform rotation to the molecule's reference
    orientation (the reference composes rotations, which has the same uniform
    distribution), so there is no bond-length drift to check (henry.jl:247-261);
  * the five statistics blocks are CTAs on one GPU instead of Julia worker processes;
  * pair terms are FP32 (the reference is FP64); the insertions carrying all but
    `refine_tail` of each block's Boltzmann weight are re-evaluated in FP64, so K_H and
    <U> agree with an FP64 evaluation of the same insertions to ~1e-8.
"""
from __future__ import annotations

import json
import math
import os
import secrets
import time
from pathlib import Path

import numpy as np

from .crystal import Crystal, assert_P1_symmetry, crystal_density, has_charges, replicate
from .ewald import setup_Ewald_sum
from .forcefield import LJForceField, replication_factors
from .molecule import Frac, Molecule
from .paths import rc
from .system import GPUSystem

UNIV_GAS_CONST = 8.3144598e-5   # m³ bar / (K mol), src/PorousMaterials.jl:11
K_TO_KJ_PER_MOL = 8.3144598e-3  # kJ / (mol K), src/PorousMaterials.jl:12
N_BLOCKS = 5                    # src/mc_helpers.jl:11
# Boltzmann weight per block left to the FP32 energies; the rest is re-evaluated in FP64, which
# holds K_H and <U> to ~1e-8 of the FP64 result (pmgb_system_set_refine)
REFINE_TAIL = 1e-3


class HenryResult(dict):
    """The reference's result Dict (same 16 keys) plus run details as attributes."""

    blocks: np.ndarray
    seed: int
    n_insertions_per_block: int
    repfactors: tuple
    n_overlaps: int


def henry_result_savename(crystal: Crystal, molecule: Molecule, temperature: float, ljff: LJForceField,
                          insertions_per_volume, comment: str = "") -> str:
    """File name of the saved result (src/henry.jl:286-294), JSON instead of JLD2."""
    if comment and not comment.startswith("_"):
        comment = "_" + comment
    return (f"henry_sim_{molecule.species}_in_{crystal.name}_{temperature:f}K_{ljff.name}_ff_"
            f"{int(insertions_per_volume)}_insertions_per_volume{comment}.json")


def _std(x: np.ndarray) -> float:
    return float(np.std(x, ddof=1)) if len(x) > 1 else 0.0


def henry_coefficient(crystal: Crystal, molecule: Molecule, temperature: float, ljforcefield: LJForceField, *,
                      insertions_per_volume: float = 200, verbose: bool = True, ewald_precision: float = 1e-6,
                      autosave: bool = True, filename_comment: str = "", accessibility_grid=None,
                      seed: int | None = None, masses: dict | None = None, system_out: list | None = None,
                      refine_tail: float = REFINE_TAIL) -> HenryResult:
    assert_P1_symmetry(crystal)
    if accessibility_grid is not None and not np.allclose(accessibility_grid.box.f_to_c, crystal.box.f_to_c,
                                                          rtol=1e-6, atol=1e-6):
        raise ValueError(f"accessibility grid box does not match box of {crystal.name}.")  # henry.jl:58-61
    t0 = time.time()
    temperature = float(temperature)
    if verbose:
        print(f"Simulating Henry coefficient of {molecule.species} in {crystal.name} at {temperature} K, using "
              f"{ljforcefield.name} force field with {insertions_per_volume} insertions per Å³.")
        if accessibility_grid is not None:
            print("Using provided accessibility grid to block inaccessible pockets")
    nb_insertions = max(N_BLOCKS, math.ceil(insertions_per_volume * crystal.box.Omega))
    if verbose:
        print(f"\t{nb_insertions} total # particle insertions")
    nb_per_block = math.ceil(nb_insertions / N_BLOCKS)
    repfactors = replication_factors(crystal.box, ljforcefield)
    if verbose:
        print(f"\tReplicating crystal {repfactors[0]} by {repfactors[1]} by {repfactors[2]} for short-range "
              f"cutoff {ljforcefield.r_cutoff:.2f}")
    charged = has_charges(crystal) and molecule.n_charges > 0
    rho = crystal_density(crystal, masses)  # the supercell's density is the unit cell's
    if seed is None:
        seed = secrets.randbits(63)
    # replication, the supercell and the Ewald set-up natively (pmgb_system_create_unitcell)
    system = GPUSystem.from_unit_cell(crystal, molecule, ljforcefield, ewald_precision=ewald_precision,
                                      refine_tail=refine_tail)
    assert system.repfactors == tuple(repfactors)
    if verbose and charged:
        setup_Ewald_sum(system.crystal.box, ljforcefield.r_cutoff, eps=ewald_precision, verbose=True)
    if accessibility_grid is not None:
        system.set_accessibility(accessibility_grid, repfactors)
    if system_out is not None:
        system_out.append(system)
    blocks, _ = system.widom(nb_per_block, N_BLOCKS, seed, temperature)

    log_bf = blocks[:, 0]
    avg_vdw, avg_es = blocks[:, 1], blocks[:, 2]
    # K_H,b = Σ_b e^{-βU} / (R T n_b), henry.jl:120, evaluated from log Σ e^{-βU}
    kh = np.exp(log_bf - math.log(UNIV_GAS_CONST * temperature * nb_per_block))
    if not charged:
        avg_es = np.zeros_like(avg_es)
    if verbose:
        for b in range(N_BLOCKS):
            print(f"\tBlock  {b + 1}/{N_BLOCKS} statistics:")
            print(f"\tHenry coeff. [mmol/(g-bar)]: {kh[b] / rho}")
            print(f"\t⟨U, vdw⟩ (K): {avg_vdw[b]}")
            print(f"\t⟨U, es⟩ (K): {avg_es[b]}")
    elapsed = time.time() - t0
    err_kh = 2.0 * _std(kh) / math.sqrt(N_BLOCKS)
    err_vdw = 2.0 * _std(avg_vdw) / math.sqrt(N_BLOCKS)
    err_es = 2.0 * _std(avg_es) / math.sqrt(N_BLOCKS)

    r = HenryResult()
    r["henry coefficient [mol/(m³-bar)]"] = float(np.mean(kh))
    r["xtal"] = crystal.name
    r["henry coefficient [mmol/(g-bar)]"] = r["henry coefficient [mol/(m³-bar)]"] / rho
    r["err henry coefficient [mmol/(g-bar)]"] = err_kh / rho
    r["henry coefficient [mol/(kg-Pa)]"] = r["henry coefficient [mmol/(g-bar)]"] / 100000.0
    r["⟨U, vdw⟩ (K)"] = float(np.mean(avg_vdw))
    r["⟨U, es⟩ (K)"] = float(np.mean(avg_es))
    r["⟨U⟩ (K)"] = r["⟨U, vdw⟩ (K)"] + r["⟨U, es⟩ (K)"]
    r["⟨U⟩ (kJ/mol)"] = r["⟨U⟩ (K)"] * K_TO_KJ_PER_MOL
    r["⟨U, vdw⟩ (kJ/mol)"] = r["⟨U, vdw⟩ (K)"] * K_TO_KJ_PER_MOL
    r["err ⟨U, vdw⟩ (kJ/mol)"] = err_vdw * K_TO_KJ_PER_MOL
    r["⟨U, es⟩ (kJ/mol)"] = r["⟨U, es⟩ (K)"] * K_TO_KJ_PER_MOL
    r["err ⟨U, es⟩ (kJ/mol)"] = err_es * K_TO_KJ_PER_MOL
    r["Qst (kJ/mol)"] = -r["⟨U⟩ (kJ/mol)"] + temperature * K_TO_KJ_PER_MOL
    r["err Qst (kJ/mol)"] = (err_vdw + err_es) * K_TO_KJ_PER_MOL
    r["elapsed time (min)"] = elapsed / 60.0
    r.blocks = blocks
    r.seed = int(seed)
    r.n_insertions_per_block = nb_per_block
    r.repfactors = repfactors
    r.n_overlaps = int(blocks[:, 3].sum())

    if autosave:
        d = Path(rc["paths"]["simulations"])
        d.mkdir(parents=True, exist_ok=True)
        name = henry_result_savename(crystal, molecule, temperature, ljforcefield, insertions_per_volume,
                                     filename_comment)
        with open(d / name, "w") as f:
            json.dump(dict(r), f, indent=1)
        if verbose:
            print(f"\tResults saved in: {os.path.join(d, name)}")
    if verbose:
        print(f"\tElapsed time (min): {r['elapsed time (min)']}")
        print("\t----- final results ----")
        for key in ["henry coefficient [mmol/(g-bar)]", "⟨U, vdw⟩ (kJ/mol)", "⟨U, es⟩ (kJ/mol)", "Qst (kJ/mol)"]:
            print(f"\t{key} = {r[key]:f} +/- {r['err ' + key]:f}")
    return r


def henry_coefficient_gradient(crystal: Crystal, molecule: Molecule, temperature: float,
                               ljforcefield: LJForceField, *, insertions_per_volume: float = 200,
                               ewald_precision: float = 1e-6, seed: int | None = None,
                               want_forces: bool = False, system_out: list | None = None,
                               refine_tail: float = REFINE_TAIL):
    """K_H and its derivatives from one adjoint pass (pair terms recomputed, not stored).

    Returns a dict: 'henry coefficient [mol/(m³-bar)]' (block mean, as henry_coefficient),
    'dKH/d epsilon' and 'dKH/d sigma' (per species, the pure LJ parameters, through the force
    field's mixing rule), 'dKH/d charge scale' (framework charges scaled by λ at λ = 1), and
    with want_forces the per-insertion dU/dx of the centre of mass (K/Å; force = -dU/dx)."""
    from .adjoint import henry_gradients

    assert_P1_symmetry(crystal)
    temperature = float(temperature)
    nb_insertions = max(N_BLOCKS, math.ceil(insertions_per_volume * crystal.box.Omega))
    nb_per_block = math.ceil(nb_insertions / N_BLOCKS)
    charged = has_charges(crystal) and molecule.n_charges > 0
    if seed is None:
        seed = secrets.randbits(63)
    system = GPUSystem.from_unit_cell(crystal, molecule, ljforcefield, ewald_precision=ewald_precision,
                                      refine_tail=refine_tail)
    if system_out is not None:
        system_out.append(system)
    blocks, adj = system.widom_adjoint(nb_per_block, N_BLOCKS, seed, temperature, want_grad=want_forces)
    kh = np.exp(blocks[:, 0] - math.log(UNIV_GAS_CONST * temperature * nb_per_block))
    d_eps, d_sig, d_lam = henry_gradients(system, blocks, adj, temperature, nb_per_block)
    out = {"henry coefficient [mol/(m³-bar)]": float(np.mean(kh)), "dKH/d epsilon": d_eps, "dKH/d sigma": d_sig,
           "dKH/d charge scale": d_lam if charged else 0.0, "blocks": blocks, "seed": int(seed),
           "n_insertions_per_block": nb_per_block}
    if want_forces:
        out["dU/dx"] = adj["grad"]
    return out
