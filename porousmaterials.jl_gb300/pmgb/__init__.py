"""pmgb -- GB300-native Widom-insertion Henry coefficients and energy grids.

The Python face of libpmgb.so, with the names and semantics of PorousMaterials.jl's
public functions on this path (henry_coefficient, energy_grid, vdw_energy,
electrostatic_potential_energy, setup_Ewald_sum, LJForceField, replication_factors, ...).
All energies are computed by the sm_103a CUDA library; there is no CPU fallback.
"""
from ._lib import Context, PMGBError
from .crystal import (Atoms, Box, Charges, Crystal, assert_P1_symmetry, crystal_density, has_charges,
                      net_charge, read_cif, replicate, replicate_box, strip_numbers_from_atom_labels)
from .energetics import (Eikr, EwaldSum, PotentialEnergy, electrostatic_potential_energy,
                         guest_host_energies, total, vdw_energy)
from .ewald import (EPS0, FOUR_PI_EPS0, EwaldParams, determine_ewald_params, precompute_kvec_wts,
                    required_kreps, setup_Ewald_sum)
from .energy_min import find_energy_minimum, find_energy_minimum_gridsearch
from .forcefield import LJForceField, forcefield_coverage, replication_factors
from .grid import (Grid, accessible, compute_accessibility_grid, energy_grid, id_to_xf, read_cube,
                   required_n_pts, write_cube, xf_to_id)
from .henry import (K_TO_KJ_PER_MOL, N_BLOCKS, UNIV_GAS_CONST, HenryResult, henry_coefficient,
                    henry_coefficient_gradient)
from .molecule import (Cart, Frac, Molecule, molecule_from_sites, needs_rotations, random_rotation_matrix,
                       read_molecule, translate_to)
from .paths import rc, set_paths
from .system import GPUSystem

__all__ = [n for n in dir() if not n.startswith("_")]
