"""Atomic masses (amu) for the crystal-density unit conversion of Henry coefficients.

Standard atomic weights of the elements plus the pseudo-atoms PorousMaterials.jl adds for
its molecule models (src/atomic_masses.jl:2-25).  Users can pass their own table to
crystal_density / henry_coefficient (`masses=`) to match another data set exactly.
"""
from __future__ import annotations

import re

ELEMENT_MASSES = {
    "H": 1.00794, "He": 4.002602, "Li": 6.941, "Be": 9.012182, "B": 10.811, "C": 12.0107,
    "N": 14.0067, "O": 15.9994, "F": 18.9984032, "Ne": 20.1797, "Na": 22.98976928, "Mg": 24.305,
    "Al": 26.9815386, "Si": 28.0855, "P": 30.973762, "S": 32.065, "Cl": 35.453, "Ar": 39.948,
    "K": 39.0983, "Ca": 40.078, "Sc": 44.955912, "Ti": 47.867, "V": 50.9415, "Cr": 51.9961,
    "Mn": 54.938045, "Fe": 55.845, "Co": 58.933195, "Ni": 58.6934, "Cu": 63.546, "Zn": 65.38,
    "Ga": 69.723, "Ge": 72.64, "As": 74.9216, "Se": 78.96, "Br": 79.904, "Kr": 83.798,
    "Rb": 85.4678, "Sr": 87.62, "Y": 88.90585, "Zr": 91.224, "Nb": 92.90638, "Mo": 95.96,
    "Tc": 98.0, "Ru": 101.07, "Rh": 102.9055, "Pd": 106.42, "Ag": 107.8682, "Cd": 112.411,
    "In": 114.818, "Sn": 118.71, "Sb": 121.76, "Te": 127.6, "I": 126.90447, "Xe": 131.293,
    "Cs": 132.9054519, "Ba": 137.327, "La": 138.90547, "Ce": 140.116, "Pr": 140.90765,
    "Nd": 144.242, "Pm": 145.0, "Sm": 150.36, "Eu": 151.964, "Gd": 157.25, "Tb": 158.92535,
    "Dy": 162.5, "Ho": 164.93032, "Er": 167.259, "Tm": 168.93421, "Yb": 173.054, "Lu": 174.9668,
    "Hf": 178.49, "Ta": 180.94788, "W": 183.84, "Re": 186.207, "Os": 190.23, "Ir": 192.217,
    "Pt": 195.084, "Au": 196.966569, "Hg": 200.59, "Tl": 204.3833, "Pb": 207.2, "Bi": 208.9804,
    "U": 238.02891,
}

PSEUDO_ATOM_MASSES = {
    "N_in_N2": 14.0067, "CH2": 14.025, "CH3": 15.035, "CH4": 16.04, "C_b": 12.0107,
    "C_tol": 12.0107, "C_ac": 12.0107, "C_RCOO": 12.0107, "C_sp2": 12.0107, "C_sp3": 12.0107,
    "C_CO2": 12.0107, "H_H2S": 1.00794, "H_b": 1.00794, "O_RCOO": 15.9994, "O_CO2": 15.9994,
    "O_zeo": 15.9994, "S_H2S": 32.065, "Si_zeo": 28.0855, "ig": 1.0, "X": 1.0,
}

DEFAULT_MASSES = {**ELEMENT_MASSES, **PSEUDO_ATOM_MASSES}


def atomic_mass(species: str, masses: dict | None = None) -> float:
    table = masses if masses is not None else DEFAULT_MASSES
    if species in table:
        return float(table[species])
    base = re.sub(r"[0-9]+$", "", species)
    if base in table:
        return float(table[base])
    raise KeyError(f"no atomic mass for species {species!r}")
