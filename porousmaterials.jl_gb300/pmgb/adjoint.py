"""Derivatives of the Henry coefficient (the adjoint path).

K_H = mean over blocks of Σ_i e^{-U_i/T} / (R T n_b) (src/henry.jl:120,141), so
dK_H/dθ = -Σ_i e^{-U_i/T} ∂U_i/∂θ / (T R T n_b N_blocks).  The device returns the
Boltzmann-weighted sums Σ w_i ∂U_i/∂ε_ab and Σ w_i ∂U_i/∂σ²_ab per (guest, framework) species
pair (w_i = e^{-U_i/T - M}); this module applies the force field's mixing rule to reach the
pure-species parameters ε_s, σ_s, and the framework-charge scale λ (∂U_es/∂λ = U_es).  This is
the Python counterpart of the rrule the Julia binding registers with ChainRulesCore.
"""
from __future__ import annotations

import math

import numpy as np

from .forcefield import LJForceField


def mixing_jacobians(ljff: LJForceField, species: list[str]):
    """∂ε_ab/∂ε_s and ∂σ²_ab/∂σ_s as arrays of shape (n, n, n) [a, b, s]."""
    n = len(species)
    eps = np.array([ljff.pure_epsilon[s] for s in species])
    sig = np.array([ljff.pure_sigma[s] for s in species])
    de = np.zeros((n, n, n))
    ds = np.zeros((n, n, n))
    rule = ljff.mixing_rules.lower()
    for a in range(n):
        for b in range(n):
            for s in (a, b) if a != b else (a,):
                if rule in ("lorentz-berthelot", "geometric"):
                    # ε_ab = sqrt(ε_a ε_b)
                    if a == b:
                        de[a, b, s] = 1.0
                    else:
                        de[a, b, s] = 0.5 * math.sqrt(eps[a] * eps[b]) / eps[s] if eps[s] > 0 else 0.0
                    if rule == "lorentz-berthelot":
                        ds[a, b, s] = 2.0 * sig[a] if a == b else 0.5 * (sig[a] + sig[b])
                    else:  # σ²_ab = σ_a σ_b
                        ds[a, b, s] = 2.0 * sig[a] if a == b else sig[b if s == a else a]
                else:
                    raise NotImplementedError(f"derivatives through {ljff.mixing_rules} mixing")
    return de, ds


def henry_gradients(system, block_out, adj: dict, temperature: float, n_per_block: int):
    """dK_H/dε_s, dK_H/dσ_s (per species name, for K_H in mol/(m³ bar)) and dK_H/dλ."""
    from .henry import UNIV_GAS_CONST

    n_blocks = block_out.shape[0]
    scale = -math.exp(adj["log_scale"]) / (temperature * UNIV_GAS_CONST * temperature * n_per_block * n_blocks)
    de, ds = mixing_jacobians(system.ljff, system.species)
    d_eps_ab = adj["d_eps"] * scale
    d_sig2_ab = adj["d_sig2"] * scale
    d_eps_s = np.einsum("ab,abs->s", d_eps_ab, de)
    d_sig_s = np.einsum("ab,abs->s", d_sig2_ab, ds)
    return ({s: float(d_eps_s[i]) for i, s in enumerate(system.species)},
            {s: float(d_sig_s[i]) for i, s in enumerate(system.species)},
            float(adj["sum_w_ues"] * scale))
