"""Test helpers: oracle systems that mirror a GPU system, random guest configurations."""
from __future__ import annotations

import math

import numpy as np

import oracle
import pmgb
from pmgb.molecule import body_offsets


def oracle_for(gs: "pmgb.GPUSystem", ljff_r2=None) -> oracle.OracleSystem:
    """FP64 oracle holding exactly the inputs of a GPU system."""
    cr = gs.crystal
    sid = {s: i for i, s in enumerate(gs.species)}
    fw_sp = [sid[s] for s in cr.atoms.species]
    g_sp = [sid[s] for s in gs.molecule.atom_species]
    r2 = gs.ljff.r2_cutoff if gs.ljff is not None else gs.eparams.sr_cutoff_r ** 2
    o = oracle.OracleSystem(cr.box.f_to_c, cr.atoms.xf, fw_sp, cr.charges.xf, cr.charges.q, gs._eps, gs._sig2,
                            r2 if ljff_r2 is None else ljff_r2, g_sp, gs.molecule.charge_q)
    if gs.eparams is not None:
        ep = gs.eparams
        o.set_ewald(ep.alpha, ep.sr_cutoff_r, ep.kreps, ep.kvec_abc, ep.kvec_wt)
    return o


def random_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    out = np.zeros((n, 3, 3))
    for i in range(n):
        out[i] = pmgb.random_rotation_matrix(rng)
    return out


def random_configs(gs: "pmgb.GPUSystem", n: int, seed: int):
    """Random poses -> (sites (n, n_sites, 3), lj_xf (n, n_atoms, 3), q_xf (n, n_charges, 3)) in FP64."""
    rng = np.random.default_rng(seed)
    box = gs.crystal.box
    xf = rng.random((n, 3))
    R = random_rotations(n, rng)
    ax, qx = body_offsets(gs.molecule, box)
    lj = xf[:, None, :] + np.einsum("ij,njk,lk->nli", box.c_to_f, R, ax) if ax.shape[0] else np.zeros((n, 0, 3))
    q = xf[:, None, :] + np.einsum("ij,njk,lk->nli", box.c_to_f, R, qx) if qx.shape[0] else None
    return gs.site_coords(lj, q), lj, q


def oracle_sites_split(gs, sites):
    """Split merged site coordinates back into LJ-atom and charge coordinates."""
    n = sites.shape[0]
    na, nq = gs.molecule.n_atoms, gs.molecule.n_charges
    lj = np.zeros((n, na, 3))
    q = np.zeros((n, nq, 3))
    for k in range(gs.n_sites):
        if gs.site_atom[k] >= 0:
            lj[:, gs.site_atom[k], :] = sites[:, k, :]
        if gs.site_charge[k] >= 0:
            q[:, gs.site_charge[k], :] = sites[:, k, :]
    return lj, q


def rel_err(a, b, floor=1e-300):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def within(a, b, rtol, atol):
    """Elementwise |a - b| <= max(rtol |b|, atol), with equal infinities allowed."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    ok = np.abs(a - b) <= np.maximum(rtol * np.abs(b), atol)
    return ok | both_inf


def deg(x):
    return math.radians(x)


def widom_with_oracle(gs, n_per_block, seed, T=298.0, use_sk=True, n_blocks=5):
    """GPU Widom blocks and per-insertion energies, and the oracle's FP64 energies of the exact
    device poses: (blocks, u (n, 2), U_vdw, U_es)."""
    from pmgb.molecule import body_offsets

    blocks, u = gs.widom(n_per_block, n_blocks, seed, T, want_energies=True)
    xf, rot = gs.ctx.sample_poses(seed, 0, n_blocks * n_per_block)
    # the device rotation is column-major R[i + 3j], the layout the oracle takes
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    o = oracle_for(gs)
    sites = o.sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    lj, q = oracle_sites_split(gs, sites)
    v, sr, lr = o.energies(lj, q, charged=gs.charged, use_sk=use_sk)
    return blocks, u, v, sr + lr
