"""Rotational energy grids (energy_grid for probes that need rotations, src/grid.jl:338-351).

At each grid point the probe takes n_rotations orientations; the grid holds
-T log(Σ_r e^{-U_r/T} / n_rotations).  The oracle evaluates the same orientations (drawn by
pmgb_sample_poses at counters p * n_rotations + r) at the same FP64 grid positions in FP64, and
every point must agree within 1e-5 relative or 1e-4 K.
"""
from __future__ import annotations

import numpy as np
import pytest

import pmgb
from pm_helpers import oracle_for, oracle_sites_split, within
from pmgb import synthetic
from pmgb.molecule import body_offsets

pytestmark = pytest.mark.gpu
T = 298.0


def _system(cr, mol):
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    charged = pmgb.crystal.has_charges(sc) and mol.n_charges > 0
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    return pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep), rep


def _grid_points(n_pts, rep):
    """FP64 supercell fractions of the grid points, i fastest (the end plane folded onto the first)."""
    ax = []
    for n, r in zip(n_pts, rep):
        f = np.arange(n) / (n - 1) if n > 1 else np.zeros(1)
        ax.append(np.where(f >= 1.0, f - 1.0, f) / r)
    k, j, i = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.stack([i, j, k], axis=-1).reshape(-1, 3)


def _oracle_points(gs, seed, n_pts, rep, n_rot, points):
    """Oracle -T log⟨e^{-U/T}⟩ at the given flat point indices, over the device's orientations."""
    o = oracle_for(gs)
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    xyz = _grid_points(n_pts, rep)
    out = []
    for p in points:
        _, rot = gs.ctx.sample_poses(seed, int(p) * n_rot, n_rot)
        com = np.repeat(xyz[p][None, :], n_rot, axis=0)
        sites = o.sites_from_poses(com, rot.astype(np.float64), body)
        lj, q = oracle_sites_split(gs, sites)
        v, sr, lr = o.energies(lj, q, charged=gs.charged, use_sk=True)
        u = v + sr + lr
        x = np.where(np.isfinite(u), -u / T, -np.inf)
        m = x.max()
        out.append(np.inf if not np.isfinite(m) else -T * (m + np.log(np.mean(np.exp(x - m)))))
    return np.array(out)


@pytest.mark.parametrize("case", ["co2_ewald_porous", "co2_uncharged_config0"])
def test_rotational_grid_matches_oracle(case):
    cr = synthetic.config1_porous() if case == "co2_ewald_porous" else synthetic.config0()
    gs, rep = _system(cr, synthetic.co2())
    n_pts, n_rot, seed = (5, 4, 3), 200, 1234
    grid = gs.energy_grid_rotational(n_pts, rep, n_rot, T, seed, 1.0)
    ref = _oracle_points(gs, seed, n_pts, rep, n_rot, range(int(np.prod(n_pts))))
    got = grid.transpose(2, 1, 0).reshape(-1).astype(np.float64)   # i fastest
    err = np.abs(got - ref)
    fin = np.isfinite(ref)
    print(f"[rot grid {case}] max |d| {err[fin].max():.3e} K, values {np.quantile(ref[fin], [0, .5, 1])}")
    assert np.array_equal(np.isinf(got), np.isinf(ref))
    assert within(got, ref, 1e-5, 1e-4).all()
    # kJ/mol as the reference's factor; a repeat gives the same values bit for bit
    kj = gs.energy_grid_rotational(n_pts, rep, n_rot, T, seed, 8.314 / 1000.0)
    np.testing.assert_allclose(kj, grid * (8.314 / 1000.0), rtol=2e-7)
    np.testing.assert_array_equal(gs.energy_grid_rotational(n_pts, rep, n_rot, T, seed, 1.0), grid)


def test_rotational_grid_in_slices():
    """Many orientations per point: the points run in several launches; each point keeps its own
    orientations (counters p * n_rotations + r) whatever the slice it falls in."""
    gs, rep = _system(synthetic.config0(), synthetic.co2())
    n_pts, n_rot, seed = (5, 5, 5), 131072, 99     # 64 points per launch: two launches
    grid = gs.energy_grid_rotational(n_pts, rep, n_rot, T, seed, 1.0)
    flat = grid.transpose(2, 1, 0).reshape(-1).astype(np.float64)
    pts = [3, 100]                                  # one point of each launch
    ref = _oracle_points(gs, seed, n_pts, rep, n_rot, pts)
    print(f"[rot grid slices] gpu {flat[pts]} oracle {ref}")
    assert within(flat[pts], ref, 1e-5, 1e-4).all()


def test_rotational_grid_drop_in_and_errors():
    cr = synthetic.config1_porous()
    co2 = synthetic.co2()
    ff = synthetic.forcefield()
    with pytest.raises(ValueError, match="temperature"):
        pmgb.energy_grid(cr, co2, ff, resolution=(3, 3, 3), verbose=False)
    g = pmgb.energy_grid(cr, co2, ff, resolution=(3, 3, 3), n_rotations=64, temperature=T, units="K",
                         verbose=False, seed=5)
    assert g.data.shape == (3, 3, 3) and np.all(np.isfinite(g.data) | (g.data > 0))
    gs, rep = _system(cr, co2)
    for bad in (dict(n_rotations=0), dict(temperature=0.0), dict(temperature=float("nan"))):
        kw = dict(n_rotations=8, temperature=T)
        kw.update(bad)
        with pytest.raises(pmgb.PMGBError):
            gs.energy_grid_rotational((3, 3, 3), rep, kw["n_rotations"], kw["temperature"], 1, 1.0)
