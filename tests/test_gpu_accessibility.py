"""The accessibility gate of Widom insertions (henry_coefficient's accessibility_grid,
src/henry.jl:225 -> src/grid.jl:778-836) on the GPU against the oracle's restatement.

Blocked insertions get U_vdw = U_es = +Inf (henry.jl:230-233): they count in the block sizes
and the overlap counts, and carry no Boltzmann weight."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import pmgb
from pm_helpers import widom_with_oracle
from pmgb import synthetic
from pmgb.grid import Grid

pytestmark = pytest.mark.gpu
T = 298.0


def _system():
    cr = synthetic.config1_porous()
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    return cr, rep, pmgb.GPUSystem(sc, pmgb.Frac(synthetic.co2(), sc.box), ff, ep)


def _grid(cr, data):
    return Grid(cr.box, tuple(data.shape), data, "K", np.zeros(3))


def test_gate_matches_oracle():
    cr, rep, gs = _system()
    rng = np.random.default_rng(5)
    data = rng.random((9, 11, 7)) < 0.02  # sparse accessible nodes: many insertions blocked
    gs.set_accessibility(_grid(cr, data), rep)
    gs.set_refine(1e-3)
    npb, seed = 8000, 61
    blocks, u, v, es = widom_with_oracle(gs, npb, seed, T)
    xf, _ = gs.ctx.sample_poses(seed, 0, 5 * npb)
    ok = oracle.accessible(data, xf.astype(np.float64), rep)
    assert 0.05 < ok.mean() < 0.95
    v = np.where(ok, v, np.inf)
    es = np.where(ok, es, np.inf)
    # blocked insertions carry U_es = +Inf (an LJ overlap alone leaves U_es finite)
    np.testing.assert_array_equal(np.isinf(u[:, 1]), ~ok)
    ref = oracle.widom_blocks_log(v, es, T, 5, npb)
    np.testing.assert_array_equal(blocks[:, 3], ref[:, 3])
    assert np.abs(blocks[:, 0] - ref[:, 0]).max() <= 1e-6
    assert gs.ctx.device_status() == 0


def test_gate_all_open_and_all_closed():
    cr, rep, gs = _system()
    npb, seed = 3000, 62
    free, _ = gs.widom(npb, 5, seed, T)
    gs.set_accessibility(_grid(cr, np.ones((5, 6, 4), dtype=bool)), rep)
    opened, _ = gs.widom(npb, 5, seed, T)
    np.testing.assert_array_equal(opened, free)
    gs.set_accessibility(_grid(cr, np.zeros((5, 6, 4), dtype=bool)), rep)
    closed, u = gs.widom(npb, 5, seed, T, want_energies=True)
    assert np.all(closed[:, 0] == -np.inf) and np.all(closed[:, 3] == npb)
    assert np.all(np.isinf(u))
    gs.set_accessibility(None, rep)
    again, _ = gs.widom(npb, 5, seed, T)
    np.testing.assert_array_equal(again, free)


def test_drop_in_with_accessibility_grid():
    cr, rep, _ = _system()
    ff = synthetic.forcefield()
    data = np.random.default_rng(6).random((9, 11, 7)) < 0.02  # sparse: the 27-node rule blocks ~half
    res = pmgb.henry_coefficient(cr, synthetic.co2(), T, ff, insertions_per_volume=5000 / cr.box.Omega,
                                 verbose=False, autosave=False, seed=9, accessibility_grid=_grid(cr, data))
    full = pmgb.henry_coefficient(cr, synthetic.co2(), T, ff, insertions_per_volume=5000 / cr.box.Omega,
                                  verbose=False, autosave=False, seed=9)
    assert res.n_overlaps > full.n_overlaps
    assert res["henry coefficient [mol/(m³-bar)]"] < full["henry coefficient [mol/(m³-bar)]"]
    wrong = Grid(pmgb.Box(10.0, 10.0, 10.0, np.pi / 2, np.pi / 2, np.pi / 2), data.shape, data, "K", np.zeros(3))
    with pytest.raises(ValueError, match="accessibility grid box"):
        pmgb.henry_coefficient(cr, synthetic.co2(), T, ff, insertions_per_volume=10, verbose=False,
                               autosave=False, accessibility_grid=wrong)


# ---- compute_accessibility_grid: the reference's own expectations (test/grid.jl:43-146) ----
def _uff_ch4():
    return pmgb.LJForceField("UFF"), pmgb.read_molecule("CH4")


@pytest.mark.parametrize("zeolite", ["LTA", "SOD"])
def test_accessibility_grid_zeolites(zeolite):
    ff, ch4 = _uff_ch4()
    cr = pmgb.read_cif(f"{zeolite}.cif")
    acc, nb, por = pmgb.compute_accessibility_grid(cr, ch4, ff, resolution=2.0, energy_tol=0.0, verbose=False,
                                                   write_b4_after_grids=True)
    print(f"[{zeolite}] blocked segments {nb}; porosity {por}")
    assert nb > 0
    if zeolite == "LTA":
        assert nb == 8
    assert por["b4_blocking"] > por["after_blocking"]
    assert np.allclose(acc.box.f_to_c, cr.box.f_to_c)
    if zeolite == "SOD":
        assert not acc.data.any()
    # random insertions: the gate with and without unit repfactors agree
    xf = np.random.default_rng(3).random((20000, 3))
    a1 = oracle.accessible(acc.data, xf, (1, 1, 1))
    if zeolite == "SOD":
        assert not a1.any()
    acc_nb, nb_nb, por_nb = pmgb.compute_accessibility_grid(cr, ch4, ff, resolution=2.0, energy_tol=0.0,
                                                            verbose=False, write_b4_after_grids=False,
                                                            block_inaccessible_pockets=False)
    assert nb_nb == 0
    assert por_nb > por["after_blocking"]
    assert por_nb == pytest.approx(por["b4_blocking"])


def test_accessibility_grid_replication():
    ff, ch4 = _uff_ch4()
    cr = pmgb.read_cif("LTA.cif")
    acc, nb, _ = pmgb.compute_accessibility_grid(cr, ch4, ff, resolution=2.0, energy_tol=0.0, verbose=False,
                                                 write_b4_after_grids=False)
    rep = (2, 3, 1)
    rep_acc, rep_nb, _ = pmgb.compute_accessibility_grid(pmgb.replicate(cr, rep), ch4, ff, resolution=2.0,
                                                         energy_tol=0.0, verbose=False, write_b4_after_grids=False)
    assert np.array_equal(acc.data, rep_acc.data[:7, :7, :7])
    assert rep_nb > 0
    xf = np.random.default_rng(4).random((10000, 3))
    np.testing.assert_array_equal(oracle.accessible(rep_acc.data, xf, (1, 1, 1)),
                                  oracle.accessible(acc.data, xf, rep))


@pytest.mark.parametrize("name", ["SBMOF-1", "CAXVII_clean"])
def test_accessibility_grid_no_pockets(name):
    ff, ch4 = _uff_ch4()
    cr = pmgb.read_cif(f"{name}.cif")
    acc, nb, por = pmgb.compute_accessibility_grid(cr, ch4, ff, energy_tol=5.0, verbose=False,
                                                   write_b4_after_grids=True, energy_units="kJ_mol")
    assert nb == 0
    acc_nb, nb_nb, por_nb = pmgb.compute_accessibility_grid(cr, ch4, ff, energy_tol=5.0, verbose=False,
                                                            energy_units="kJ_mol", write_b4_after_grids=True,
                                                            block_inaccessible_pockets=False)
    assert por_nb == pytest.approx(por["b4_blocking"])
    assert nb_nb == 0
    assert np.array_equal(acc.data, acc_nb.data)
