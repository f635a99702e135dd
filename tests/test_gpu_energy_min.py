"""Energy minimisation (src/energy_min.jl) against the reference's own expectations
(test/energy_min.jl:12-53): Xe in FIQCEN_clean with UFF and a cage in empty space."""
from __future__ import annotations

import numpy as np
import pytest

import pmgb

pytestmark = pytest.mark.gpu


def _xe_uff():
    return pmgb.read_molecule("Xe"), pmgb.LJForceField("UFF")


def test_fiqcen_xe():
    xe, ff = _xe_uff()
    cr = pmgb.read_cif("FIQCEN_clean.cif")
    pmgb.strip_numbers_from_atom_labels(cr)  # in place
    gs_mol, gs_e = pmgb.find_energy_minimum_gridsearch(cr, xe, ff, n_pts=(15, 15, 15))
    print(f"[FIQCEN] grid search {gs_e:.4f} kJ/mol at {gs_mol.com}")
    assert gs_e == pytest.approx(-25.1, abs=1.0)
    # FIQCEN's lowest grid points 3/14 and 11/14 (per axis) are inversion images with equal
    # energies: the reference's FP64 rounding picked 11/14 ([0.785]), FP32 rounding may pick
    # either, so the position is checked up to x -> 1 - x
    fold = lambda x: np.minimum(x, 1.0 - np.asarray(x))
    np.testing.assert_allclose(fold(gs_mol.com), fold([0.785, 0.785, 0.785]), atol=0.05)
    mol, e = pmgb.find_energy_minimum(cr, gs_mol, ff)
    print(f"[FIQCEN] minimum {e:.4f} kJ/mol at {mol.com}")
    assert e == pytest.approx(-27.0269, abs=0.01)
    assert e < gs_e
    np.testing.assert_allclose(fold(mol.com), fold([0.75, 0.75, 0.75]), atol=0.001)
    # the minimum's energy through the drop-in vdw_energy on the replicated crystal
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    cart = pmgb.Cart(mol, cr.box)
    assert pmgb.vdw_energy(sc, cart, ff) * 8.314 / 1000 == pytest.approx(e, abs=0.1)
    # from Cartesian coordinates too
    xe2 = pmgb.read_molecule("Xe")
    pmgb.translate_to(xe2, cr.box.f_to_c @ np.array([0.785, 0.785, 0.785]))
    mol2, e2 = pmgb.find_energy_minimum(cr, xe2, ff)
    assert e2 == pytest.approx(-27.0269, abs=0.01)
    np.testing.assert_allclose(mol2.com, [0.75, 0.75, 0.75], atol=0.001)


def test_cage_in_space():
    xe, ff = _xe_uff()
    cr = pmgb.read_cif("cage_in_space.cif")
    mol, e = pmgb.find_energy_minimum_gridsearch(cr, xe, ff, n_pts=(15, 15, 15))
    np.testing.assert_allclose(mol.com, [0.5, 0.5, 0.5], atol=0.1)
    mol, e = pmgb.find_energy_minimum(cr, mol, ff)
    print(f"[cage] minimum {e:.4f} kJ/mol at {mol.com}")
    assert e == pytest.approx(-38.55, abs=0.1)
    np.testing.assert_allclose(mol.com, [0.5, 0.5, 0.5], atol=0.1)
    rep = pmgb.replication_factors(cr.box, ff)
    assert pmgb.vdw_energy(pmgb.replicate(cr, rep), pmgb.Cart(mol, cr.box), ff) * 8.314 / 1000 == \
        pytest.approx(e, abs=0.1)
