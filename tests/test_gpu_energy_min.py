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
    # FIQCEN's lowest grid points 3/14 and 11/14 (per axis) are inversion images with energies
    # equal in exact arithmetic; the FP64 re-evaluation in the reference's operation order tells
    # them apart as the reference does (test/energy_min.jl:22)
    np.testing.assert_allclose(gs_mol.com, [0.785, 0.785, 0.785], atol=0.05)
    mol, e = pmgb.find_energy_minimum(cr, gs_mol, ff)
    print(f"[FIQCEN] minimum {e:.4f} kJ/mol at {mol.com}")
    assert e == pytest.approx(-27.0269, abs=0.01)
    assert e < gs_e
    np.testing.assert_allclose(mol.com, [0.75, 0.75, 0.75], atol=0.001)
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


def _ordered_fp64(f2c, axf, e_x, s_x, r2c, xi):
    """The reference's vdw_energy (src/vdw_energetics.jl:25-47) for one site in plain FP64, every
    operation rounded separately, the atoms summed in order."""
    d = axf - xi[None, :]
    m = np.abs(d) > 0.5
    d[m] -= np.sign(d[m])
    c = [(f2c[k, 0] * d[:, 0] + f2c[k, 1] * d[:, 1]) + f2c[k, 2] * d[:, 2] for k in range(3)]
    r2 = (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]
    e = 0.0
    for j in np.flatnonzero(r2 < r2c):
        if r2[j] < 0.1:
            return np.inf
        u = s_x[j] / r2[j]
        t = (u * u) * u
        e += ((4.0 * e_x[j]) * t) * (t - 1.0)
    return e


def test_vdw_energy_ordered_bitwise(ctx):
    """pmgb_vdw_energy_ordered equals the plain FP64 restatement bit for bit, overlaps included."""
    xe, ff = _xe_uff()
    cr = pmgb.read_cif("FIQCEN_clean.cif")
    pmgb.strip_numbers_from_atom_labels(cr)
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    species = sorted(set(sc.atoms.species) | {"Xe"})
    sid = {s: i for i, s in enumerate(species)}
    eps, sig2 = ff.tables(species)
    rng = np.random.default_rng(5)
    pts = rng.random((200, 3))
    pts[:3] = sc.atoms.xf[:3] + 1e-4          # overlaps: +Inf
    pts[3] = [3 / 28, 3 / 28, 3 / 28]         # the inversion pair of the grid search
    pts[4] = [11 / 28, 11 / 28, 11 / 28]
    got = ctx.vdw_energy_ordered(sc.box.f_to_c, sc.atoms.xf, [sid[s] for s in sc.atoms.species], eps, sig2,
                                 ff.r2_cutoff, [sid["Xe"]], pts[:, None, :])
    e_x = np.array([eps[sid["Xe"], sid[s]] for s in sc.atoms.species])
    s_x = np.array([sig2[sid["Xe"], sid[s]] for s in sc.atoms.species])
    ref = np.array([_ordered_fp64(sc.box.f_to_c, np.asarray(sc.atoms.xf), e_x, s_x, ff.r2_cutoff, p) for p in pts])
    assert np.isinf(got[:3]).all()
    assert np.array_equal(got, ref), f"max |diff| {np.nanmax(np.abs(got - ref)[np.isfinite(ref)]):.3e}"
    assert got[4] < got[3]                     # the reference's FP64 pick (test/energy_min.jl:22)
