"""Spatially ordered evaluation with cutoff culling (pmgb_system_set_cull).

The ordered path sorts each block's insertions by the Hilbert-curve cell of their centre of mass,
lets a warp skip framework records beyond the cutoff of all its items (whole chunks of records
by their bounding boxes in large cells, groups of four after their distances otherwise), and
forms the block sums in insertion order.  Skipped terms are exact zeros, so every per-insertion energy and
every block result must be bit-identical to the unordered path; likewise the energy grid with
brick-ordered warps.
"""
from __future__ import annotations

import numpy as np
import pytest

import pmgb
from pmgb import synthetic

pytestmark = pytest.mark.gpu
T = 298.0


def _system(cr, mol, charged):
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    return pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)


@pytest.mark.parametrize("case", ["co2_dense", "co2_porous", "ch4_config0", "co2_config4"])
@pytest.mark.parametrize("npb", [1, 257, 20000])
def test_culled_widom_is_bit_identical(case, npb):
    make = {"co2_dense": (synthetic.config1, synthetic.co2, True),
            "co2_porous": (synthetic.config1_porous, synthetic.co2, True),
            "ch4_config0": (synthetic.config0, synthetic.ch4, False),
            "co2_config4": (synthetic.config4, synthetic.co2, True)}[case]
    if case == "co2_config4" and npb > 257:
        npb = 4000  # 20,000 framework atoms: keep the unordered reference run short
    gs = _system(make[0](), make[1](), make[2])
    gs.set_image_lists(False)  # culling of the per-site pass (image lists: tests/test_gpu_image_lists.py)
    gs.set_cull(False)
    b0, u0 = gs.widom(npb, 5, 123, T, want_energies=True)
    gs.set_cull(True)
    b1, u1 = gs.widom(npb, 5, 123, T, want_energies=True)
    np.testing.assert_array_equal(u1, u0)
    np.testing.assert_array_equal(b1, b0)
    gs.set_refine(1e-3)  # with the FP64 tail refinement on top
    b2, _ = gs.widom(npb, 5, 123, T)
    gs.set_cull(False)
    b3, _ = gs.widom(npb, 5, 123, T)
    np.testing.assert_array_equal(b2, b3)
    assert gs.ctx.device_status() == 0


@pytest.mark.parametrize("n_pts", [(9, 8, 7), (33, 17, 5), (1, 1, 1), (48, 48, 48)])
def test_culled_grid_is_bit_identical(n_pts):
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.xe(), sc.box), ff)
    gs.set_exact(False)  # the FP32 grid kernels themselves, ordered and unordered
    gs.set_cull(False)
    g0 = gs.energy_grid(n_pts, rep, 1.0)
    gs.set_cull(True)
    g1 = gs.energy_grid(n_pts, rep, 1.0)
    np.testing.assert_array_equal(g1, g0)


@pytest.mark.parametrize("want_grad", [True, False])
@pytest.mark.parametrize("case", ["co2_porous", "ch4_config0", "co2_config4"])
def test_culled_adjoint_is_bit_identical(case, want_grad):
    # config4 (a 52 A cell) is large enough that whole chunks of records are skipped
    make = {"co2_porous": (synthetic.config1_porous, synthetic.co2, True),
            "ch4_config0": (synthetic.config0, synthetic.ch4, False),
            "co2_config4": (synthetic.config4, synthetic.co2, True)}[case]
    gs = _system(make[0](), make[1](), make[2])
    out = []
    for cull in (False, True):
        gs.set_cull(cull)
        b, adj = gs.widom_adjoint(3000, 5, 77, T, want_energies=True, want_grad=want_grad)
        out.append((b, adj))
    (b0, a0), (b1, a1) = out
    np.testing.assert_array_equal(b1, b0)
    for key in ("log_scale", "sum_w", "sum_w_ues", "d_eps", "d_sig2", "u", "grad"):
        np.testing.assert_array_equal(a1[key], a0[key])


@pytest.mark.parametrize("exact", [True, False])
def test_culled_grid_adjoint_is_bit_identical(exact):
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.xe(), sc.box), ff)
    gs.set_exact(exact)
    res = []
    for cull in (False, True):
        gs.set_cull(cull)
        res.append(gs.energy_grid_adjoint((19, 18, 17), rep, 1.0, T))
    for x, y in zip(res[0][:2], res[1][:2]):
        np.testing.assert_array_equal(y, x)
    for key in ("log_scale", "d_eps", "d_sig2"):
        np.testing.assert_array_equal(res[1][2][key], res[0][2][key])
