"""Image lists in the spatially ordered Widom pass (csrc/pmgb_img.cu; pmgb_system_set_image_lists).

Each warp gathers the framework images within (cutoff + its sites' spread) of its centre and its
lanes take distances from that list.  The per-insertion energies are checked against the FP64
oracle on the exact device poses at the FP32 tolerance of the per-site pass (a multiple of the sum
of the terms' magnitudes), the refined K_H against the oracle at 1e-6, overlaps exactly, and the
results are deterministic.  Few insertions spread a warp over the whole cell, so that its list
takes images shifted by one or more cells; the same checks hold there.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import pmgb
from pm_helpers import oracle_for, oracle_sites_split
from pmgb import synthetic
from pmgb.molecule import body_offsets

pytestmark = pytest.mark.gpu

T = 298.0
FP32_SCALE_TOL, ATOL = 8e-6, 1e-4  # twice the per-site pass's bound: list offsets are rounded once more

CASES = {
    "co2_dense": (synthetic.config1, synthetic.co2),
    "co2_porous": (synthetic.config1_porous, synthetic.co2),
    "ch4_config0": (synthetic.config0, synthetic.ch4),
    "co2_config4": (synthetic.config4, synthetic.co2),
}


def _system(case):
    cr, mol = CASES[case][0](), CASES[case][1]()
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    charged = pmgb.crystal.has_charges(sc) and mol.n_charges > 0
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    gs = pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)
    gs.set_image_lists(True)  # wherever they apply, also in these sparse runs
    return gs


def _oracle(gs, npb, seed, nb=5):
    """FP64 energies of the device poses and the magnitudes their FP32 sums are formed from."""
    xf, rot = gs.ctx.sample_poses(seed, 0, nb * npb)
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    o = oracle_for(gs)
    sites = o.sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    lj, q = oracle_sites_split(gs, sites)
    if gs.charged:
        v, sr, lr, sv, ss = o.energies(lj, q, charged=True, use_sk=True, scales=True)
        sl = np.abs(gs.eparams.kvec_wt * gs.structure_factor()).sum() * q.shape[1]
        return v, sr + lr, sv, ss + sl
    v, _, _, sv, _ = o.energies(lj, None, charged=False, use_sk=True, scales=True)
    return v, np.zeros_like(v), sv, np.zeros_like(v)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("npb", [1, 7, 300, 4000])
def test_image_list_energies_and_kh(case, npb):
    if case == "co2_config4" and npb > 300:
        npb = 1000  # 20,000 framework atoms: keep the oracle short
    gs = _system(case)
    seed = 77 + npb
    gs.set_refine(1e-3)
    assert gs.image_lists(5 * npb)
    blocks, u = gs.widom(npb, 5, seed, T, want_energies=True)
    again, u2 = gs.widom(npb, 5, seed, T, want_energies=True)
    np.testing.assert_array_equal(again, blocks)  # deterministic
    np.testing.assert_array_equal(u2, u)
    v, es, sv, se = _oracle(gs, npb, seed)
    fin = np.isfinite(v)
    assert np.array_equal(np.isinf(u[:, 0]), ~fin)  # overlaps exactly
    dv = np.abs(u[fin, 0] - v[fin]) - (FP32_SCALE_TOL * sv[fin] + ATOL)
    de = np.abs(u[fin, 1] - es[fin]) - (FP32_SCALE_TOL * se[fin] + ATOL)
    print(f"[image lists {case} {npb}] worst margin vdw {dv.max() if dv.size else 0:.3e} es {de.max() if de.size else 0:.3e}")
    assert np.all(dv <= 0) and np.all(de <= 0)
    ref = oracle.widom_blocks_log(v, es, T, 5, npb)
    has = np.isfinite(ref[:, 0])
    assert np.array_equal(np.isfinite(blocks[:, 0]), has)
    # log K_H within 1e-6 (K_H within 1e-6 relative), or within the double-float re-evaluation's
    # relative precision (~1e-14) of U/T where one insertion's U of 1e10 K or more sets a block
    tol = 1e-6 + 1e-13 * np.abs(ref[has, 0])
    dlog = np.abs(blocks[has, 0] - ref[has, 0])
    print(f"[image lists {case} {npb}] |Δ log K_H| {dlog.max(initial=0.0):.2e}")
    assert np.all(dlog <= tol)
    # the per-site refined pass agrees to the same tolerance
    gs.set_image_lists(False)
    assert not gs.image_lists(5 * npb)
    per_site, _ = gs.widom(npb, 5, seed, T)
    assert np.all(np.abs(per_site[has, 0] - blocks[has, 0]) <= 2 * tol)
    assert gs.ctx.device_status() == 0


def test_image_lists_modes():
    """Off, on wherever they apply, and auto: by the run's insertion density (a CTA's list expected
    under 90% of the records, in a run of at least two CTAs per SM) -- the 1e6-insertion config1
    run takes them, a 1e4-insertion run of the same cell does not."""
    gs = _system("co2_dense")
    assert gs.image_lists(1000)          # on (set by _system)
    gs.set_cull(False)                   # no spatial order: the per-site pass
    assert not gs.image_lists(1000)
    gs.set_cull(True)
    gs.set_image_lists(False)
    assert not gs.image_lists(10 ** 6)
    gs.set_image_lists("auto")
    assert gs.image_lists(10 ** 6) and not gs.image_lists(10 ** 4)
    c4 = _system("co2_config4")
    c4.set_image_lists("auto")
    assert c4.image_lists(10 ** 5)       # 20,000 atoms in a 52 A cell: lists pay at any density


@pytest.mark.parametrize("case", ["co2_dense", "co2_porous", "ch4_config0"])
def test_image_list_fp32_pass(case):
    """Without refinement: per-insertion energies and K_H of the FP32 pass against the oracle at
    the per-site pass's FP32 bounds, and the per-site pass within the same distance of it."""
    gs = _system(case)
    npb, seed = 3000, 19
    assert gs.image_lists(5 * npb)
    blocks, u = gs.widom(npb, 5, seed, T, want_energies=True)
    v, es, sv, se = _oracle(gs, npb, seed)
    fin = np.isfinite(v)
    assert np.array_equal(np.isinf(u[:, 0]), ~fin)
    assert np.all(np.abs(u[fin, 0] - v[fin]) <= FP32_SCALE_TOL * sv[fin] + ATOL)
    assert np.all(np.abs(u[fin, 1] - es[fin]) <= FP32_SCALE_TOL * se[fin] + ATOL)
    gs.set_image_lists(False)
    b_ps, u_ps = gs.widom(npb, 5, seed, T, want_energies=True)
    d = np.abs(u[fin].sum(axis=1) - u_ps[fin].sum(axis=1))
    print(f"[image lists fp32 {case}] max |img - per-site| {d.max():.3e} K")
    assert np.all(d <= 2 * FP32_SCALE_TOL * (sv[fin] + se[fin]) + 2 * ATOL)


def test_image_list_work_counts():
    """The counted work of the image-list pass: the pairs inside the cutoff are the per-site
    pass's; the distances are fewer where the insertions are dense enough for compact warps (2e5
    insertions in the 28,700 A^3 supercell; the list holds the images within reach of each warp)."""
    gs = _system("co2_dense")
    gs.set_refine(1e-3)
    npb, nb, seed = 40000, 5, 31
    c_img = gs.widom_work_counts(npb, nb, seed)
    gs.set_image_lists(False)
    c_ps = gs.widom_work_counts(npb, nb, seed)
    print(f"[image lists work] {c_img} vs per-site {c_ps}")
    assert abs(c_img["lj_terms"] - c_ps["lj_terms"]) <= 1e-5 * c_ps["lj_terms"] + 4
    assert abs(c_img["es_terms"] - c_ps["es_terms"]) <= 1e-5 * c_ps["es_terms"] + 4
    assert c_img["lj_terms"] < c_img["distances"] < c_ps["distances"]
