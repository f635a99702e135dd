"""Centre-image distances (pmgb_system_set_centre_image) against the per-site form and the oracle.

Where every perpendicular width of the supercell is at least 2 (cutoff + the guest's reach from
its pose centre), the Widom kernels take each framework record's minimum image from the pose
centre and subtract the sites' offsets.  The pairs inside the cutoff are the per-site minimum
images, so the energies must match the FP64 oracle to the FP32 tolerance of the per-site form;
culled and unculled runs, and a batch and its single systems, bit for bit; the refined K_H within
1e-6 of the oracle; the adjoint without forces (centre images) the one with forces (per-site
images) to the gradient tolerance 1e-4.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import pmgb
from pm_helpers import oracle_for, oracle_sites_split
from pmgb import synthetic
from pmgb.batch import BatchScreen, system_seed

pytestmark = pytest.mark.gpu
T = 298.0
ATOL = 1e-4
FP32_SCALE_TOL = 4e-6


def _system(cr):
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    return pmgb.GPUSystem(sc, pmgb.Frac(synthetic.co2(), sc.box), ff, ep)


@pytest.fixture(scope="module")
def wide():
    """CO2 in the 52 A cubic cell: every width exceeds 2 (12.5 + 1.16) A.  Image lists off, so that
    the Widom passes here take the centre-image or the per-site distances."""
    gs = _system(synthetic.config4())
    gs.set_image_lists(False)
    return gs


def _oracle_energies(gs, n_per_block, seed, n_blocks=5):
    """FP64 energies of the device poses with the magnitudes their FP32 sums are formed from."""
    from pmgb.molecule import body_offsets

    xf, rot = gs.ctx.sample_poses(seed, 0, n_blocks * n_per_block)
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    o = oracle_for(gs)
    sites = o.sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    lj, q = oracle_sites_split(gs, sites)
    v, sr, lr, sv, ss = o.energies(lj, q, charged=True, use_sk=True, scales=True)
    # reciprocal space: the FP32 sum is formed from sum_k |wt_k S(k)| |G(k)|, bounded by sum_k |wt S|
    sl = np.full(v.shape, np.abs(gs.eparams.kvec_wt * gs.structure_factor()).sum() * np.abs(q.shape[1]))
    return v, sr + lr, sv, ss + sl


def test_centre_image_applies_where_the_cell_is_wide(wide):
    assert wide.info()["centre_image"]
    narrow = _system(synthetic.config1())  # 2x2x3 of a 13.2 x 18.9 x 9.8 A cell: 25.8 A across a
    assert not narrow.info()["centre_image"]
    try:
        wide.set_centre_image(False)
        assert not wide.info()["centre_image"]
    finally:
        wide.set_centre_image(True)
    assert wide.info()["centre_image"]
    ch4 = pmgb.GPUSystem(wide.crystal, pmgb.Frac(synthetic.ch4(), wide.crystal.box), synthetic.forcefield())
    assert not ch4.info()["centre_image"]  # one site: it is the centre


def test_centre_image_energies_match_oracle(wide):
    npb, seed = 200, 5
    v, es, sv, se = _oracle_energies(wide, npb, seed)
    fin = np.isfinite(v)
    out = {}
    try:
        for on in (True, False):
            wide.set_centre_image(on)
            _, u = wide.widom(npb, 5, seed, T, want_energies=True)
            out[on] = u
            assert np.array_equal(np.isinf(u[:, 0]), ~fin)
            assert np.all(np.abs(u[fin, 0] - v[fin]) <= FP32_SCALE_TOL * sv[fin] + ATOL)
            assert np.all(np.abs(u[fin, 1] - es[fin]) <= FP32_SCALE_TOL * se[fin] + ATOL)
    finally:
        wide.set_centre_image(True)
    d = np.abs(out[True][fin].sum(axis=1) - out[False][fin].sum(axis=1))
    print(f"[centre image] max |centre - per-site| {d.max():.3e} K over {fin.sum()} insertions")
    assert np.all(d <= 2 * FP32_SCALE_TOL * (sv[fin] + se[fin]) + 2 * ATOL)


def test_centre_image_refined_kh_matches_oracle(wide):
    npb, seed = 200, 9
    v, es, _, _ = _oracle_energies(wide, npb, seed)
    ref = oracle.widom_blocks_log(v, es, T, 5, npb)
    wide.set_refine(1e-3)
    try:
        blocks, _ = wide.widom(npb, 5, seed, T)
    finally:
        wide.set_refine(0.0)
    assert np.abs(blocks[:, 0] - ref[:, 0]).max() <= 1e-6  # log K_H: 1e-6 relative


def test_centre_image_culled_is_bit_identical(wide):
    npb, seed = 257, 123
    try:
        wide.set_cull(False)
        b0, u0 = wide.widom(npb, 5, seed, T, want_energies=True)
        wide.set_cull(True)
        b1, u1 = wide.widom(npb, 5, seed, T, want_energies=True)
    finally:
        wide.set_cull(True)
    np.testing.assert_array_equal(u1, u0)
    np.testing.assert_array_equal(b1, b0)


@pytest.mark.parametrize("tail", [0.0, 1e-3])
def test_centre_image_batch_matches_single_system(wide, tail):
    npb, nb, seed = 300, 5, 44
    ch4 = pmgb.GPUSystem(wide.crystal, pmgb.Frac(synthetic.ch4(), wide.crystal.box), synthetic.forcefield())
    systems = [wide, ch4]
    screen = BatchScreen(systems, npb, nb, refine_tail=tail)
    blocks, _ = screen.run(seed, T)
    try:
        for s, gs in enumerate(systems):
            gs.set_refine(tail)
            ref, _ = gs.widom(npb, nb, system_seed(seed, s), T)
            np.testing.assert_array_equal(blocks[s], ref)
    finally:
        for gs in systems:
            gs.set_refine(0.0)
        screen.close()


def test_centre_image_adjoint_matches_per_site_forces(wide):
    from pmgb.adjoint import henry_gradients

    npb, seed = 300, 12
    b0, a0 = wide.widom_adjoint(npb, 5, seed, T, want_energies=True)                  # centre images
    b1, a1 = wide.widom_adjoint(npb, 5, seed, T, want_energies=True, want_grad=True)  # per-site images
    fwd, u_fwd = wide.widom(npb, 5, seed, T, want_energies=True)
    np.testing.assert_array_equal(a0["u"], u_fwd)  # the columns ride on the forward loops
    g0 = henry_gradients(wide, b0, a0, T, npb)
    g1 = henry_gradients(wide, b1, a1, T, npb)
    for x, y in zip(g0[:2], g1[:2]):
        scale = max(abs(val) for val in y.values())
        for sp in y:
            assert x[sp] == pytest.approx(y[sp], rel=1e-4, abs=1e-6 * scale), sp
    assert g0[2] == pytest.approx(g1[2], rel=1e-4)
