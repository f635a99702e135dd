"""Batched persistent screening (pmgb_batch_*) against the single-system entry points.

Every system of a batch must see exactly the insertions of pmgb_widom with its own seed
system_seed(seed, s), so block results agree to the last bit; the adjoint sums are
accumulated in another order and with other weight offsets, so they agree to 1e-9
relative.  The single-system results are themselves checked against the FP64 oracle and
finite differences in test_gpu_parity.py and test_gpu_adjoint.py; the LJ-only members are
also checked against the oracle here.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
import pmgb
from pmgb import synthetic
from pmgb.adjoint import henry_gradients
from pmgb.batch import BatchScreen, build_systems, henry_coefficient_screen, system_seed
from pm_helpers import oracle_for

pytestmark = pytest.mark.gpu
T = 298.0


@pytest.fixture(scope="module")
def mixed_systems():
    """Frameworks of uneven size, each with CH4 (LJ only) and CO2 (LJ + Ewald)."""
    ff = synthetic.forcefield()
    fws = synthetic.batch_frameworks(6, seed=77)
    ctx = pmgb.Context.default()
    systems = build_systems(fws, synthetic.ch4(), ff, ctx=ctx) + build_systems(fws, synthetic.co2(), ff, ctx=ctx)
    sizes = [gs.info()["n_records"] for gs in systems]
    assert max(sizes) > 4 * min(sizes)  # uneven on purpose
    return systems


def test_batch_forward_matches_single_system(mixed_systems):
    npb, nb, seed = 700, 5, 1234
    screen = BatchScreen(mixed_systems, npb, nb)
    blocks, adj = screen.run(seed, T)
    assert adj is None
    for s, gs in enumerate(mixed_systems):
        ref, _ = gs.widom(npb, nb, system_seed(seed, s), T)
        np.testing.assert_array_equal(blocks[s], ref)
    # a replay with the same seed reproduces the run; another seed changes it
    again, _ = screen.run(seed, T)
    np.testing.assert_array_equal(again, blocks)
    other, _ = screen.run(seed + 1, T)
    assert not np.array_equal(other[:, :, 0], blocks[:, :, 0])
    assert screen.ctx.device_status() == 0


def test_batch_orders_and_shapes_agree(mixed_systems):
    npb, nb, seed = 300, 5, 99
    screen = BatchScreen(mixed_systems, npb, nb)
    base, _ = screen.run(seed, T)
    for n_ctas, order, mflop in ((1, 0, 0.0), (7, 1, 0.0), (0, 1, 1.0), (0, 0, 64.0), (3, 0, 1e6), (0, 0, 0.0)):
        screen.configure(n_ctas, order, mflop)
        got, _ = screen.run(seed, T)
        np.testing.assert_array_equal(got, base)
    screen.configure(0, 0, 0.0)
    with pytest.raises(pmgb.PMGBError, match="no run"):
        screen.results()  # configure discards the previous run
    ms = screen.tune(seed, T, repeats=2)
    assert ms > 0.0
    got, _ = screen.run(seed, T)
    np.testing.assert_array_equal(got, base)


def test_batch_ragged_insertion_counts(mixed_systems):
    npb = [1 + 97 * i for i in range(len(mixed_systems))]  # 1 insertion per block up to several units
    screen = BatchScreen(mixed_systems, npb, 5)
    blocks, _ = screen.run(5, T)
    for s, gs in enumerate(mixed_systems):
        ref, _ = gs.widom(npb[s], 5, system_seed(5, s), T)
        np.testing.assert_array_equal(blocks[s], ref)


@pytest.mark.parametrize("unit_mflop", [0.0, 64.0])
def test_batch_adjoint_matches_single_system(mixed_systems, unit_mflop):
    npb, nb, seed = 600, 5, 4321
    screen = BatchScreen(mixed_systems, npb, nb, with_adjoint=True)
    screen.configure(0, 0, unit_mflop)  # 64 MFLOP: several chunks per unit over a resident framework
    assert (screen.info()["n_units"] < screen.info()["n_chunks"]) == (unit_mflop > 0)
    blocks, adj = screen.run(seed, T)
    for s, gs in enumerate(mixed_systems):
        ref_b, ref_a = gs.widom_adjoint(npb, nb, system_seed(seed, s), T)
        np.testing.assert_array_equal(blocks[s], ref_b)
        got = henry_gradients(gs, blocks[s], adj[s], T, npb)
        want = henry_gradients(gs, ref_b, ref_a, T, npb)
        for g, w in zip(got[:2], want[:2]):
            scale = max(abs(v) for v in w.values())
            for sp in w:
                assert g[sp] == pytest.approx(w[sp], rel=1e-9, abs=1e-12 * scale), (s, sp)
        assert got[2] == pytest.approx(want[2], rel=1e-9, abs=1e-12 * abs(want[2]) + 1e-300)


def test_batch_lj_members_match_oracle(mixed_systems):
    """Block K_H of LJ members against the FP64 oracle on the same poses.

    FP32 alone, the log-sum may differ by no more than the Boltzmann-weighted FP32 error bound
    of the insertions' energies (4e-6 x the sum of |pair terms| + 1e-4 K) divided by T: up to
    ~1e-5 where a block's weight sits on a few deep sites.  With the FP64 tail refinement every
    block is within 1e-6 relative."""
    ff = synthetic.forcefield()
    porous = build_systems([synthetic.config0(), synthetic.config1_porous()], synthetic.ch4(), ff,
                           ctx=mixed_systems[0].ctx)
    lj_systems = porous + [gs for gs in mixed_systems if not gs.charged]
    npb, nb, seed = 400, 5, 2024
    screen = BatchScreen(lj_systems, npb, nb)
    blocks, _ = screen.run(seed, T)
    screen.set_refine(1e-3)
    refined, _ = screen.run(seed, T)
    for s, gs in enumerate(lj_systems):
        o = oracle_for(gs)
        xf, _ = gs.ctx.sample_poses(system_seed(seed, s), 0, npb * nb)
        v, _, _, scale, _ = o.energies(xf.astype(np.float64)[:, None, :], scales=True)  # one bead at the COM
        ref = oracle.widom_blocks_log(v, np.zeros_like(v), T, nb, npb)
        tol = 4e-6 * scale + 1e-4
        for b in range(nb):
            vb, tb = v[b * npb:(b + 1) * npb], tol[b * npb:(b + 1) * npb]
            fin = np.isfinite(vb)
            assert blocks[s, b, 3] == np.count_nonzero(~fin)
            if not fin.any():
                assert blocks[s, b, 0] == -np.inf and refined[s, b, 0] == -np.inf
                continue
            x = -vb[fin] / T
            p = np.exp(x - x.max())
            bound = float(np.sum(p * tb[fin]) / np.sum(p)) / T
            d = abs(blocks[s, b, 0] - ref[b, 0])
            assert d <= bound + 1e-12, (s, b, d, bound)
            assert abs(refined[s, b, 0] - ref[b, 0]) <= 1e-6, (s, b)  # K_H within 1e-6 relative


def test_batch_energies_match_single_system(mixed_systems):
    """pmgb_batch_energies: every system's per-insertion energies, refined ones in FP64, equal
    pmgb_widom's with the system's own seed; without culling and refinement there are none."""
    npb, nb, seed = 300, 5, 71
    screen = BatchScreen(mixed_systems, npb, nb, refine_tail=1e-3)
    try:
        screen.run(seed, T)
        energies = screen.energies()
        assert len(energies) == len(mixed_systems)
        for s, gs in enumerate(mixed_systems):
            gs.set_refine(1e-3)
            _, u = gs.widom(npb, nb, system_seed(seed, s), T, want_energies=True)
            gs.set_refine(0.0)
            assert energies[s].shape == (npb * nb, 2)
            np.testing.assert_array_equal(energies[s], u)
        screen.set_refine(0.0)
        screen.set_cull(False)
        screen.run(seed, T)
        with pytest.raises(pmgb.PMGBError):
            screen.energies()
    finally:
        screen.close()


def test_batch_refine_matches_single_system(mixed_systems):
    npb, nb, seed = 500, 5, 66
    screen = BatchScreen(mixed_systems, npb, nb, refine_tail=1e-3)
    blocks, _ = screen.run(seed, T)
    try:
        for s, gs in enumerate(mixed_systems):
            gs.set_refine(1e-3)
            ref, _ = gs.widom(npb, nb, system_seed(seed, s), T)
            np.testing.assert_array_equal(blocks[s], ref)
    finally:
        for gs in mixed_systems:
            gs.set_refine(0.0)
    assert screen.ctx.device_status() == 0


def test_batch_cull_matches_unordered(mixed_systems):
    """Spatial order + cutoff culling: block results equal the unordered run's bit for bit
    (ragged counts, several unit shapes, with and without the FP64 refinement).  Per-site
    distances (image lists off: those change FP32 roundings; tests/test_gpu_image_lists.py)."""
    npb = [1 + 251 * i for i in range(len(mixed_systems))]
    seed = 31
    for gs in mixed_systems:
        gs.set_image_lists(False)
    try:
        plain = BatchScreen(mixed_systems, npb, 5, cull=False)
        base, _ = plain.run(seed, T)
        culled = BatchScreen(mixed_systems, npb, 5)
        for n_ctas, order, mflop in ((0, 0, 0.0), (5, 1, 64.0), (0, 0, 1e6)):
            culled.configure(n_ctas, order, mflop)
            got, _ = culled.run(seed, T)
            np.testing.assert_array_equal(got, base)
        plain.set_refine(1e-3)
        culled.set_refine(1e-3)
        np.testing.assert_array_equal(culled.run(seed, T)[0], plain.run(seed, T)[0])
        np.testing.assert_array_equal(culled.refined_counts(), plain.refined_counts())
        culled.set_cull(False)
        np.testing.assert_array_equal(culled.run(seed, T)[0], plain.run(seed, T)[0])
    finally:
        for gs in mixed_systems:
            gs.set_image_lists("auto")
    assert culled.ctx.device_status() == 0


def test_batch_image_lists_match_single_system(mixed_systems):
    """Image lists in the batch (the systems that qualify) over the same insertion order as the
    single-system runs: equal block results and energies bit for bit, with and without the FP64
    refinement, ragged counts and several unit shapes."""
    npb = [1 + 173 * i for i in range(len(mixed_systems))]
    seed = 57
    for gs in mixed_systems:
        gs.set_image_lists(True)  # wherever they apply: these runs are sparse
    assert all(gs.image_lists(5 * n) for gs, n in zip(mixed_systems, npb))
    screen = BatchScreen(mixed_systems, npb, 5)
    try:
        for tail in (0.0, 1e-3):
            screen.set_refine(tail)
            for n_ctas, order, mflop in ((0, 0, 0.0), (5, 1, 64.0)):
                screen.configure(n_ctas, order, mflop)
                got, _ = screen.run(seed, T)
                for s, gs in enumerate(mixed_systems):
                    gs.set_refine(tail)
                    ref, _ = gs.widom(npb[s], 5, system_seed(seed, s), T)
                    np.testing.assert_array_equal(got[s], ref)
    finally:
        for gs in mixed_systems:
            gs.set_refine(0.0)
            gs.set_image_lists("auto")
        screen.close()
    assert mixed_systems[0].ctx.device_status() == 0


def test_batch_image_lists_adjoint_match_single_system(mixed_systems):
    """The adjoint with image lists: the batch's units form the columns in the list loop and weigh
    them per processing chunk; block results equal the single-system adjoint's (which takes the
    lists too: no forces) bit for bit, gradients to 1e-9 relative (FP64 sums in another order)."""
    npb, seed = [1 + 173 * i for i in range(len(mixed_systems))], 61
    for gs in mixed_systems:
        gs.set_image_lists(True)
    screen = BatchScreen(mixed_systems, npb, 5, with_adjoint=True)
    try:
        for n_ctas, order, mflop in ((0, 0, 0.0), (5, 1, 64.0)):
            screen.configure(n_ctas, order, mflop)
            blocks, adj = screen.run(seed, T)
            for s, gs in enumerate(mixed_systems):
                ref_b, ref_a = gs.widom_adjoint(npb[s], 5, system_seed(seed, s), T)
                np.testing.assert_array_equal(blocks[s], ref_b)
                got = henry_gradients(gs, blocks[s], adj[s], T, npb[s])
                want = henry_gradients(gs, ref_b, ref_a, T, npb[s])
                for g, w in zip(got[:2], want[:2]):
                    scale = max(abs(v) for v in w.values())
                    for sp in w:
                        assert g[sp] == pytest.approx(w[sp], rel=1e-9, abs=1e-12 * scale), (s, sp)
                assert got[2] == pytest.approx(want[2], rel=1e-9, abs=1e-12 * abs(want[2]) + 1e-300)
    finally:
        for gs in mixed_systems:
            gs.set_image_lists("auto")
        screen.close()
    assert mixed_systems[0].ctx.device_status() == 0


@pytest.mark.parametrize("unit_mflop", [0.0, 64.0])
def test_batch_cull_adjoint(mixed_systems, unit_mflop):
    """With culling, the adjoint's columns are weighted relative to each processing chunk's own
    maximum: same blocks, gradients equal to 1e-9 relative."""
    npb, nb, seed = 600, 5, 4321
    plain = BatchScreen(mixed_systems, npb, nb, with_adjoint=True, cull=False)
    culled = BatchScreen(mixed_systems, npb, nb, with_adjoint=True)
    culled.configure(0, 0, unit_mflop)
    b0, a0 = plain.run(seed, T)
    b1, a1 = culled.run(seed, T)
    np.testing.assert_array_equal(b1, b0)
    for s, gs in enumerate(mixed_systems):
        got = henry_gradients(gs, b1[s], a1[s], T, npb)
        want = henry_gradients(gs, b0[s], a0[s], T, npb)
        for g, w in zip(got[:2], want[:2]):
            scale = max(abs(v) for v in w.values())
            for sp in w:
                assert g[sp] == pytest.approx(w[sp], rel=1e-9, abs=1e-12 * scale), (s, sp)
        assert got[2] == pytest.approx(want[2], rel=1e-9, abs=1e-12 * abs(want[2]) + 1e-300)


def test_screen_driver(mixed_systems):
    res = henry_coefficient_screen(None, None, T, synthetic.forcefield(), insertions=1000, seed=8,
                                   systems=mixed_systems, tune=False, refine_tail=0.0)
    assert len(res) == len(mixed_systems)
    for s, (r, gs) in enumerate(zip(res, mixed_systems)):
        out = gs.widom_adjoint(200, 5, system_seed(8, s), T)[0]  # the adjoint kernel's energies
        kh = float(np.mean(np.exp(out[:, 0] - math.log(pmgb.UNIV_GAS_CONST * T * 200))))
        assert r["henry coefficient [mol/(m³-bar)]"] == kh
        assert set(r["dKH/d epsilon"]) == set(gs.species)


def test_batch_errors(mixed_systems):
    ctx = mixed_systems[0].ctx
    with pytest.raises(pmgb.PMGBError, match="n_per_block"):
        BatchScreen(mixed_systems[:2], 0, 5)
    other = pmgb.Context(0)
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    foreign = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.ch4(), sc.box), ff, ctx=other)
    with pytest.raises(pmgb.PMGBError, match="another context"):
        BatchScreen([mixed_systems[0], foreign], 10, 5, ctx=ctx)
    screen = BatchScreen(mixed_systems[:2], 10, 5)
    with pytest.raises(pmgb.PMGBError, match="no run"):
        screen.results()
    with pytest.raises(pmgb.PMGBError, match="n_ctas"):
        screen.configure(10 ** 6, 0)
    with pytest.raises(pmgb.PMGBError, match="unit_mflop"):
        screen.configure(0, 0, -1.0)
    assert ctx.device_status() == 0


def test_many_systems_in_one_call_match_single_set_up():
    """pmgb_systems_create_unitcell (host set-up on several threads, device set-up back to back)
    builds exactly the systems pmgb_system_create_unitcell builds one at a time: the same records,
    k-vectors kept, S(k) and Widom results to the last bit, whatever the number of threads."""
    ff = synthetic.forcefield()
    fws = synthetic.batch_frameworks(10, seed=5)
    mols = [synthetic.co2() if i % 2 else synthetic.ch4() for i in range(len(fws))]
    ctx = pmgb.Context.default()
    one_by_one = [pmgb.GPUSystem.from_unit_cell(cr, m, ff, ctx=ctx) for cr, m in zip(fws, mols)]
    for threads in (1, 4, 0):
        many = pmgb.GPUSystem.many_from_unit_cells(fws, mols, ff, ctx=ctx, n_threads=threads)
        for a, b in zip(one_by_one, many):
            assert a.repfactors == b.repfactors and a.charged == b.charged
            assert a.info() == b.info()
            if a.charged:
                ep = a.eparams
                assert ep is not None and b.eparams.n_kvecs == ep.n_kvecs
                np.testing.assert_array_equal(a.structure_factor(), b.structure_factor())
                if threads == 1:
                    # a replica's S(k) is evaluated from its unit cell; the supercell sum agrees
                    sup = pmgb.GPUSystem(a.crystal, a.molecule, ff, ep, ctx=ctx)
                    sk_a, sk_s = a.structure_factor(), sup.structure_factor()
                    scale = np.abs(sk_s).max()
                    np.testing.assert_allclose(sk_a, sk_s, rtol=0, atol=1e-12 * scale)
                    assert sup.info()["n_kvecs_evaluated"] == a.info()["n_kvecs_evaluated"]
                    np.testing.assert_allclose(a.widom(400, 5, 17, T)[0], sup.widom(400, 5, 17, T)[0],
                                               rtol=1e-7, atol=1e-9)
                    sup.close()
            ra, _ = a.widom(400, 5, 17, T)
            rb, _ = b.widom(400, 5, 17, T)
            np.testing.assert_array_equal(ra, rb)
        for g in many:
            g.close()
    assert any(g.charged for g in one_by_one) and not all(g.charged for g in one_by_one)


def test_many_systems_all_or_nothing():
    """A framework that cannot be set up fails the whole call, naming the system; none is created
    and the context stays usable."""
    ff = synthetic.forcefield()
    fws = synthetic.batch_frameworks(4, seed=8)
    bad = fws[2]
    bad.box.f_to_c[:, 1] = bad.box.f_to_c[:, 0]   # singular box
    ctx = pmgb.Context.default()
    with pytest.raises(pmgb.PMGBError, match="system 2"):
        pmgb.GPUSystem.many_from_unit_cells(fws, [synthetic.co2()] * 4, ff, ctx=ctx, n_threads=2)
    good = pmgb.GPUSystem.many_from_unit_cells(fws[:2], [synthetic.co2()] * 2, ff, ctx=ctx)
    assert len(good) == 2 and all(g.info()["n_records"] > 0 for g in good)
    assert pmgb.GPUSystem.many_from_unit_cells([], [], ff, ctx=ctx) == []
