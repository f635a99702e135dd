"""Latency path for Monte Carlo moves: pmgb_energies with up to 64 configurations and the
graph-captured pmgb_move_* evaluator, against the FP64 oracle.  With exact energies (the
default) every configuration is evaluated in double-float and must meet 1e-5 relative or
1e-4 K; the FP32 latency kernel (one CTA per configuration, exact energies off) is checked with
the FP32 error model of the parity tests (4e-6 x the sum of term magnitudes + 1e-4 K) and
against the many-configuration kernel."""
from __future__ import annotations

import time

import numpy as np
import pytest

import pmgb
from pm_helpers import oracle_for, random_configs, within
from pmgb import synthetic
from pmgb.batch import BatchScreen

pytestmark = pytest.mark.gpu
TOL, ATOL = 4e-6, 1e-4


def _system(cr, mol, charged):
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    return pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("case", ["co2_ewald", "ch4"])
def test_latency_path_matches_oracle(case, exact):
    gs = _system(synthetic.config1(), synthetic.co2(), True) if case == "co2_ewald" else \
        _system(synthetic.config0(), synthetic.ch4(), False)
    gs.set_exact(exact)
    sites, lj, q = random_configs(gs, 64, seed=71)
    small = gs.energies(sites)                       # 64 configurations: latency kernel (FP32 pass)
    big = gs.energies(np.concatenate([sites, sites[:1]]))[:64]  # 65: the many-configuration kernel
    o = oracle_for(gs)
    if gs.charged:
        v, sr, lr, sv, ss = o.energies(lj, q, charged=True, use_sk=True, scales=True)
    else:
        v, sr, lr, sv, ss = o.energies(lj, scales=True)
        lr = np.zeros_like(v)
    for gpu in (small, big):
        assert np.array_equal(np.isinf(gpu[:, 0]), np.isinf(v))
        fin = np.isfinite(v)
        if exact:
            assert within(gpu[fin].sum(axis=1), (v + sr + lr)[fin], 1e-5, ATOL).all()
            assert within(gpu[fin, 0], v[fin], 1e-5, ATOL).all()
            continue
        assert np.all(np.abs(gpu[fin, 0] - v[fin]) <= TOL * sv[fin] + ATOL)
        if gs.charged:
            assert np.all(np.abs(gpu[:, 1] - sr) <= TOL * ss + ATOL)
    if gs.charged and not exact:
        # reciprocal space: the same FP32 recurrence, rows split over threads instead of one thread
        # per configuration (checked against the oracle with its own error scale in the parity tests)
        assert np.all(np.abs(small[:, 2] - big[:, 2]) <= 2e-3 + 1e-6 * np.abs(big[:, 2]))


@pytest.mark.parametrize("exact", [True, False])
def test_move_evaluator_matches_energies(exact):
    gs = _system(synthetic.config1(), synthetic.co2(), True)
    gs.set_exact(exact)
    sites, _, _ = random_configs(gs, 40, seed=72)
    ev = gs.move_evaluator(max_conf=8)
    ref = gs.energies(sites)
    for k in range(0, 40, 8):
        got = ev.energies(sites[k:k + 8])
        np.testing.assert_array_equal(got, ref[k:k + 8])  # same kernels, same inputs
    one = ev.energies(sites[3])
    np.testing.assert_array_equal(one, gs.energies(sites[3:4]))
    # the FP64 chunking of an exact pass follows the number of configurations in the call (a finer
    # partition for one configuration): the last bits may differ from the 40-configuration call
    np.testing.assert_allclose(one[0], ref[3], rtol=1e-13, atol=0.0)
    with pytest.raises(pmgb.PMGBError, match="n_conf"):
        ev.energies(sites[:9])
    # latency of one move (host call, graph replay), printed for the record
    ev1 = gs.move_evaluator(1)
    for _ in range(20):
        ev1.energies(sites[0])
    t = time.perf_counter()
    n = 200
    for i in range(n):
        ev1.energies(sites[i % 40])
    dt = (time.perf_counter() - t) / n
    print(f"[move] CO2 + Ewald in 7,200 sites ({'exact' if exact else 'FP32'}): {dt * 1e6:.1f} us per "
          f"single-configuration call")
    assert gs.ctx.device_status() == 0


def test_handles_destroyed_in_any_order():
    """A move handle and a batch hold their system: destroying the system handle first (the order a
    garbage-collected host may choose) leaves them working, and no error of the teardown is reported
    by a later, unrelated call."""
    gs = _system(synthetic.config0(), synthetic.ch4(), False)
    sites, _, _ = random_configs(gs, 4, seed=5)
    want = gs.energies(sites[:2])
    ev = gs.move_evaluator(max_conf=2)
    bs = BatchScreen([gs], 1000, n_blocks=2)
    ctx = gs.ctx
    gs.close()
    np.testing.assert_array_equal(ev.energies(sites[:2]), want)
    bs.launch(seed=3, temperature=298.0)
    blocks, _ = bs.results()
    assert blocks.shape == (1, 2, 4) and np.isfinite(blocks).all()
    ev.close()
    bs.close()
    xf, _ = ctx.sample_poses(seed=1, start=0, n=8)
    assert xf.shape == (8, 3)
    assert ctx.device_status() == 0
