"""FP64 refinement of the Boltzmann tail (pmgb_system_set_refine) against the FP64 oracle.

With refinement the block K_H and <U> must agree with the oracle's FP64 evaluation of the
same insertions to 1e-6 relative (the accuracy target of the path); the refined insertions'
energies must agree to FP64 rounding.  Cases: the porous and the dense config1 cells with CO2
and Ewald, CH4 (LJ only) in the porous config1 cell and in config0.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import pmgb
from pm_helpers import widom_with_oracle
from pmgb import synthetic

pytestmark = pytest.mark.gpu
T = 298.0


def _system(cr, mol, charged):
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    return pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)


CASES = {
    "co2_ewald_porous": (synthetic.config1_porous, synthetic.co2, True, 20000),
    "co2_ewald_dense": (synthetic.config1, synthetic.co2, True, 4000),
    "ch4_porous": (synthetic.config1_porous, synthetic.ch4, False, 20000),
    "ch4_config0": (synthetic.config0, synthetic.ch4, False, 20000),
}


@pytest.mark.parametrize("case", list(CASES))
def test_refined_blocks_match_oracle(case):
    make_cr, make_mol, charged, npb = CASES[case]
    gs = _system(make_cr(), make_mol(), charged)
    seed = 51
    b32, _ = gs.widom(npb, 5, seed, T, want_energies=True)
    gs.set_refine(1e-3)
    blocks, u, v, es = widom_with_oracle(gs, npb, seed, T)
    ref = oracle.widom_blocks_log(v, es, T, 5, npb)
    d32 = np.abs(b32[:, 0] - ref[:, 0]).max()
    d64 = np.abs(blocks[:, 0] - ref[:, 0]).max()
    n_ref = gs.refined_count()
    print(f"[refine {case}] |Δ log K_H| FP32 {d32:.2e} -> refined {d64:.2e}; refined insertions "
          f"{n_ref} of {u.shape[0]}")
    assert d64 <= 1e-6                                   # K_H within 1e-6 relative
    u_ref = ref[:, 1] + ref[:, 2]
    assert np.all(np.abs(blocks[:, 1] + blocks[:, 2] - u_ref) <= 1e-6 * np.abs(u_ref) + 1e-9)
    np.testing.assert_array_equal(blocks[:, 3], ref[:, 3])
    # the refined insertions carry FP64 energies (the others keep the FP32 pass's, which with a
    # refinement to follow skips the box-matrix residual), and they include every insertion
    # among those carrying 99% of a block's Boltzmann weight
    fin = np.isfinite(v)
    exact = fin & (np.abs(u[:, 0] - v) <= 1e-10 * np.abs(v) + 1e-8) & (np.abs(u[:, 1] - es) <= 1e-10 * np.abs(es) + 1e-8)
    assert n_ref > 0 and exact.sum() + np.count_nonzero(~fin) >= n_ref
    x = np.where(fin, -(v + es) / T, -np.inf).reshape(5, npb)
    for b in range(5):
        if not np.isfinite(x[b]).any():
            continue
        w = np.exp(x[b] - x[b].max())
        top = np.argsort(-w)
        head = top[:np.searchsorted(np.cumsum(w[top]) / w.sum(), 0.99) + 1]
        assert exact.reshape(5, npb)[b, head].all(), (case, b)
    # deterministic, and tail 0 restores the FP32 results
    again, _ = gs.widom(npb, 5, seed, T)
    np.testing.assert_array_equal(again, blocks)
    gs.set_refine(0.0)
    plain, _ = gs.widom(npb, 5, seed, T)
    np.testing.assert_array_equal(plain, b32)
    assert gs.ctx.device_status() == 0


def test_refine_in_adjoint_and_drop_in():
    gs = _system(synthetic.config1_porous(), synthetic.co2(), True)
    npb, seed = 8000, 52
    gs.set_refine(1e-3)
    b_w, _ = gs.widom(npb, 5, seed, T)
    b_a, adj = gs.widom_adjoint(npb, 5, seed, T)
    # the adjoint kernel's FP32 energies differ in rounding; after refinement both sit on FP64
    np.testing.assert_allclose(b_a[:, 0], b_w[:, 0], rtol=0, atol=2e-7)
    assert np.isfinite(adj["log_scale"])
    with pytest.raises(pmgb.PMGBError, match="tail fraction"):
        gs.set_refine(1.5)
