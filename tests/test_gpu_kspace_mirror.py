"""Reciprocal space of guests with mirror-image sites (pmgb_system_kspace_mirror).

CO2 as the reference's data files give it (C at the centre of mass, the two O at +-1.16 A with
equal charges) takes the shortened k-space loop: e^{-ik.d_2} = conj(e^{-ik.d_1}).  The same
molecule with its sites listed O, C, O puts site 0 off the centre and takes the general loop.  The
poses (centre and rotation) are the same, so both must give the oracle's energies at the FP32
bound, and each other's K_H.
"""
from __future__ import annotations

import numpy as np
import pytest

import pmgb
from pm_helpers import oracle_for, oracle_sites_split
from pmgb import synthetic
from pmgb.molecule import body_offsets, molecule_from_sites

pytestmark = pytest.mark.gpu

T = 298.0
FP32_SCALE_TOL, ATOL = 8e-6, 1e-4


def _co2_oco():
    x = [[-1.16, 0.0, 0.0], [0.0, 0.0, 0.0], [1.16, 0.0, 0.0]]
    return molecule_from_sites("CO2", ["O_CO2", "C_CO2", "O_CO2"], x, [-0.35, 0.70, -0.35], x)


def _system(cell, mol, image_lists):
    cr, ff = cell(), synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)
    gs.set_image_lists(image_lists)
    return gs


def _oracle_es(gs, npb, seed, nb=5):
    xf, rot = gs.ctx.sample_poses(seed, 0, nb * npb)
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    o = oracle_for(gs)
    sites = o.sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    lj, q = oracle_sites_split(gs, sites)
    v, sr, lr, sv, ss = o.energies(lj, q, charged=True, use_sk=True, scales=True)
    sl = np.abs(gs.eparams.kvec_wt * gs.structure_factor()).sum() * q.shape[1]
    return v, sr + lr, ss + sl


@pytest.mark.parametrize("cell,npb,image_lists", [(synthetic.config1, 4000, "auto"),
                                                  (synthetic.config1_porous, 4000, False),
                                                  (synthetic.config4, 600, True)])
def test_mirror_sites_match_general_loop(cell, npb, image_lists):
    mirror = _system(cell, synthetic.co2(), image_lists)
    general = _system(cell, _co2_oco(), image_lists)
    assert mirror.info()["kspace_mirror"] and not general.info()["kspace_mirror"]
    seed = 5 + npb
    for gs in (mirror, general):
        gs.set_refine(1e-3)
    bm, um = mirror.widom(npb, 5, seed, T, want_energies=True)
    bg, ug = general.widom(npb, 5, seed, T, want_energies=True)
    v, es, se = _oracle_es(mirror, npb, seed)
    fin = np.isfinite(v)
    for u in (um, ug):
        d = np.abs(u[fin, 1] - es[fin]) - (FP32_SCALE_TOL * se[fin] + ATOL)
        print(f"[kspace mirror {cell.__name__}] worst es margin {d.max():.3e}")
        assert np.all(d <= 0)
    # refined K_H of the two site orders: both within 1e-6 of the oracle, so within 2e-6 of each other
    has = np.isfinite(bm[:, 0])
    assert np.array_equal(has, np.isfinite(bg[:, 0]))
    dlog = np.abs(bm[has, 0] - bg[has, 0])
    print(f"[kspace mirror {cell.__name__}] |d log K_H| {dlog.max(initial=0.0):.2e}")
    assert np.all(dlog <= 2e-6 + 2e-13 * np.abs(bm[has, 0]))
    assert mirror.ctx.device_status() == 0
