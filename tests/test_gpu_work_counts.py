"""The work counts behind the counted-work roofline (pmgb_widom_work_counts,
pmgb_energy_grid_work_counts).

The counting pass must report what the forward kernel does: every (guest site, record) distance
of the records it does not skip, and the pair terms inside the cutoffs.  The pairs inside the
cutoff are counted again here in FP64 from the device's own poses (only pairs within FP32
rounding of the cutoff may differ); the distances are all pairs where no sub-chunk can be skipped
(the config1 cell) and fewer where sub-chunks are skipped (the 52 A config4 cell), never fewer
than the pairs inside the cutoff.
"""
from __future__ import annotations

import numpy as np
import pytest

import pmgb
from pm_helpers import oracle_for
from pmgb import synthetic
from pmgb.molecule import body_offsets

pytestmark = pytest.mark.gpu


def _system(cr, mol):
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    charged = pmgb.crystal.has_charges(sc) and mol.n_charges > 0
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    return pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)


def _pairs_inside(gs, seed, n, r_cut):
    """FP64 count of (guest site, framework atom) pairs within r_cut over the device poses."""
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    xf, rot = gs.ctx.sample_poses(seed, 0, n)
    sites = oracle_for(gs).sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    atoms = gs.crystal.atoms.xf
    f2c = gs.crystal.box.f_to_c
    total = 0
    for i in range(n):
        d = atoms[None, :, :] - sites[i][:, None, :]
        d -= np.round(d)
        c = d @ f2c.T
        total += int(((c * c).sum(-1) < r_cut ** 2).sum())
    return total


@pytest.mark.parametrize("case", ["config1", "config4"])
def test_widom_work_counts(case):
    gs = _system(synthetic.config1() if case == "config1" else synthetic.config4(), synthetic.co2())
    gs.set_image_lists(False)  # the per-site pass (image lists: tests/test_gpu_image_lists.py)
    npb, nb, seed = 200, 5, 31
    n = npb * nb
    c = gs.widom_work_counts(npb, nb, seed)
    every = n * gs.n_sites * gs.info()["n_records"]
    inside = _pairs_inside(gs, seed, n, 12.5)
    print(f"[work {case}] distances {c['distances']} of {every}; LJ terms {c['lj_terms']} (FP64 count {inside}); "
          f"real-space terms {c['es_terms']}")
    assert abs(c["lj_terms"] - inside) <= 1e-5 * inside + 4
    assert c["es_terms"] == pytest.approx(c["lj_terms"], rel=1e-5, abs=4)  # the same cutoff, charges on the atoms
    if case == "config1":
        assert c["distances"] == every          # no sub-chunk of this cell is skipped
    else:
        assert c["lj_terms"] < c["distances"] < every
    # the counts depend only on the insertions, not on the call
    assert gs.widom_work_counts(npb, nb, seed) == c


def test_grid_work_counts():
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.xe(), sc.box), ff)
    n_pts = (9, 8, 7)
    c = gs.energy_grid_work_counts(n_pts, rep)
    n = int(np.prod(n_pts))
    assert c["distances"] == n * sc.atoms.n and c["es_terms"] == 0
    pts = np.stack(np.meshgrid(*[np.arange(k) / (k - 1) for k in n_pts], indexing="ij"), -1).reshape(-1, 3)
    pts = np.where(pts >= 1.0, 0.0, pts) / np.array(rep)
    d = sc.atoms.xf[None, :, :] - pts[:, None, :]
    d -= np.round(d)
    cc = d @ sc.box.f_to_c.T
    inside = int(((cc * cc).sum(-1) < 12.5 ** 2).sum())
    assert abs(c["lj_terms"] - inside) <= 1e-5 * inside + 4
    with pytest.raises(pmgb.PMGBError, match="single site"):
        _system(synthetic.config0(), synthetic.co2()).energy_grid_work_counts(n_pts, rep)
