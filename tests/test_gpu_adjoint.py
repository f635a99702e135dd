"""GPU adjoint against central finite differences of the FP64 oracle.

Gradients must agree within 1e-4 relative (the hot-path contract): per-configuration dU/dx,
dK_H/dε_s and dK_H/dσ_s for every species (through Lorentz-Berthelot mixing), dK_H/dλ for the
framework charge scale, and the energy-grid adjoint.  Finite differences use h = 1e-4 relative
on parameters and 1e-5 Å on positions, on the exact poses the device used.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
import pmgb
from pm_helpers import oracle_sites_split, random_configs
from pmgb import synthetic
from pmgb.molecule import body_offsets

pytestmark = pytest.mark.gpu
T = 298.0


def _system(cr, mol, ff, charged):
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    return pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep)


def _oracle(gs, pure=None, qscale=1.0):
    """Oracle of a GPU system, optionally with perturbed pure LJ parameters / charge scale."""
    ff = gs.ljff
    if pure is not None:
        ff = pmgb.LJForceField({s: (pure[s][0], pure[s][1]) for s in pure}, r_cutoff=gs.ljff.r_cutoff,
                               mixing_rules=gs.ljff.mixing_rules)
    eps, sig2 = ff.tables(gs.species)
    cr = gs.crystal
    sid = {s: i for i, s in enumerate(gs.species)}
    o = oracle.OracleSystem(cr.box.f_to_c, cr.atoms.xf, [sid[s] for s in cr.atoms.species], cr.charges.xf,
                            cr.charges.q * qscale, eps, sig2, ff.r2_cutoff,
                            [sid[s] for s in gs.molecule.atom_species], gs.molecule.charge_q)
    if gs.eparams is not None:
        ep = gs.eparams
        o.set_ewald(ep.alpha, ep.sr_cutoff_r, ep.kreps, ep.kvec_abc, ep.kvec_wt)
    return o


def _pose_sites(gs, seed, n):
    xf, rot = gs.ctx.sample_poses(seed, 0, n)
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    body = np.zeros((gs.n_sites, 3))
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    sites = _oracle(gs).sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    return oracle_sites_split(gs, sites)


def _oracle_kh(o, lj, q, charged, npb):
    v, sr, lr = o.energies(lj, q, charged=charged, use_sk=True)
    blocks = oracle.widom_blocks_log(v, sr + lr, T, 5, npb)
    return float(np.mean(np.exp(blocks[:, 0] - math.log(pmgb.UNIV_GAS_CONST * T * npb))))


def _check_dkh(gs, npb, seed, charged):
    from pmgb.adjoint import henry_gradients

    blocks, adj = gs.widom_adjoint(npb, 5, seed, T)
    d_eps, d_sig, d_lam = henry_gradients(gs, blocks, adj, T, npb)
    lj, q = _pose_sites(gs, seed, 5 * npb)
    pure = {s: (gs.ljff.pure_sigma[s], gs.ljff.pure_epsilon[s]) for s in gs.species}
    h = 1e-4
    fd_eps, fd_sig = {}, {}
    for s in gs.species:
        for which, store in ((1, fd_eps), (0, fd_sig)):
            p0 = pure[s][which]
            vals = []
            for sgn in (+1, -1):
                p = dict(pure)
                t = list(p[s])
                t[which] = p0 * (1 + sgn * h)
                p[s] = tuple(t)
                vals.append(_oracle_kh(_oracle(gs, p), lj, q, charged, npb))
            store[s] = (vals[0] - vals[1]) / (2 * h * p0)
    scale = max(max(abs(v) for v in fd_eps.values()), max(abs(v) for v in fd_sig.values()))
    for s in gs.species:
        print(f"  {s:6s} dK/deps gpu {d_eps[s]: .6e} fd {fd_eps[s]: .6e} | dK/dsig gpu {d_sig[s]: .6e} "
              f"fd {fd_sig[s]: .6e}")
        assert d_eps[s] == pytest.approx(fd_eps[s], rel=1e-4, abs=1e-5 * scale)
        assert d_sig[s] == pytest.approx(fd_sig[s], rel=1e-4, abs=1e-5 * scale)
    if charged:
        vals = [_oracle_kh(_oracle(gs, qscale=1 + sgn * h), lj, q, True, npb) for sgn in (+1, -1)]
        fd_lam = (vals[0] - vals[1]) / (2 * h)
        print(f"  dK/dlambda gpu {d_lam:.6e} fd {fd_lam:.6e}")
        assert d_lam == pytest.approx(fd_lam, rel=1e-4, abs=1e-5 * abs(fd_lam))
    kh_gpu = float(np.mean(np.exp(blocks[:, 0] - math.log(pmgb.UNIV_GAS_CONST * T * npb))))
    return kh_gpu


@pytest.mark.parametrize("mol", ["co2", "ch4"])
def test_adjoint_without_forces(mol):
    """Without forces the adjoint runs the forward loops with the r^-12 / r^-6 columns added: its
    energies and block results are the forward pass's bit for bit, and its dK_H/d(eps, sigma,
    charge scale) agree with the pass that also forms dU/dx to FP32 rounding of the columns."""
    from pmgb.adjoint import henry_gradients

    ff = synthetic.forcefield()
    cr = synthetic.config1_porous()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    charged = mol == "co2"
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    gs = pmgb.GPUSystem(sc, pmgb.Frac(getattr(synthetic, mol)(), sc.box), ff, ep)
    gs.set_image_lists(False)  # the forward pass in the adjoint's own distance forms
    npb, seed = 3000, 12
    b1, a1 = gs.widom_adjoint(npb, 5, seed, T, want_energies=True, want_grad=True)  # with forces
    g1 = henry_gradients(gs, b1, a1, T, npb)
    # per-site images: the same pair arithmetic as the forces pass, so FP32 rounding of the columns;
    # centre images (CO2, the default): to the gradient tolerance
    for centre, rel in ((False, 1e-5), (True, 1e-4)):
        gs.set_centre_image(centre)
        fwd, u_fwd = gs.widom(npb, 5, seed, T, want_energies=True)
        b0, a0 = gs.widom_adjoint(npb, 5, seed, T, want_energies=True)  # columns only
        np.testing.assert_array_equal(a0["u"], u_fwd)
        np.testing.assert_array_equal(b0, fwd)
        g0 = henry_gradients(gs, b0, a0, T, npb)
        for x, y in zip(g0[:2], g1[:2]):
            scale = max(abs(v) for v in y.values())
            for sp in y:
                assert x[sp] == pytest.approx(y[sp], rel=rel, abs=1e-7 * scale), (centre, sp)
        if charged:
            assert g0[2] == pytest.approx(g1[2], rel=rel), centre
    gs.set_centre_image(True)


@pytest.mark.parametrize("mol", ["co2", "ch4"])
def test_adjoint_with_image_lists(mol):
    """Without forces, a run that takes image lists forms the columns in the image-list pass: its
    energies and block results are the forward image-list pass's bit for bit, and its dK_H/d(eps,
    sigma, charge scale) agree with the per-site pass that also forms dU/dx to the gradient
    tolerance (the two passes' FP32 energies and columns differ by rounding)."""
    from pmgb.adjoint import henry_gradients

    ff = synthetic.forcefield()
    cr = synthetic.config1_porous()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    charged = mol == "co2"
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6) if charged else None
    gs = pmgb.GPUSystem(sc, pmgb.Frac(getattr(synthetic, mol)(), sc.box), ff, ep)
    npb, seed = 3000, 14
    gs.set_image_lists(False)
    b1, a1 = gs.widom_adjoint(npb, 5, seed, T, want_energies=True, want_grad=True)  # per site, forces
    g1 = henry_gradients(gs, b1, a1, T, npb)
    gs.set_image_lists(True)
    assert gs.image_lists(5 * npb)
    fwd, u_fwd = gs.widom(npb, 5, seed, T, want_energies=True)
    b0, a0 = gs.widom_adjoint(npb, 5, seed, T, want_energies=True)  # columns from the lists
    np.testing.assert_array_equal(a0["u"], u_fwd)
    np.testing.assert_array_equal(b0, fwd)
    g0 = henry_gradients(gs, b0, a0, T, npb)
    for x, y in zip(g0[:2], g1[:2]):
        scale = max(abs(v) for v in y.values())
        for sp in y:
            assert x[sp] == pytest.approx(y[sp], rel=1e-4, abs=1e-7 * scale), sp
    if charged:
        assert g0[2] == pytest.approx(g1[2], rel=1e-4)
    assert gs.ctx.device_status() == 0


def test_dkh_lj():
    gs = _system(synthetic.config0(), synthetic.ch4(), synthetic.forcefield(), charged=False)
    _check_dkh(gs, 2000, seed=31, charged=False)


def test_dkh_ewald_porous():
    gs = _system(synthetic.config1_porous(), synthetic.co2(), synthetic.forcefield(), charged=True)
    _check_dkh(gs, 400, seed=32, charged=True)


def _fd_grad(o, lj, q, charged, box, h):
    """Central differences of the oracle's total energy for a rigid translation (Cartesian)."""
    g = np.zeros((lj.shape[0], 3))
    for d in range(3):
        e = np.zeros(3)
        e[d] = h
        df = box.c_to_f @ e
        up = o.energies(lj + df, q + df if q is not None else None, charged=charged, use_sk=True)
        dn = o.energies(lj - df, q - df if q is not None else None, charged=charged, use_sk=True)
        g[:, d] = (sum(up) - sum(dn)) / (2 * h)
    return g


@pytest.mark.parametrize("case", ["lj", "ewald"])
def test_forces_match_finite_differences(case):
    if case == "lj":
        gs = _system(synthetic.config0(), synthetic.ch4(), synthetic.forcefield(), charged=False)
    else:
        gs = _system(synthetic.config1_porous(), synthetic.co2(), synthetic.forcefield(), charged=True)
    sites, lj, q = random_configs(gs, 4000, seed=41)
    e, g = gs.energies_grad(sites)
    u = e.sum(axis=1)
    # the 300 lowest-energy configurations: those that carry Boltzmann weight
    order = np.argsort(np.where(np.isfinite(u), u, np.inf))[:300]
    sites, lj, e, g, u = sites[order], lj[order], e[order], g[order], u[order]
    q = q[order] if q is not None else None
    keep = np.isfinite(u)
    o = _oracle(gs)
    qq = q if gs.charged else None
    box = gs.crystal.box
    fd1 = _fd_grad(o, lj, qq, gs.charged, box, 1e-5)
    fd2 = _fd_grad(o, lj, qq, gs.charged, box, 5e-6)
    smooth = np.all(np.abs(fd1 - fd2) <= 1e-6 * np.abs(fd1) + 1e-4, axis=1)  # no cutoff crossing
    sel = keep & smooth
    assert sel.sum() > 50
    err = np.linalg.norm(g[sel] - fd1[sel], axis=1)
    ref = np.linalg.norm(fd1[sel], axis=1)
    print(f"[{case} forces] n={sel.sum()} max |Δ|/|g| {np.max(err / ref):.2e}; median {np.median(err / ref):.2e}")
    assert np.all(err <= 1e-4 * ref + 2e-3)


def test_grid_adjoint():
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.xe(), sc.box), ff)
    n_pts = (9, 8, 7)
    data, grad, adj = gs.energy_grid_adjoint(n_pts, rep, 1.0, T)
    ref = _oracle(gs).energy_grid(n_pts, rep)
    assert np.array_equal(np.isinf(data), np.isinf(ref))
    # dU/dr at each point against central differences of the oracle
    pts = np.stack(np.meshgrid(*[np.arange(n) / (n - 1) for n in n_pts], indexing="ij"), axis=-1).reshape(-1, 3)
    pts = pts / np.array(rep)
    o = _oracle(gs)
    fd = np.zeros_like(pts)
    for d in range(3):
        e = np.zeros(3)
        e[d] = 1e-5
        df = sc.box.c_to_f @ e
        fd[:, d] = (o.energies((pts + df)[:, None, :])[0] - o.energies((pts - df)[:, None, :])[0]) / 2e-5
    g = grad.reshape(-1, 3)
    u = data.reshape(-1)
    sel = np.isfinite(u) & (u < 5000.0)
    err = np.linalg.norm(g[sel] - fd[sel], axis=1)
    assert np.all(err <= 1e-4 * np.linalg.norm(fd[sel], axis=1) + 2e-3)
    # dK_H,grid/dε_s against finite differences of the oracle grid
    n_tot = int(np.prod(n_pts))
    scale = -math.exp(adj["log_scale"]) / (T * pmgb.UNIV_GAS_CONST * T * n_tot)
    from pmgb.adjoint import mixing_jacobians
    de, ds = mixing_jacobians(ff, gs.species)
    d_eps = np.einsum("ab,abs->s", adj["d_eps"] * scale, de)
    pure = {s: (ff.pure_sigma[s], ff.pure_epsilon[s]) for s in gs.species}

    def kh_grid(p):
        u = _oracle(gs, p).energy_grid(n_pts, rep).reshape(-1)
        fin = np.isfinite(u)
        return np.sum(np.exp(-u[fin] / T)) / (pmgb.UNIV_GAS_CONST * T * n_tot)

    for i, s in enumerate(gs.species):
        p0 = pure[s][1]
        plus, minus = dict(pure), dict(pure)
        plus[s] = (pure[s][0], p0 * (1 + 1e-4))
        minus[s] = (pure[s][0], p0 * (1 - 1e-4))
        fd_e = (kh_grid(plus) - kh_grid(minus)) / (2e-4 * p0)
        print(f"  grid {s:4s} dK/deps gpu {d_eps[i]: .6e} fd {fd_e: .6e}")
        assert d_eps[i] == pytest.approx(fd_e, rel=1e-4, abs=1e-6 * max(abs(fd_e), 1e-30) + 1e-20)
