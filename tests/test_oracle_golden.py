"""The FP64 oracle pinned against the reference's own golden values (no GPU needed).

Each test cites the reference test file:line whose known answer it reproduces.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
import pmgb
from conftest import DATA


def _sys_from_crystal(cr, mol, ljff, charged=False):
    species = list(dict.fromkeys(list(cr.atoms.species) + list(mol.atom_species)))
    sid = {s: i for i, s in enumerate(species)}
    eps, sig2 = ljff.tables(species)
    return oracle.OracleSystem(cr.box.f_to_c, cr.atoms.xf, [sid[s] for s in cr.atoms.species], cr.charges.xf,
                               cr.charges.q, eps, sig2, ljff.r2_cutoff, [sid[s] for s in mol.atom_species],
                               mol.charge_q if charged else np.zeros(0)), species


def test_lennard_jones_identities(golden):
    # test/vdw_energetics.jl:18-21
    for r2, s2, eps, want in golden["lennard_jones"]["cases"]:
        assert oracle.lennard_jones(r2, s2, eps) == pytest.approx(want, abs=1e-12)


def test_box_matches_host(golden):
    for args in [(11.6193, 5.5667, 22.9312, math.pi / 2, math.radians(100.897), math.pi / 2),
                 (6.8945, 15.2403, 15.2403, math.radians(117.768), math.radians(98.673), math.radians(98.673))]:
        f, cf, r, om = oracle.box(*args)
        b = pmgb.Box(*args)
        np.testing.assert_allclose(f, b.f_to_c, rtol=1e-14, atol=1e-14)
        np.testing.assert_allclose(r, b.reciprocal_lattice, rtol=1e-12, atol=1e-12)
        assert om == pytest.approx(b.Omega, rel=1e-14)
        np.testing.assert_allclose(r @ f, 2 * math.pi * np.eye(3), atol=1e-12)


def test_sbmof1_xe_dreiding(golden):
    # test/vdw_energetics.jl:26-41 (RASPA-matched)
    g = golden["sbmof1_xe_dreiding"]
    ljff = pmgb.LJForceField("Dreiding", r_cutoff=g["r_cutoff"])
    cr = pmgb.read_cif(DATA / "crystals" / "SBMOF-1.cif")
    rep = pmgb.replication_factors(cr.box, ljff)
    assert rep == oracle.replication_factors(cr.box.f_to_c, g["r_cutoff"])
    sc = pmgb.replicate(cr, rep)
    xe = pmgb.read_molecule("Xe")
    osys, _ = _sys_from_crystal(sc, xe, ljff)
    e0 = osys.energies(np.zeros((1, 1, 3)))[0][0]
    assert e0 == pytest.approx(g["origin_energy"], abs=g["atol"])
    x2 = sc.box.c_to_f @ np.array(g["point2_cart"])
    e2 = osys.energies(x2.reshape(1, 1, 3))[0][0]
    assert e2 == pytest.approx(g["point2_energy"], abs=g["atol"])


def _nu1000():
    cr = pmgb.read_cif(DATA / "crystals" / "NU-1000_Greg.cif")
    rep = oracle.replication_factors(cr.box.f_to_c, 12.5)
    return pmgb.replicate(cr, rep)


def test_nu1000_ewald_params_and_ions(golden):
    # test/electrostatics.jl:12-46
    g = golden["nu1000_ewald"]
    sc = _nu1000()
    alpha, k2 = oracle.determine_ewald_params(g["sr_cutoff"], g["eps"])
    f, cf, r, om = oracle.box(sc.box.a, sc.box.b, sc.box.c, sc.box.alpha, sc.box.beta, sc.box.gamma)
    kreps = oracle.required_kreps(r, k2)
    assert list(kreps) == g["kreps"]
    assert alpha == pytest.approx(g["alpha"], abs=g["alpha_atol"])
    abc, wt = oracle.precompute_kvec_wts(kreps, r, alpha, om, k2)
    sid = {s: i for i, s in enumerate(sorted(set(sc.atoms.species)))}
    osys = oracle.OracleSystem(sc.box.f_to_c, sc.atoms.xf, [sid[s] for s in sc.atoms.species], sc.charges.xf,
                               sc.charges.q, np.zeros((len(sid), len(sid))), np.ones((len(sid), len(sid))),
                               g["sr_cutoff"] ** 2, [], [g["q"]])
    osys.set_ewald(alpha, g["sr_cutoff"], kreps, abc, wt)
    for x, want, atol in g["ions"]:
        xf = (sc.box.c_to_f @ np.array(x)).reshape(1, 1, 3)
        _, sr, lr = osys.energies(np.zeros((1, 0, 3)), xf, charged=True, use_sk=False)
        assert sr[0] + lr[0] == pytest.approx(want, abs=atol)
        # the structure-factor form of the same long-range sum
        _, sr2, lr2 = osys.energies(np.zeros((1, 0, 3)), xf, charged=True, use_sk=True)
        assert lr2[0] == pytest.approx(lr[0], rel=1e-10, abs=1e-8)
        assert sr2[0] == sr[0]


def test_host_ewald_setup_equals_oracle():
    # the product's host-side Ewald set-up (pmgb.setup_Ewald_sum) against the oracle
    for sc in [_nu1000(), pmgb.replicate(pmgb.read_cif(DATA / "crystals" / "CAXVII_clean.cif"), (2, 1, 1))]:
        ep = pmgb.setup_Ewald_sum(sc.box, 12.5, eps=1e-6)
        alpha, k2 = oracle.determine_ewald_params(12.5, 1e-6)
        assert ep.alpha == alpha
        kreps = oracle.required_kreps(sc.box.reciprocal_lattice, k2)
        assert tuple(ep.kreps) == kreps
        abc, wt = oracle.precompute_kvec_wts(kreps, sc.box.reciprocal_lattice, alpha, sc.box.Omega, k2)
        np.testing.assert_array_equal(ep.kvec_abc, abc)
        np.testing.assert_allclose(ep.kvec_wt, wt, rtol=1e-13)


def test_required_kreps(golden):
    # test/electrostatics.jl:27-31
    g = golden["required_kreps"]
    b = [x * 2 * math.pi for x in g["box"]]
    f, cf, r, om = oracle.box(*b, math.pi / 2, math.pi / 2, math.pi / 2)
    for kmag, want in g["cases"]:
        assert list(oracle.required_kreps(r, kmag ** 2)) == want
        assert list(pmgb.required_kreps(pmgb.Box(*b, math.pi / 2, math.pi / 2, math.pi / 2), kmag ** 2)) == want


def _nist_config(c, q_h):
    lines = (DATA / "nist" / f"spce_sample_config_periodic{c}.txt").read_text().splitlines()
    dims = [float(v) for v in lines[0].split()]
    n = int(lines[1]) * 3
    x = np.array([[float(v) for v in lines[2 + i].split()[1:4]] for i in range(n)])
    q = np.array([(-2 * q_h if lines[2 + i].split()[-1] == "O" else q_h) for i in range(n)])
    return dims, x, q


@pytest.mark.parametrize("c", [1, 2, 3, 4])
def test_nist_spce_real_fourier_self(golden, c):
    # test/electrostatics.jl:48-125: the NIST SPC/E reference sums, rebuilt from the
    # guest-host primitives (S(k) weights and the erfc real-space pair term)
    g = golden["nist_spce"]
    dims, x, q = _nist_config(c, g["q_H"])
    box = pmgb.Box(*dims, math.pi / 2, math.pi / 2, math.pi / 2)
    xf = (box.c_to_f @ x.T).T
    alpha = g["alpha_times_L"] / box.a
    abc, wt = oracle.precompute_kvec_wts(g["kreps"], box.reciprocal_lattice, alpha, box.Omega)
    keep = (abc ** 2).sum(axis=1) < g["k2_int_max"]
    abc, wt = abc[keep], wt[keep]
    one = np.zeros((1, 1))
    full = oracle.OracleSystem(box.f_to_c, np.zeros((0, 3)), [], xf, q, one, one + 1, g["sr_cutoff"] ** 2, [], [])
    full.set_ewald(alpha, g["sr_cutoff"], g["kreps"], abc, wt)
    sk = full.structure_factor()
    fourier = 0.5 * np.sum(wt * np.abs(sk) ** 2)
    assert fourier == pytest.approx(g["fourier"][c - 1], rel=g["rtol"])
    self_e = -alpha / math.sqrt(math.pi) / oracle.four_pi_eps0() * np.sum(q ** 2)
    assert self_e == pytest.approx(g["self"][c - 1], rel=g["rtol"])
    # real space: every molecule against the charges of all other molecules
    nmol = x.shape[0] // 3
    real = 0.0
    for m in range(nmol):
        others = np.ones(x.shape[0], dtype=bool)
        others[3 * m:3 * m + 3] = False
        s = oracle.OracleSystem(box.f_to_c, np.zeros((0, 3)), [], xf[others], q[others], one, one + 1,
                                g["sr_cutoff"] ** 2, [], q[3 * m:3 * m + 3])
        s.set_ewald(alpha, g["sr_cutoff"], (0, 0, 0), np.zeros((0, 3)), np.zeros(0))
        _, sr, _ = s.energies(np.zeros((1, 0, 3)), xf[3 * m:3 * m + 3].reshape(1, 3, 3), charged=True, use_sk=True)
        real += sr[0]
    assert 0.5 * real == pytest.approx(g["real"][c - 1], rel=g["rtol"])


def test_zif71_co2(golden):
    # test/electrostatics.jl:130-160 (guest-host parts)
    g = golden["zif71_co2"]
    cr = pmgb.read_cif(DATA / "crystals" / "zif71_bogus_charges.cif")
    pmgb.strip_numbers_from_atom_labels(cr)
    ff = pmgb.LJForceField("Greg_bogus_ZIF71", r_cutoff=g["r_cutoff"])
    co2 = pmgb.read_molecule("CO2EPM2")
    osys, _ = _sys_from_crystal(cr, co2, ff, charged=True)
    ep = pmgb.setup_Ewald_sum(cr.box, g["es_sr_cutoff"], eps=1e-6)
    osys.set_ewald(ep.alpha, ep.sr_cutoff_r, ep.kreps, ep.kvec_abc, ep.kvec_wt)
    pos1 = np.array(g["co2_1"]).reshape(1, 3, 3)
    pos2 = np.array(g["co2_2"]).reshape(1, 3, 3)
    v1, sr1, lr1 = osys.energies(pos1, pos1, charged=True)
    v2, sr2, lr2 = osys.energies(pos2, pos2, charged=True)
    assert v1[0] == pytest.approx(g["vdw_1"], abs=g["vdw_atol"])
    assert sr1[0] + lr1[0] == pytest.approx(g["es_1"], abs=g["es_atol"])
    assert v1[0] + v2[0] == pytest.approx(g["vdw_both"], abs=g["vdw_both_atol"])
    assert sr1[0] + lr1[0] + sr2[0] + lr2[0] == pytest.approx(g["es_both"], abs=g["es_both_atol"])


def test_forcefield_and_replication(golden):
    # test/forcefield.jl:12-30
    g = golden["forcefield_dreiding"]
    ljff = pmgb.LJForceField("Dreiding", r_cutoff=12.5, mixing_rules="Lorentz-Berthelot")
    assert ljff.pure_sigma["He"] == g["sigma_He"]
    assert ljff.pure_epsilon["Zn"] == g["epsilon_Zn"]
    assert ljff.sigma2["Zn"]["He"] == g["sigma2_Zn_He"]
    assert ljff.epsilon["He"]["Zn"] == g["epsilon_He_Zn"]
    assert ljff.epsilon["He"]["Zn"] == ljff.epsilon["Zn"]["He"]
    assert ljff.r2_cutoff == 12.5 ** 2
    cr = pmgb.read_cif(DATA / "crystals" / "test_structure.cif")
    pmgb.strip_numbers_from_atom_labels(cr)
    assert pmgb.replication_factors(cr.box, ljff) == tuple(g["rep_test_structure"])
    assert oracle.replication_factors(cr.box.f_to_c, 12.5) == tuple(g["rep_test_structure"])
    sb = pmgb.read_cif(DATA / "crystals" / "SBMOF-1.cif")
    assert pmgb.forcefield_coverage(sb, ljff)


def test_philox_known_answers():
    # Philox4x32-10 known-answer vectors (Salmon et al., SC'11 reference implementation)
    ctr = [[0, 0, 0, 0], [0xFFFFFFFF] * 4, [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]]
    key = [[0, 0], [0xFFFFFFFF] * 2, [0xA4093822, 0x299F31D0]]
    want = [[0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8],
            [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD],
            [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]]
    np.testing.assert_array_equal(oracle.philox4x32_10(ctr, key), np.array(want, dtype=np.uint32))


def test_direct_and_sk_forms_agree_triclinic():
    # the S(k) restatement equals the reference's direct e^{ik·r} form on a fully
    # triclinic charged cell (CAXVII, three non-90° angles)
    cr = pmgb.read_cif(DATA / "crystals" / "CAXVII_clean.cif")
    rep = oracle.replication_factors(cr.box.f_to_c, 12.5)
    sc = pmgb.replicate(cr, rep)
    ep = pmgb.setup_Ewald_sum(sc.box, 12.5, eps=1e-6)
    sid = {s: i for i, s in enumerate(sorted(set(sc.atoms.species)))}
    z = np.zeros((len(sid), len(sid)))
    osys = oracle.OracleSystem(sc.box.f_to_c, sc.atoms.xf, [sid[s] for s in sc.atoms.species], sc.charges.xf,
                               sc.charges.q, z, z + 1, 12.5 ** 2, [], [0.7, -0.35, -0.35])
    osys.set_ewald(ep.alpha, 12.5, ep.kreps, ep.kvec_abc, ep.kvec_wt)
    rng = np.random.default_rng(7)
    pos = rng.random((20, 3, 3))
    _, sr_d, lr_d = osys.energies(np.zeros((20, 0, 3)), pos, charged=True, use_sk=False)
    _, sr_s, lr_s = osys.energies(np.zeros((20, 0, 3)), pos, charged=True, use_sk=True)
    np.testing.assert_array_equal(sr_d, sr_s)
    np.testing.assert_allclose(lr_s, lr_d, rtol=1e-11, atol=1e-9)


def test_oracle_accessible_matches_host_mirror():
    """The oracle's vectorised gate and the Python mirror of grid.jl:813-836 agree, including
    points on the periodic faces and rounding ties."""
    import pmgb
    from pmgb.grid import Grid, accessible

    rng = np.random.default_rng(8)
    data = rng.random((4, 5, 3)) < 0.15
    g = Grid(pmgb.Box(10.0, 11.0, 12.0, np.pi / 2, np.pi / 2, np.pi / 2), data.shape, data, "K", np.zeros(3))
    rep = (2, 1, 3)
    xf = np.vstack([rng.random((400, 3)), [[0.0, 0.0, 0.0], [0.5 / 2, 0.5, 0.5 / 3], [0.999999, 0.5, 0.25]]])
    got = oracle.accessible(data, xf, rep)
    want = np.array([accessible(g, x, rep) for x in xf])
    np.testing.assert_array_equal(got, want)
