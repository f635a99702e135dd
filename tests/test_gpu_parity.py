"""GPU parity: libpmgb (sm_103a) against the FP64 oracle and the reference's golden values.

Tolerances (from the hot-path contract): per-configuration energies within 1e-5 relative
or 1e-4 K absolute -- asserted for every configuration and grid point of the exact path
(the default); block log Σ e^{-U/T} and ⟨U⟩ within 1e-6 relative; golden values at the
reference tests' own tolerances.  The FP32 pass alone (exact energies off) is checked against
its own error model: 4e-6 of the sum of the terms' magnitudes plus 1e-4 K.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
import pmgb
from conftest import DATA
from pm_helpers import oracle_for, oracle_sites_split, random_configs, widom_with_oracle, within
from pmgb import synthetic

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-4
# FP32 pair math: each pair term carries ~1e-7 relative rounding (more for the r^-12 part),
# so an energy is accurate to a small multiple of 1e-7 of the sum of its terms' magnitudes
FP32_SCALE_TOL = 4e-6
# the double-float pass (~48 bits): far inside the tolerance, relative to the terms' magnitudes
DF_SCALE_TOL, DF_ATOL = 1e-9, 1e-8


def _report(name, gpu, ref):
    fin = np.isfinite(ref)
    err = np.abs(gpu[fin] - ref[fin])
    rel = err / np.maximum(np.abs(ref[fin]), 1e-30)
    print(f"[{name}] n={fin.sum()} max|d|={err.max():.3e} K  max rel={rel.max():.3e}  "
          f"median|d|={np.median(err):.3e} K")


# ---------------------------------------------------------------------------- RNG
def test_philox_device_matches_oracle(ctx):
    rng = np.random.default_rng(3)
    ctr = rng.integers(0, 2 ** 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, size=(4096, 2), dtype=np.uint64).astype(np.uint32)
    ctr[0], key[0] = 0, 0
    np.testing.assert_array_equal(ctx.philox4x32_10(ctr, key), oracle.philox4x32_10(ctr, key))


def test_poses_are_uniform_rotations(ctx):
    xf, rot = ctx.sample_poses(seed=11, start=0, n=20000)
    assert np.all((xf >= 0) & (xf < 1))
    R = rot.reshape(-1, 3, 3).transpose(0, 2, 1).astype(np.float64)  # column-major -> matrices
    np.testing.assert_allclose(np.einsum("nij,nkj->nik", R, R), np.broadcast_to(np.eye(3), R.shape), atol=2e-6)
    np.testing.assert_allclose(np.linalg.det(R), 1.0, atol=5e-6)
    # uniformity: a rotated unit vector covers the sphere evenly (mean ~ 0, second moment ~ I/3)
    v = R @ np.array([1.0, 0.0, 0.0])
    assert np.abs(v.mean(axis=0)).max() < 0.02
    np.testing.assert_allclose(v.T @ v / len(v), np.eye(3) / 3, atol=0.01)
    # same seed + start -> same poses; different start continues the stream
    xf2, rot2 = ctx.sample_poses(seed=11, start=100, n=10)
    np.testing.assert_array_equal(xf2, xf[100:110])
    np.testing.assert_array_equal(rot2, rot[100:110])


# ------------------------------------------------------------------- golden values
def test_golden_sbmof1_xe(golden):
    g = golden["sbmof1_xe_dreiding"]
    ljff = pmgb.LJForceField("Dreiding", r_cutoff=g["r_cutoff"])
    cr = pmgb.read_cif(DATA / "crystals" / "SBMOF-1.cif")
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ljff))
    xe = pmgb.Frac(pmgb.read_molecule("Xe"), sc.box)
    # the golden tolerance (±0.005 K) is tighter than FP32 pair math on a 12945 K repulsive
    # energy (~1e-6 relative), so the bound widens by 1e-6 of the value
    for x, want in ((np.zeros(3), g["origin_energy"]), (sc.box.c_to_f @ np.array(g["point2_cart"]),
                                                         g["point2_energy"])):
        pmgb.translate_to(xe, x)
        e = pmgb.vdw_energy(sc, xe, ljff)
        assert e == pytest.approx(want, abs=g["atol"] + 1e-6 * abs(want))


def test_golden_nu1000_ions(golden):
    g = golden["nu1000_ewald"]
    cr = pmgb.read_cif(DATA / "crystals" / "NU-1000_Greg.cif")
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, g["sr_cutoff"]))
    ep = pmgb.setup_Ewald_sum(sc.box, g["sr_cutoff"], eps=g["eps"])
    assert tuple(ep.kreps) == tuple(g["kreps"])
    for x, want, atol in g["ions"]:
        ion = pmgb.molecule_from_sites("ion", [], np.zeros((0, 3)), [g["q"]], [[0.0, 0.0, 0.0]])
        ion = pmgb.Frac(ion, sc.box)
        pmgb.translate_to(ion, sc.box.c_to_f @ np.array(x))
        phi = pmgb.electrostatic_potential_energy(sc, ion, ep)
        assert pmgb.total(phi) == pytest.approx(want, abs=atol)


def test_golden_zif71_co2(golden):
    g = golden["zif71_co2"]
    cr = pmgb.read_cif(DATA / "crystals" / "zif71_bogus_charges.cif")
    pmgb.strip_numbers_from_atom_labels(cr)
    ff = pmgb.LJForceField("Greg_bogus_ZIF71", r_cutoff=g["r_cutoff"])
    ep = pmgb.setup_Ewald_sum(cr.box, g["es_sr_cutoff"], eps=1e-6)
    tot_v, tot_e = 0.0, 0.0
    for pos, wv, we in [(g["co2_1"], g["vdw_1"], g["es_1"]), (g["co2_2"], None, None)]:
        co2 = pmgb.Frac(pmgb.read_molecule("CO2EPM2"), cr.box)
        co2.atom_x = np.array(pos)
        co2.charge_x = np.array(pos)
        v = pmgb.vdw_energy(cr, co2, ff)
        e = pmgb.total(pmgb.electrostatic_potential_energy(cr, co2, ep))
        if wv is not None:
            assert v == pytest.approx(wv, abs=g["vdw_atol"])
            assert e == pytest.approx(we, abs=g["es_atol"])
        tot_v += v
        tot_e += e
    assert tot_v == pytest.approx(g["vdw_both"], abs=g["vdw_both_atol"])
    assert tot_e == pytest.approx(g["es_both"], abs=g["es_both_atol"])


# ------------------------------------------------------ random configurations
def _c0_system():
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    return pmgb.GPUSystem(sc, pmgb.Frac(synthetic.ch4(), sc.box), ff)


def _c1_system(cr=None):
    cr = cr or synthetic.config1()
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    return pmgb.GPUSystem(sc, pmgb.Frac(synthetic.co2(), sc.box), ff, ep)


@pytest.fixture(scope="module")
def c0():
    return _c0_system()


@pytest.fixture(scope="module")
def c1():
    return _c1_system()


@pytest.fixture(scope="module")
def c1p():
    return _c1_system(synthetic.config1_porous())


class _fp32_only:
    """Run a block with exact energies off (the FP32 pass alone), restoring them after."""

    def __init__(self, gs):
        self.gs = gs

    def __enter__(self):
        self.gs.set_exact(False)

    def __exit__(self, *exc):
        self.gs.set_exact(True)


def test_random_configs_lj(c0):
    sites, lj, _ = random_configs(c0, 4000, seed=5)
    gpu = c0.energies(sites)
    o = oracle_for(c0)
    v, _, _, sv, _ = o.energies(lj, scales=True)
    _report("c0 vdw", gpu[:, 0], v)
    assert np.array_equal(np.isinf(gpu[:, 0]), np.isinf(v))
    ok = within(gpu[:, 0], v, RTOL, ATOL)
    for i in np.flatnonzero(~ok)[:12]:
        print(f"  outlier {i}: gpu {gpu[i, 0]!r} oracle {v[i]!r} term scale {sv[i]:.4g} K")
    print(f"[c0 vdw] {ok.mean() * 100:.3f}% within 1e-5 rel / 1e-4 K")
    assert ok.all(), f"{(~ok).sum()} configurations outside tolerance"
    fin = np.isfinite(v)
    assert np.all(np.abs(gpu[fin, 0] - v[fin]) <= DF_SCALE_TOL * sv[fin] + DF_ATOL)
    assert c0.refined_count() == len(sites)


def test_random_configs_lj_fp32(c0):
    sites, lj, _ = random_configs(c0, 4000, seed=5)
    with _fp32_only(c0):
        gpu = c0.energies(sites)
    v, _, _, sv, _ = oracle_for(c0).energies(lj, scales=True)
    assert np.array_equal(np.isinf(gpu[:, 0]), np.isinf(v))
    ok = within(gpu[:, 0], v, RTOL, ATOL)
    print(f"[c0 vdw, FP32 pass] {ok.mean() * 100:.3f}% within 1e-5 rel / 1e-4 K")
    fin = np.isfinite(v)
    assert np.all(np.abs(gpu[fin, 0] - v[fin]) <= FP32_SCALE_TOL * sv[fin] + ATOL)


def _lr_scale(gs, q_sites):
    """Σ_k |wt_k S(k)| |Σ_g q_g e^{-ik.x_g}| per configuration (the magnitude the FP32
    reciprocal-space sum is computed from)."""
    ep = gs.eparams
    sk = gs.structure_factor()
    abc = ep.kvec_abc.astype(np.float64)
    q = gs.molecule.charge_q
    G = np.zeros((q_sites.shape[0], abc.shape[0]), dtype=complex)
    for g in range(q_sites.shape[1]):
        G += q[g] * np.exp(-2j * np.pi * (q_sites[:, g, :] @ abc.T))
    return (np.abs(ep.kvec_wt * sk)[None, :] * np.abs(G)).sum(axis=1)


@pytest.mark.parametrize("exact", [True, False])
def test_random_configs_ewald(c1, exact):
    sites, lj, q = random_configs(c1, 1024, seed=6)
    c1.set_exact(exact)
    try:
        gpu = c1.energies(sites)
    finally:
        c1.set_exact(True)
    o = oracle_for(c1)
    v, sr, lr, sv, ss = o.energies(lj, q, charged=True, use_sk=True, scales=True)
    tag = "" if exact else ", FP32 pass"
    _report("c1 vdw" + tag, gpu[:, 0], v)
    _report("c1 es sr" + tag, gpu[:, 1], sr)
    _report("c1 es lr" + tag, gpu[:, 2], lr)
    assert np.array_equal(np.isinf(gpu[:, 0]), np.isinf(v))
    fin = np.isfinite(v)
    sl = _lr_scale(c1, q)
    tol, atol = (DF_SCALE_TOL, DF_ATOL) if exact else (FP32_SCALE_TOL, ATOL)
    assert np.all(np.abs(gpu[fin, 0] - v[fin]) <= tol * sv[fin] + atol)
    assert np.all(np.abs(gpu[:, 1] - sr) <= tol * ss + atol)
    assert np.all(np.abs(gpu[:, 2] - lr) <= tol * sl + atol)
    tot_g = gpu[fin].sum(axis=1)
    tot_o = (v + sr + lr)[fin]
    _report("c1 total" + tag, tot_g, tot_o)
    ok = within(tot_g, tot_o, RTOL, ATOL)
    print(f"[c1 total{tag}] {ok.mean() * 100:.2f}% within 1e-5 rel / 1e-4 K; median term scales: LJ "
          f"{np.median(sv[fin]):.3g} K, real {np.median(ss):.3g} K, recip {np.median(sl):.3g} K")
    if exact:
        # every component and the total within the per-configuration tolerance
        assert ok.all()
        for g, ref in ((gpu[fin, 0], v[fin]), (gpu[:, 1], sr), (gpu[:, 2], lr)):
            assert within(g, ref, RTOL, ATOL).all()


def test_kvectors_of_replicated_cells(c1):
    """A replicated framework: S(k) vanishes unless n_d | k_d for the replication factors n, so
    only those k-vectors are evaluated; with one charge moved off its replica positions every
    k-vector is kept.  Both agree with the oracle, which sums over every k-vector."""
    from dataclasses import replace

    cr, ff = synthetic.config1(), synthetic.forcefield()
    reps = np.asarray(pmgb.replication_factors(cr.box, ff))
    abc = c1.eparams.kvec_abc
    info = c1.info()
    assert info["n_kvecs"] == len(abc)
    assert info["n_kvecs_evaluated"] == np.all(abc % reps == 0, axis=1).sum() < len(abc) // 4
    sc = pmgb.replicate(cr, reps)
    xf = sc.charges.xf.copy()
    xf[0] += 1e-3
    moved = replace(sc, charges=replace(sc.charges, xf=xf))
    ep = pmgb.setup_Ewald_sum(moved.box, ff.r_cutoff, eps=1e-6)
    gs = pmgb.GPUSystem(moved, pmgb.Frac(synthetic.co2(), moved.box), ff, ep)
    assert gs.info()["n_kvecs_evaluated"] == len(ep.kvec_abc)
    for sys_ in (c1, gs):
        sites, lj, q = random_configs(sys_, 512, seed=16)
        with _fp32_only(sys_):  # the FP32 pass evaluates only the kept k-vectors
            gpu = sys_.energies(sites)
        _, _, lr, _, _ = oracle_for(sys_).energies(lj, q, charged=True, use_sk=True, scales=True)
        assert np.all(np.abs(gpu[:, 2] - lr) <= FP32_SCALE_TOL * _lr_scale(sys_, q) + ATOL)


def test_direct_form_cross_check(c1):
    # a few configurations against the reference's direct e^{ik·r} form
    sites, lj, q = random_configs(c1, 8, seed=9)
    gpu = c1.energies(sites)
    o = oracle_for(c1)
    v, sr, lr = o.energies(lj, q, charged=True, use_sk=False)
    fin = np.isfinite(v)
    assert within(gpu[fin].sum(axis=1), (v + sr + lr)[fin], RTOL, 1e-3).all()


# ------------------------------------------------------------------ Widom path
def _widom_parity(gs, n_per_block, seed, T=298.0, use_sk=True):
    return widom_with_oracle(gs, n_per_block, seed, T, use_sk)


def _check_blocks(blocks, u_gpu, T, n_per_block):
    # the device log-sum-exp reduction against FP64 sums of the device's own energies
    ref = oracle.widom_blocks_log(u_gpu[:, 0], u_gpu[:, 1], T, 5, n_per_block)
    np.testing.assert_allclose(blocks[:, 0], ref[:, 0], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(blocks[:, 1], ref[:, 1], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(blocks[:, 2], ref[:, 2], rtol=1e-10, atol=1e-9)
    np.testing.assert_array_equal(blocks[:, 3], ref[:, 3])


def _kh_u_errors(blocks, v, es, T, npb):
    ref = oracle.widom_blocks_log(v, es, T, 5, npb)
    kh_rel = np.abs(np.expm1(blocks[:, 0] - ref[:, 0]))       # relative error of Σ e^{-U/T}
    u_ref = ref[:, 1] + ref[:, 2]
    u_rel = np.abs((blocks[:, 1] + blocks[:, 2]) - u_ref) / np.abs(u_ref)
    return kh_rel, u_rel, ref


def test_widom_parity_lj(c0):
    npb, T = 4000, 298.0
    blocks, u, v, es = _widom_parity(c0, npb, seed=21, T=T)
    _report("widom c0 vdw", u[:, 0], v)
    assert np.array_equal(np.isinf(u[:, 0]), np.isinf(v))
    _check_blocks(blocks, u, T, npb)
    kh_rel, u_rel, ref = _kh_u_errors(blocks, v, es, T, npb)
    print(f"[widom c0] block K_H rel err max {kh_rel.max():.3e}; <U> rel err max {u_rel.max():.3e}")
    assert kh_rel.max() < 1e-6
    assert u_rel.max() < 1e-6
    # the reference's plain FP64 sums agree where they do not underflow
    plain = oracle.widom_blocks(v, es, T, 5, npb)
    np.testing.assert_allclose(np.log(plain[:, 0]), ref[:, 0], rtol=1e-12)


def test_widom_parity_ewald_porous(c1p):
    npb, T = 40000, 298.0
    blocks, u, v, es = _widom_parity(c1p, npb, seed=22, T=T)
    _report("widom c1 porous vdw", u[:, 0], v)
    _report("widom c1 porous es", u[:, 1], es)
    _check_blocks(blocks, u, T, npb)
    ref = oracle.widom_blocks_log(v, es, T, 5, npb)
    dlog = blocks[:, 0] - ref[:, 0]                    # log K_H(GPU) - log K_H(oracle), per block
    # first-order propagation of the per-insertion energy differences through the weights
    uo = (v + es).reshape(5, npb)
    ug = (u[:, 0] + u[:, 1]).reshape(5, npb)
    fin = np.isfinite(uo) & np.isfinite(ug)
    x = np.where(fin, -uo / T, -np.inf)
    w = np.exp(x - x.max(axis=1, keepdims=True))
    w /= w.sum(axis=1, keepdims=True)
    pred = -(w * np.where(fin, ug - uo, 0.0)).sum(axis=1) / T
    n_eff = 1.0 / (w ** 2).sum(axis=1)
    print(f"[widom c1 porous] Δlog K_H {dlog}; first-order prediction {pred}; N_eff {n_eff}")
    # the device weighting is the Boltzmann weighting (to second order in the tiny δU/T)
    np.testing.assert_allclose(dlog, pred, atol=1e-8)
    # FP32 Coulomb pair terms (~1e-7 relative on terms of 1e4 K) bound the per-insertion
    # error; with N_eff ~ 1 a block's K_H inherits it directly
    assert np.abs(dlog).max() < 5e-5


def test_widom_parity_ewald_dense(c1):
    # the dense 600-atom cell: every insertion is repulsive, so Σ e^{-U/T} underflows in
    # plain FP64 (the reference would report K_H = 0 and <U> = NaN); compare in log space
    npb, T = 1000, 298.0
    blocks, u, v, es = _widom_parity(c1, npb, seed=23, T=T)
    _report("widom c1 vdw", u[:, 0], v)
    _check_blocks(blocks, u, T, npb)
    kh_rel, u_rel, ref = _kh_u_errors(blocks, v, es, T, npb)
    print(f"[widom c1 dense] |Δ log Σbf| max {np.abs(blocks[:, 0] - ref[:, 0]).max():.3e}; log Σbf {ref[:, 0]}")
    assert np.abs(blocks[:, 0] - ref[:, 0]).max() < 1e-6 * np.abs(ref[:, 0]).max()


def test_kernel_timing(c0):
    """pmgb_set_kernel_timing: one event pair per Widom pass around its pair kernel."""
    ctx = c0.ctx
    ctx.set_kernel_timing(True)
    c0.widom(2000, 5, 1, 298.0)
    c0.widom(2000, 5, 2, 298.0)
    ms, n = ctx.kernel_timing()
    assert n == 2 and ms > 0.0
    assert ctx.kernel_timing() == (0.0, 0)  # cleared by the read
    ctx.set_kernel_timing(False)
    c0.widom(2000, 5, 3, 298.0)
    assert ctx.kernel_timing() == (0.0, 0)


def test_widom_deterministic(c0):
    a, _ = c0.widom(3000, 5, 77, 298.0)
    b, _ = c0.widom(3000, 5, 77, 298.0)
    np.testing.assert_array_equal(a, b)


def test_widom_ragged_block_sizes(c0):
    # block sizes that are not multiples of the CTA size, including a single insertion
    for npb in (1, 255, 257, 1000):
        blocks, u = c0.widom(npb, 5, 5, 298.0, want_energies=True)
        _check_blocks(blocks, u, 298.0, npb)


# ------------------------------------------------------------------ energy grid
def test_energy_grid_parity():
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    g = pmgb.energy_grid(cr, synthetic.xe(), ff, resolution=(17, 13, 11), units="K", verbose=False)
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.xe(), sc.box), ff)
    ref = oracle_for(gs).energy_grid((17, 13, 11), rep)
    _report("grid", g.data.astype(np.float64).ravel(), ref.ravel())
    assert np.array_equal(np.isinf(g.data), np.isinf(ref))
    ok = within(g.data.astype(np.float64), ref, RTOL, ATOL)
    print(f"[grid] {ok.mean() * 100:.3f}% of points within 1e-5 rel / 1e-4 K")
    assert ok.all()
    # every point within the FP32 error bound of its terms' magnitudes (the end planes
    # evaluate the first plane's position, as the reference's periodic images)
    pts = np.stack(np.meshgrid(*[np.arange(n) / (n - 1) for n in (17, 13, 11)], indexing="ij"), axis=-1)
    pts = (np.where(pts >= 1.0, 0.0, pts) / np.array(rep)).reshape(-1, 3)
    v, _, _, sv, _ = oracle_for(gs).energies(pts[:, None, :], scales=True)
    gd = g.data.astype(np.float64).reshape(-1)
    fin = np.isfinite(v)
    assert np.all(np.abs(gd[fin] - v[fin]) <= FP32_SCALE_TOL * sv[fin] + ATOL)
    gk = pmgb.energy_grid(cr, synthetic.xe(), ff, resolution=(17, 13, 11), units="kJ_mol", verbose=False)
    np.testing.assert_allclose(gk.data, g.data * (8.314 / 1000.0), rtol=2e-7)


@pytest.mark.parametrize("case", ["config0_xe", "config1_ch4", "porous_ch4"])
def test_energy_grid_every_point_within_tolerance(case):
    """The exact grid on tens of thousands of points: the FP32 pass with its per-point error
    estimate, and the points the estimate cannot clear re-evaluated in double-float.  Every
    point meets 1e-5 relative or 1e-4 K; the points left at their FP32 values are exactly those
    the FP32-only grid holds, and only a small fraction is re-evaluated."""
    cr, probe = {"config0_xe": (synthetic.config0, synthetic.xe), "config1_ch4": (synthetic.config1, synthetic.ch4),
                 "porous_ch4": (synthetic.config1_porous, synthetic.ch4)}[case]
    cr, probe = cr(), probe()
    ff = synthetic.forcefield()
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(probe, sc.box), ff)
    n_pts = (41, 37, 33)
    exact = gs.energy_grid(n_pts, rep, 1.0)
    n_ref = gs.refined_count()
    with _fp32_only(gs):
        fp32 = gs.energy_grid(n_pts, rep, 1.0)
    ref = oracle_for(gs).energy_grid(n_pts, rep)
    assert np.array_equal(np.isinf(exact), np.isinf(ref))
    e64 = exact.astype(np.float64)
    ok = within(e64, ref, RTOL, ATOL)
    ok32 = within(fp32.astype(np.float64), ref, RTOL, ATOL)
    changed = (exact != fp32) & np.isfinite(fp32)
    print(f"[grid {case}] {exact.size} points: {n_ref} re-evaluated ({n_ref / exact.size * 100:.2f}%); FP32 pass alone "
          f"{ok32.mean() * 100:.3f}% within tolerance; exact {ok.mean() * 100:.3f}%")
    assert ok.all(), f"{(~ok).sum()} points outside tolerance"
    assert changed.sum() <= n_ref
    assert n_ref < 0.1 * exact.size


@pytest.mark.parametrize("name", ["LTA.cif", "SOD.cif"])
def test_energy_grid_periodic_endpoints(golden, name):
    # test/grid.jl:43-55
    g = golden["grid_periodic"]
    cr = pmgb.read_cif(DATA / "crystals" / name)
    grid = pmgb.energy_grid(cr, pmgb.read_molecule("CH4"), pmgb.LJForceField("UFF"), resolution=g["resolution"],
                            verbose=False)
    d = grid.data.astype(np.float64).copy()
    d[d > g["cap"]] = 0.0
    np.testing.assert_allclose(d[0], d[-1], atol=g["atol"])
    np.testing.assert_allclose(d[:, 0], d[:, -1], atol=g["atol"])
    np.testing.assert_allclose(d[:, :, 0], d[:, :, -1], atol=g["atol"])


# ------------------------------------------------------ henry_coefficient drop-in
def test_henry_drop_in_matches_oracle():
    cr = synthetic.config0()
    ff = synthetic.forcefield()
    holder = []
    res = pmgb.henry_coefficient(cr, synthetic.ch4(), 298.0, ff, insertions_per_volume=0.5, verbose=False,
                                 autosave=False, seed=1234, system_out=holder)
    assert len(res) == 16
    gs = holder[0]
    npb = res.n_insertions_per_block
    blocks, u, v, es = _widom_parity(gs, npb, seed=1234)
    ref = oracle.widom_blocks(v, es, 298.0, 5, npb)  # the reference's own block sums
    kh_ref = np.mean(ref[:, 0] / (pmgb.UNIV_GAS_CONST * 298.0 * npb))
    print(f"[henry drop-in] K_H {res['henry coefficient [mol/(m³-bar)]']:.9e} vs oracle {kh_ref:.9e}")
    assert res["henry coefficient [mol/(m³-bar)]"] == pytest.approx(kh_ref, rel=1e-6)
    assert res["⟨U, vdw⟩ (K)"] == pytest.approx(np.mean(ref[:, 1] / ref[:, 0]), rel=1e-6)


def test_henry_statistical_xe_sbmof1(golden, ref_masses):
    # test/henry.jl:13-21 (rtol 2.5%, 500 insertions per Å³)
    g = golden["henry_statistical"]
    cr = pmgb.read_cif(DATA / "crystals" / "SBMOF-1.cif")
    res = pmgb.henry_coefficient(cr, pmgb.read_molecule("Xe"), 298.0, pmgb.LJForceField("Dreiding", r_cutoff=12.5),
                                 insertions_per_volume=g["insertions_per_volume"], verbose=False, autosave=False,
                                 seed=1, masses=ref_masses)
    assert res["henry coefficient [mol/(kg-Pa)]"] == pytest.approx(g["xe_sbmof1"]["kh_mol_kg_pa"], rel=g["rtol"])
    assert res["⟨U⟩ (kJ/mol)"] == pytest.approx(g["xe_sbmof1"]["u_kj_mol"], rel=g["rtol"])


def test_henry_statistical_co2_caxvii(golden, ref_masses):
    # test/henry.jl:26-34 (charged, fully triclinic cell)
    g = golden["henry_statistical"]
    cr = pmgb.read_cif(DATA / "crystals" / "CAXVII_clean.cif")
    mol = pmgb.read_molecule("CO2")
    res = pmgb.henry_coefficient(cr, mol, 298.0, pmgb.LJForceField("Dreiding", r_cutoff=12.5),
                                 insertions_per_volume=g["insertions_per_volume"], verbose=False, autosave=False,
                                 seed=2, masses=ref_masses)
    assert res["henry coefficient [mol/(kg-Pa)]"] == pytest.approx(g["co2_caxvii"]["kh_mol_kg_pa"], rel=g["rtol"])
    assert res["⟨U⟩ (kJ/mol)"] == pytest.approx(g["co2_caxvii"]["u_kj_mol"], rel=g["rtol"])
    np.testing.assert_array_equal(mol.atom_x, pmgb.read_molecule("CO2").atom_x)  # the molecule is not modified


# ------------------------------------------------------------------ error paths
def test_errors_are_reported_not_crashes(c0, c1, ctx):
    with pytest.raises(pmgb.PMGBError, match="temperature"):
        c0.widom(10, 5, 1, 0.0)
    with pytest.raises(pmgb.PMGBError, match="single site"):
        c1.energy_grid((4, 4, 4), (1, 1, 1), 1.0)
    cr = synthetic.config1()
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, (2, 2, 3))
    no_ewald = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.co2(), sc.box), ff, None)
    with pytest.raises(pmgb.PMGBError, match="set_ewald"):
        no_ewald.widom(10, 5, 1, 298.0)
    assert ctx.device_status() == 0
