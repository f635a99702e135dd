"""Host-side logic and the C-ABI library surface (no GPU needed)."""
from __future__ import annotations

import ctypes
import math
import re
from pathlib import Path

import numpy as np
import pytest

import pmgb
from conftest import DATA, ROOT


def test_abi_exports_every_declared_symbol():
    header = (ROOT / "include" / "pmgb.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|void|const char\*)\s+(pmgb_\w+)\s*\(", header, flags=re.M))
    assert len(declared) >= 20
    lib_path = ROOT / "porousmaterials.jl_gb300" / "pmgb" / "libpmgb.so"
    if not lib_path.exists():
        pytest.skip("libpmgb.so not built")
    lib = ctypes.CDLL(str(lib_path))  # loads without a GPU: no CUDA call happens at load time
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    bound = {name for name, _, _ in pmgb._lib.SIGNATURES}
    assert declared == bound, (declared ^ bound)
    lib.pmgb_abi_version.restype = ctypes.c_int
    assert lib.pmgb_abi_version() == 1


def test_cif_reader_and_replicate():
    cr = pmgb.read_cif(DATA / "crystals" / "SBMOF-1.cif")
    assert cr.atoms.n == 120 and cr.charges.n == 120
    assert cr.box.Omega == pytest.approx(1456.472102, rel=1e-6)
    assert np.all((cr.atoms.xf >= 0) & (cr.atoms.xf < 1))
    sc = pmgb.replicate(cr, (3, 5, 2))
    assert sc.atoms.n == 120 * 30
    assert sc.box.a == pytest.approx(3 * cr.box.a)
    # image (0,0,0) first, coordinates rescaled into the supercell
    np.testing.assert_allclose(sc.atoms.xf[:120] * [3, 5, 2], cr.atoms.xf)
    assert np.all(sc.atoms.xf < 1.0)
    assert pmgb.crystal_density(cr) > 0


def test_non_p1_rejected(tmp_path):
    text = (DATA / "crystals" / "SOD.cif").read_text().replace("'x, y, z'", "'x, y, z'\n '-x, -y, z'")
    p = tmp_path / "sym.cif"
    p.write_text(text)
    cr = pmgb.read_cif(p)
    assert not cr.symmetry_is_p1
    with pytest.raises(ValueError):
        pmgb.assert_P1_symmetry(cr)


def test_molecule_reading_and_frames():
    co2 = pmgb.read_molecule("CO2")
    assert co2.atom_species == ["C_CO2", "O_CO2", "O_CO2"]
    np.testing.assert_allclose(co2.com, [0, 0, 0], atol=1e-12)
    assert pmgb.needs_rotations(co2) and not pmgb.needs_rotations(pmgb.read_molecule("Xe"))
    box = pmgb.Box(10.0, 11.0, 12.0, math.radians(80), math.radians(95), math.radians(100))
    f = pmgb.Frac(co2, box)
    back = pmgb.Cart(f, box)
    np.testing.assert_allclose(back.atom_x, co2.atom_x, atol=1e-12)
    pmgb.translate_to(f, np.array([0.25, 0.5, 0.75]))
    np.testing.assert_allclose(f.com, [0.25, 0.5, 0.75])
    R = pmgb.random_rotation_matrix(np.random.default_rng(1))
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
    assert np.linalg.det(R) == pytest.approx(1.0)


def test_grid_helpers(golden):
    # test/grid.jl:16-40, 148-177
    g = golden["required_n_pts"]
    assert pmgb.required_n_pts(pmgb.Box(*g["box"], math.pi / 2, math.pi / 2, math.pi / 2), g["dx"]) == tuple(g["n_pts"])
    nn = pmgb.grid._arg_nearest_neighbor
    assert nn((10, 20, 30), [0.001, 0.001, 0.001]) == [1, 1, 1]
    assert nn((10, 20, 30), [0.999, 0.999, 0.999]) == [10, 20, 30]
    idx = [0, 21, 31]
    pmgb.grid._apply_pbc_to_index(idx, (10, 20, 30))
    assert idx == [10, 1, 1]
    assert nn((3, 3, 3), [0.001, 0.001, 0.26]) == [1, 1, 2]
    assert nn((3, 3, 3), [0.76, 0.001, 0.26]) == [3, 1, 2]
    assert nn((4, 6, 11), [0.32, 0.42, 0.61]) == [2, 3, 7]
    assert pmgb.xf_to_id((4, 4, 4), [0.0001, 0.2400, 0.2600]) == [1, 1, 2]
    assert pmgb.xf_to_id((4, 4, 4), [-0.0001, 0.2400, 1.01]) == [4, 1, 1]
    np.testing.assert_allclose(pmgb.id_to_xf((2, 2, 2), (3, 3, 3)), [0.5, 0.5, 0.5])


def test_cube_round_trip(tmp_path):
    # test/grid.jl:20-24
    pmgb.rc["paths"]["grids"] = str(tmp_path)
    rng = np.random.default_rng(0)
    grid = pmgb.Grid(pmgb.Box(0.7, 0.8, 0.9, 1.5, 1.6, 1.7), (3, 3, 3), rng.random((3, 3, 3)), "kJ_mol",
                     np.array([1.0, 2.0, 3.0]))
    pmgb.write_cube(grid, "test_grid.cube", verbose=False)
    assert grid.isapprox(pmgb.read_cube("test_grid.cube"), atol=1e-5)


def test_accessible_lookup():
    data = np.zeros((5, 5, 5), dtype=bool)
    data[2, 2, 2] = True
    grid = pmgb.Grid(pmgb.Box(1, 1, 1, math.pi / 2, math.pi / 2, math.pi / 2), (5, 5, 5), data, "K", np.zeros(3))
    assert pmgb.accessible(grid, [0.5, 0.5, 0.5])
    assert pmgb.accessible(grid, [0.75, 0.5, 0.5])     # a neighbour of the accessible node
    assert not pmgb.accessible(grid, [0.0, 0.0, 0.0])
    assert pmgb.accessible(grid, [0.25, 0.25, 0.25], (2, 2, 2))


def test_synthetic_workloads_shapes():
    from pmgb import synthetic

    c0 = synthetic.config0()
    assert c0.atoms.n == 424 and c0.charges.n == 0
    assert {s: c0.atoms.species.count(s) for s in "Zn O C H".split()} == {"Zn": 32, "O": 104, "C": 192, "H": 96}
    c1 = synthetic.config1()
    assert c1.atoms.n == 600 and abs(c1.charges.q.sum()) < 1e-12
    ff = synthetic.forcefield()
    assert pmgb.replication_factors(c1.box, ff) == (2, 2, 3)
    ep = pmgb.setup_Ewald_sum(pmgb.replicate(c1, (2, 2, 3)).box, 12.5, eps=1e-6)
    assert ep.alpha == pytest.approx(0.24713, abs=1e-5)
    assert ep.n_kvecs == 1424
    # minimum-image separation >= 1.2 Å
    d = c0.atoms.xf[:, None, :] - c0.atoms.xf[None, :, :]
    d -= np.round(d)
    r = np.linalg.norm(d @ c0.box.f_to_c.T, axis=-1) + np.eye(c0.atoms.n) * 10
    assert r.min() >= 1.2


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from pmgb import _lib

    monkeypatch.setattr(_lib, "LIB_PATH", Path(tmp_path) / "absent.so")
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="libpmgb.so not found"):
        _lib.lib()


def test_pocket_classification_on_built_grids():
    """Flood fill, face connections and cycle classification (src/grid.jl:383-616) on grids
    built by hand: a channel that wraps along z is accessible, a closed pocket is blocked, a
    region touching only one face is blocked, and a channel that leaves by +x and comes back
    through a second segment by +y is accessible."""
    from pmgb.grid import _classify_segments, _segment_connections, _segment_grid

    hi = 1e3
    g = np.full((8, 8, 8), hi)
    g[1:3, 1:3, :] = -1.0          # tube through the z faces (the end planes coincide)
    g[5:7, 5:7, 3:5] = -1.0        # closed pocket
    g[5:7, 1:3, 0:3] = -1.0        # touches the z = 0 face only
    seg, n = _segment_grid(g, 0.0)
    assert n == 3
    cls = _classify_segments(n, _segment_connections(seg))
    label = lambda p: seg[p] - 1
    assert cls[label((1, 1, 4))] == 1
    assert cls[label((5, 5, 3))] == 0
    assert cls[label((5, 1, 1))] == 0

    # two segments that pass into each other's images: A leaves through +x into B, B leaves
    # through +y into A, so the cycle A -> B -> A ends one cell over in x and y
    g = np.full((6, 6, 6), hi)
    g[3:6, 0:2, 2:4] = -1.0        # A
    g[0:2, 0:6, 2:4] = -1.0        # B: a column along y at x = 0..1 ...
    g[0:6, 5, 2:4] = -1.0          # ... and a row along x on the y = end plane
    seg, n = _segment_grid(g, 0.0)
    assert n == 2
    a, b = seg[4, 0, 2] - 1, seg[0, 3, 2] - 1
    cls = _classify_segments(n, _segment_connections(seg))
    assert cls[a] == 1 and cls[b] == 1
    # without B's row A only bounces back and forth across one face (net translation zero):
    # blocked, as in the reference, although it touches an accessible channel
    g[2:6, 5, 2:4] = hi
    seg, n = _segment_grid(g, 0.0)
    a, b = seg[4, 0, 2] - 1, seg[0, 3, 2] - 1
    cls = _classify_segments(n, _segment_connections(seg))
    assert cls[a] == 0 and cls[b] == 1


def _native():
    lib_path = ROOT / "porousmaterials.jl_gb300" / "pmgb" / "libpmgb.so"
    if not lib_path.exists():
        pytest.skip("libpmgb.so not built")
    return pmgb._lib.lib()


def test_native_replication_factors_match_the_host_mirror(golden):
    """pmgb_replication_factors (host-only, no device work) against the Python restatement of
    src/forcefield.jl:120-158 over the synthetic frameworks, the reference's crystals and skewed
    random cells."""
    L = _native()
    from pmgb import synthetic

    boxes = [cr.box for cr in synthetic.batch_frameworks(24)] + [synthetic.config0().box, synthetic.config1().box]
    boxes += [pmgb.read_cif(DATA / "crystals" / n).box for n in ("SBMOF-1.cif", "NU-1000_Greg.cif", "CAXVII_clean.cif")]
    rng = np.random.default_rng(4)
    for _ in range(40):
        boxes.append(pmgb.Box(*rng.uniform(3.0, 30.0, 3), *np.radians(rng.uniform(65.0, 115.0, 3))))
    for box in boxes:
        for rc in (8.0, 12.5, 14.0):
            f = np.ascontiguousarray(box.f_to_c.T.reshape(-1))
            out = (ctypes.c_int32 * 3)()
            assert L.pmgb_replication_factors(f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), rc, out) == 0
            assert tuple(out) == pmgb.replication_factors(box, rc)
    # the reference's own case (test/forcefield.jl:27-30: Dreiding at its 12.5 A cutoff)
    cr = pmgb.read_cif(DATA / "crystals" / "test_structure.cif")
    out = (ctypes.c_int32 * 3)()
    f = np.ascontiguousarray(cr.box.f_to_c.T.reshape(-1))
    L.pmgb_replication_factors(f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 12.5, out)
    assert list(out) == golden["forcefield_dreiding"]["rep_test_structure"]
    # degenerate input is refused, not looped on
    assert L.pmgb_replication_factors(np.zeros(9).ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 12.5, out) == -1


def test_native_ewald_setup_matches_the_restated_steps():
    """setup_Ewald_sum (through pmgb_ewald_setup) against the Python restatements of its steps
    (determine_ewald_params, required_kreps, precompute_kvec_wts): the same alpha, kreps and
    k-vectors, weights within rounding; the count query and the capacity check."""
    L = _native()
    from pmgb import synthetic

    for cr in [synthetic.config1(), synthetic.config4()] + synthetic.batch_frameworks(8):
        sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, 12.5))
        ep = pmgb.setup_Ewald_sum(sc.box, 12.5, eps=1e-6)
        alpha, k2 = pmgb.determine_ewald_params(12.5, 1e-6)
        kreps = pmgb.required_kreps(sc.box, k2)
        abc, wt = pmgb.precompute_kvec_wts(kreps, sc.box, alpha, k2)
        assert ep.alpha == alpha and tuple(ep.kreps) == tuple(kreps)
        np.testing.assert_array_equal(ep.kvec_abc, abc)
        np.testing.assert_allclose(ep.kvec_wt, wt, rtol=1e-13)
    f = np.ascontiguousarray(sc.box.f_to_c.T.reshape(-1))
    fp = f.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    n = ctypes.c_int64()
    small = np.zeros(3, dtype=np.int32)
    w = np.zeros(1)
    rc = L.pmgb_ewald_setup(fp, 12.5, 1e-6, 1, None, None, None, ctypes.byref(n),
                            small.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == -1 and n.value == ep.n_kvecs    # too small a capacity: refused, count still given
    assert L.pmgb_ewald_setup(fp, 12.5, 0.0, 0, None, None, None, ctypes.byref(n), None, None) == -1


def test_reference_grid_positions_replay_the_grid_loop():
    """reference_grid_positions equals a literal replay of energy_grid's loop (src/grid.jl:331-333)
    with translate_to!'s FP64 steps (src/molecule.jl:147-151,176-179), bit for bit."""
    from pmgb.energy_min import reference_grid_positions

    for n_pts, rep, atom0, com0 in (((4, 3, 5), (2, 1, 3), [0.1234567, 0.7, 0.33], [0.1234567, 0.7, 0.33]),
                                    ((15, 15, 15), (2, 2, 2), [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]),
                                    ((3, 6, 7), (3, 2, 1), [0.31, 0.29, 0.71], [0.3100000000000001, 0.29, 0.7])):
        pts = [[(m / (n - 1.0)) for m in range(n)] for n in n_pts]
        atom, com = np.array(atom0, dtype=float), np.array(com0, dtype=float)
        seen = {}
        for i in range(n_pts[0]):
            for j in range(n_pts[1]):
                for k in range(n_pts[2]):
                    target = np.array([pts[0][i], pts[1][j], pts[2][k]]) / np.array(rep, dtype=float)
                    d = target - com
                    atom = atom + d
                    com = com + d
                    seen[(i, j, k)] = atom.copy()
        ids = list(seen)
        got = reference_grid_positions(n_pts, rep, atom0, com0, ids)
        want = np.array([seen[t] for t in ids])
        assert np.array_equal(got, want)


def test_hilbert_order_of_the_runs():
    """pmgb_hilbert_cell (the host build of the order kernels' hilbert_cell): for 2^3 to 2^6
    cells per axis a bijection onto [0, 8^bits) along which consecutive cells share a face, so
    that runs of consecutive insertions stay compact; out-of-range arguments are refused."""
    L = _native()
    for bits in (3, 4, 5, 6):
        n = 1 << bits
        cells = np.array(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")).reshape(3, -1).T
        codes = np.array([L.pmgb_hilbert_cell(int(x), int(y), int(z), bits) for x, y, z in cells])
        assert codes.min() == 0 and codes.max() == n ** 3 - 1
        order = np.full(n ** 3, -1)
        order[codes] = np.arange(n ** 3)
        assert (order >= 0).all()  # every index taken once
        steps = np.abs(np.diff(cells[order], axis=0)).sum(axis=1)
        assert (steps == 1).all()
    assert L.pmgb_hilbert_cell(8, 0, 0, 3) == -1
    assert L.pmgb_hilbert_cell(0, 0, 0, 0) == -1 and L.pmgb_hilbert_cell(0, 0, 0, 11) == -1
