"""A (replicated crystal, guest molecule, force field, Ewald) system resident on the GPU.

Wraps a `pmgb_system` handle of libpmgb: species names are mapped to dense ids, the
force-field ε / σ² tables are built over those ids, and the guest's LJ sites and charges
are given as Cartesian offsets from its centre of mass.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Context, ptr
from .crystal import Crystal, has_charges
from .ewald import EwaldParams
from .forcefield import LJForceField
from .molecule import Molecule, body_offsets


class GPUSystem:
    def __init__(self, crystal: Crystal, molecule: Molecule, ljff: LJForceField | None,
                 eparams: EwaldParams | None = None, ctx: Context | None = None, refine_tail: float = 0.0):
        """ljff=None builds a charge-only system (all ε = 0, cutoff from eparams); refine_tail > 0
        turns on the FP64 refinement of the Boltzmann tail of Widom runs (set_refine)."""
        self.ctx = ctx or Context.default()
        self.crystal = crystal
        self.molecule = molecule
        self.ljff = ljff
        species = list(dict.fromkeys([*dict.fromkeys(crystal.atoms.species), *molecule.atom_species]))
        self.species = species
        sid = {s: i for i, s in enumerate(species)}
        if ljff is not None:
            eps, sig2 = ljff.tables(species)
            r2_cutoff = ljff.r2_cutoff
        else:
            if eparams is None:
                raise ValueError("a charge-only system needs Ewald parameters")
            eps, sig2 = np.zeros((len(species),) * 2), np.ones((len(species),) * 2)
            r2_cutoff = eparams.sr_cutoff_r ** 2
        self._eps = np.ascontiguousarray(eps)
        self._sig2 = np.ascontiguousarray(sig2)
        atom_xf = np.ascontiguousarray(crystal.atoms.xf, dtype=np.float64)
        atom_sp = np.fromiter(map(sid.__getitem__, crystal.atoms.species), dtype=np.int32,
                              count=len(crystal.atoms.species))
        q_xf = np.ascontiguousarray(crystal.charges.xf, dtype=np.float64)
        q = np.ascontiguousarray(crystal.charges.q, dtype=np.float64)
        box = crystal.box
        f_to_c = np.ascontiguousarray(box.f_to_c.T.reshape(-1))  # column-major
        ax, qx = body_offsets(molecule, box)
        self._gax = np.ascontiguousarray(ax, dtype=np.float64)
        self._gsp = np.ascontiguousarray([sid[s] for s in molecule.atom_species], dtype=np.int32)
        self._gqx = np.ascontiguousarray(qx, dtype=np.float64)
        self._gq = np.ascontiguousarray(molecule.charge_q, dtype=np.float64)
        h = C.c_void_p()
        lib = self.ctx._lib
        self.ctx.check(lib.pmgb_system_create(
            self.ctx.handle, ptr(f_to_c, C.c_double),
            len(atom_sp), ptr(atom_xf, C.c_double), ptr(atom_sp, C.c_int32),
            q.shape[0], ptr(q_xf, C.c_double), ptr(q, C.c_double),
            len(species), ptr(self._eps, C.c_double), ptr(self._sig2, C.c_double), r2_cutoff,
            len(self._gsp), ptr(self._gax, C.c_double), ptr(self._gsp, C.c_int32),
            self._gq.shape[0], ptr(self._gqx, C.c_double), ptr(self._gq, C.c_double),
            C.byref(h)))
        self.handle = h
        self.charged = has_charges(crystal) and molecule.n_charges > 0
        self.n_sites = int(lib.pmgb_system_n_sites(h))
        sa = np.zeros(self.n_sites, dtype=np.int32)
        sc = np.zeros(self.n_sites, dtype=np.int32)
        self.ctx.check(lib.pmgb_system_sites(h, ptr(sa, C.c_int32), ptr(sc, C.c_int32)))
        self.site_atom, self.site_charge = sa, sc
        self.eparams = None
        self.refine_tail = 0.0
        if eparams is not None:
            self.set_ewald(eparams)
        if refine_tail:
            self.set_refine(refine_tail)

    @classmethod
    def _unit_cell_prep(cls, crystal: Crystal, molecule: Molecule, ljff: LJForceField, ewald_precision: float,
                        ctx: Context) -> "GPUSystem":
        """A GPUSystem shell holding the host arrays of pmgb_system_create_unitcell (no handle yet)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.ljff = ljff
        self._unit = crystal
        self._ewald_precision = float(ewald_precision)
        self._guest = molecule
        species = list(dict.fromkeys([*dict.fromkeys(crystal.atoms.species), *molecule.atom_species]))
        self.species = species
        sid = {s_: i for i, s_ in enumerate(species)}
        eps, sig2 = ljff.tables(species)
        self._eps = np.ascontiguousarray(eps)
        self._sig2 = np.ascontiguousarray(sig2)
        self._atom_xf = np.ascontiguousarray(crystal.atoms.xf, dtype=np.float64)
        self._atom_sp = np.fromiter(map(sid.__getitem__, crystal.atoms.species), dtype=np.int32,
                                    count=len(crystal.atoms.species))
        self._q_xf = np.ascontiguousarray(crystal.charges.xf, dtype=np.float64)
        self._q = np.ascontiguousarray(crystal.charges.q, dtype=np.float64)
        self._f_to_c = np.ascontiguousarray(crystal.box.f_to_c.T.reshape(-1))  # column-major
        ax, qx = body_offsets(molecule, crystal.box)
        self._gax = np.ascontiguousarray(ax, dtype=np.float64)
        self._gsp = np.ascontiguousarray([sid[s_] for s_ in molecule.atom_species], dtype=np.int32)
        self._gqx = np.ascontiguousarray(qx, dtype=np.float64)
        self._gq = np.ascontiguousarray(molecule.charge_q, dtype=np.float64)
        self.charged = has_charges(crystal) and molecule.n_charges > 0
        self.refine_tail = 0.0
        return self

    def _unit_cell_done(self, handle, rep) -> None:
        """Take the handle made from the arrays of _unit_cell_prep (which are then released)."""
        lib = self.ctx._lib
        self.handle = handle
        self.repfactors = tuple(int(r) for r in rep)
        for k in ("_atom_xf", "_atom_sp", "_q_xf", "_q", "_f_to_c"):
            del self.__dict__[k]
        self.n_sites = int(lib.pmgb_system_n_sites(handle))
        sa = np.zeros(self.n_sites, dtype=np.int32)
        sc = np.zeros(self.n_sites, dtype=np.int32)
        self.ctx.check(lib.pmgb_system_sites(handle, ptr(sa, C.c_int32), ptr(sc, C.c_int32)))
        self.site_atom, self.site_charge = sa, sc

    @classmethod
    def from_unit_cell(cls, crystal: Crystal, molecule: Molecule, ljff: LJForceField, *,
                       ewald_precision: float = 1e-6, ctx: Context | None = None,
                       refine_tail: float = 0.0) -> "GPUSystem":
        """The system henry_coefficient sets up from a UNIT cell (src/henry.jl:78-97), built natively
        by pmgb_system_create_unitcell: replication for the cutoff, the replicated supercell and, when
        framework and guest are charged, the Ewald parameters at ewald_precision.  The supercell
        `crystal`, the guest in its fractions `molecule` and the `eparams` are built on the host only
        if a caller reads them."""
        self = cls._unit_cell_prep(crystal, molecule, ljff, ewald_precision, ctx or Context.default())
        h = C.c_void_p()
        rep_ = (C.c_int32 * 3)()
        lib = self.ctx._lib
        self.ctx.check(lib.pmgb_system_create_unitcell(
            self.ctx.handle, ptr(self._f_to_c, C.c_double),
            len(self._atom_sp), ptr(self._atom_xf, C.c_double), ptr(self._atom_sp, C.c_int32),
            self._q.shape[0], ptr(self._q_xf, C.c_double), ptr(self._q, C.c_double),
            len(self.species), ptr(self._eps, C.c_double), ptr(self._sig2, C.c_double), float(ljff.r_cutoff),
            len(self._gsp), ptr(self._gax, C.c_double), ptr(self._gsp, C.c_int32),
            self._gq.shape[0], ptr(self._gqx, C.c_double), ptr(self._gq, C.c_double),
            float(ewald_precision), rep_, C.byref(h)))
        self._unit_cell_done(h.value, rep_)
        if refine_tail:
            self.set_refine(refine_tail)
        return self

    @classmethod
    def many_from_unit_cells(cls, crystals: list[Crystal], molecules: list[Molecule], ljff: LJForceField, *,
                             ewald_precision: float = 1e-6, ctx: Context | None = None,
                             n_threads: int = 0) -> list["GPUSystem"]:
        """from_unit_cell for every (crystal, molecule) pair in one native call
        (pmgb_systems_create_unitcell): the host set-up of the systems runs on n_threads host threads
        (0: all) and their device set-up back to back, with two synchronisations in all."""
        ctx = ctx or Context.default()
        shells = [cls._unit_cell_prep(cr, mol, ljff, ewald_precision, ctx) for cr, mol in zip(crystals, molecules)]
        n = len(shells)
        if n == 0:
            return []

        def ptrs(attr, ctype):
            return (C.POINTER(ctype) * n)(*[ptr(getattr(g, attr), ctype) for g in shells])

        def counts(fn):
            return np.ascontiguousarray([fn(g) for g in shells], dtype=np.int32)

        n_atoms = counts(lambda g: len(g._atom_sp))
        n_q = counts(lambda g: g._q.shape[0])
        n_sp = counts(lambda g: len(g.species))
        n_ga = counts(lambda g: len(g._gsp))
        n_gq = counts(lambda g: g._gq.shape[0])
        rep = np.zeros((n, 3), dtype=np.int32)
        handles = (C.c_void_p * n)()
        ctx.check(ctx._lib.pmgb_systems_create_unitcell(
            ctx.handle, n, ptrs("_f_to_c", C.c_double), ptr(n_atoms, C.c_int32), ptrs("_atom_xf", C.c_double),
            ptrs("_atom_sp", C.c_int32), ptr(n_q, C.c_int32), ptrs("_q_xf", C.c_double), ptrs("_q", C.c_double),
            ptr(n_sp, C.c_int32), ptrs("_eps", C.c_double), ptrs("_sig2", C.c_double), float(ljff.r_cutoff),
            ptr(n_ga, C.c_int32), ptrs("_gax", C.c_double), ptrs("_gsp", C.c_int32), ptr(n_gq, C.c_int32),
            ptrs("_gqx", C.c_double), ptrs("_gq", C.c_double), float(ewald_precision), int(n_threads),
            ptr(rep, C.c_int32), handles))
        for g, h, r in zip(shells, handles, rep):
            g._unit_cell_done(h, r)
        return shells

    def __getattr__(self, name):
        # the host-side objects of a system built from its unit cell, made on first use
        if name in ("crystal", "molecule", "eparams") and "_unit" in self.__dict__:
            from .crystal import replicate
            from .ewald import setup_Ewald_sum
            from .molecule import Frac

            sc = replicate(self._unit, self.repfactors)
            self.crystal = sc
            self.molecule = Frac(self._guest, sc.box)
            self.eparams = setup_Ewald_sum(sc.box, self.ljff.r_cutoff, eps=self._ewald_precision) \
                if self.charged else None
            return self.__dict__[name]
        raise AttributeError(name)

    # -- set-up ------------------------------------------------------------------------
    def set_ewald(self, ep: EwaldParams) -> None:
        abc = np.ascontiguousarray(ep.kvec_abc, dtype=np.int32)
        wt = np.ascontiguousarray(ep.kvec_wt, dtype=np.float64)
        self.ctx.check(self.ctx._lib.pmgb_system_set_ewald(self.handle, ep.alpha, ep.sr_cutoff_r, wt.shape[0],
                                                           ptr(abc, C.c_int32), ptr(wt, C.c_double)))
        self.eparams = ep

    def structure_factor(self) -> np.ndarray:
        out = np.zeros((self.eparams.n_kvecs, 2))
        self.ctx.check(self.ctx._lib.pmgb_structure_factor(self.handle, ptr(out, C.c_double)))
        return out[:, 0] + 1j * out[:, 1]

    def info(self) -> dict:
        out = np.zeros(6, dtype=np.int64)
        self.ctx.check(self.ctx._lib.pmgb_system_info(self.handle, ptr(out, C.c_int64)))
        keys = ("n_records", "n_segments", "n_kvecs", "n_kvecs_evaluated", "n_sites", "h2d_bytes")
        info = {k: int(v) for k, v in zip(keys, out)}
        on = C.c_int32()
        self.ctx.check(self.ctx._lib.pmgb_system_centre_image(self.handle, C.byref(on)))
        info["centre_image"] = bool(on.value)  # Widom distances from the pose centre (set_centre_image)
        self.ctx.check(self.ctx._lib.pmgb_system_kspace_mirror(self.handle, C.byref(on)))
        info["kspace_mirror"] = bool(on.value)  # sites 1, 2 mirror images through site 0 (CO2)
        return info

    # -- evaluation ----------------------------------------------------------------------
    def site_coords(self, atom_xf: np.ndarray, charge_xf: np.ndarray | None) -> np.ndarray:
        """Pack per-configuration LJ-site and charge coordinates ((n, n_atoms, 3) and
        (n, n_charges, 3), fractional) into the system's merged site order."""
        atom_xf = np.asarray(atom_xf, dtype=np.float64)
        n = atom_xf.shape[0] if atom_xf.size else (charge_xf.shape[0] if charge_xf is not None else 0)
        out = np.zeros((n, self.n_sites, 3))
        for k in range(self.n_sites):
            a, c = int(self.site_atom[k]), int(self.site_charge[k])
            if a >= 0:
                out[:, k, :] = atom_xf[:, a, :]
                if c >= 0 and charge_xf is not None and not np.allclose(charge_xf[:, c, :], atom_xf[:, a, :],
                                                                        rtol=0, atol=1e-12):
                    raise ValueError("a guest charge that shares an LJ site's body offset was moved apart from it")
            else:
                out[:, k, :] = charge_xf[:, c, :]
        return np.ascontiguousarray(out)

    def energies(self, site_xf: np.ndarray) -> np.ndarray:
        """(n, 3) array of (U_vdw, U_es short-range, U_es long-range) in K."""
        site_xf = np.ascontiguousarray(site_xf, dtype=np.float64).reshape(-1, self.n_sites, 3)
        n = site_xf.shape[0]
        out = np.zeros((n, 3))
        self.ctx.check(self.ctx._lib.pmgb_energies(self.handle, n, ptr(site_xf, C.c_double), ptr(out, C.c_double)))
        return out

    def set_refine(self, tail_fraction: float) -> None:
        """FP64 refinement of the Boltzmann tail of Widom runs (see pmgb_system_set_refine);
        0 switches it off."""
        self.ctx.check(self.ctx._lib.pmgb_system_set_refine(self.handle, float(tail_fraction)))
        self.refine_tail = float(tail_fraction)

    def set_accessibility(self, grid, repfactors) -> None:
        """Gate Widom insertions by a Bool `Grid` over the unit cell (src/henry.jl:225): blocked
        insertions get U = +Inf.  grid=None removes the gate."""
        if grid is None:
            self.ctx.check(self.ctx._lib.pmgb_system_set_accessibility(self.handle, None, None, None))
            return
        data = np.asarray(grid.data, dtype=bool)
        n = np.ascontiguousarray(data.shape, dtype=np.int32)
        r = np.ascontiguousarray(repfactors, dtype=np.int32)
        flat = np.ascontiguousarray(data.transpose(2, 1, 0).reshape(-1).astype(np.uint8))  # i fastest
        self._acc = flat
        self.ctx.check(self.ctx._lib.pmgb_system_set_accessibility(self.handle, ptr(n, C.c_int32), ptr(r, C.c_int32),
                                                                   ptr(flat, C.c_uint8)))

    def set_exact(self, on: bool) -> None:
        """Exact single-configuration energies and grids (pmgb_system_set_exact; default on):
        every energy within 1e-5 relative or 1e-4 K of the FP64 reference.  Off: FP32 only."""
        self.ctx.check(self.ctx._lib.pmgb_system_set_exact(self.handle, int(bool(on))))

    def set_cull(self, on: bool) -> None:
        """Spatially ordered evaluation with cutoff culling (pmgb_system_set_cull; default on)."""
        self.ctx.check(self.ctx._lib.pmgb_system_set_cull(self.handle, int(bool(on))))

    def set_image_lists(self, on) -> None:
        """Image lists in the ordered Widom pass (pmgb_system_set_image_lists): False off, "auto"
        (the default: where the run's insertions are dense enough to pay), True wherever they apply."""
        mode = 1 if on == "auto" else (2 if on else 0)
        self.ctx.check(self.ctx._lib.pmgb_system_set_image_lists(self.handle, mode))

    def image_lists(self, n_insertions: int) -> bool:
        """Whether a Widom run of n_insertions insertions of this system takes image lists
        (pmgb_system_image_lists)."""
        on = C.c_int32(0)
        self.ctx.check(self.ctx._lib.pmgb_system_image_lists(self.handle, int(n_insertions), C.byref(on)))
        return bool(on.value)

    def set_centre_image(self, on: bool) -> None:
        """Centre-image distances for multi-site guests where the cell allows them
        (pmgb_system_set_centre_image; default on)."""
        self.ctx.check(self.ctx._lib.pmgb_system_set_centre_image(self.handle, int(bool(on))))

    def widom_work_counts(self, n_per_block: int, n_blocks: int, seed: int) -> dict:
        """The work the ordered forward Widom pass does (pmgb_widom_work_counts): distances evaluated,
        LJ and real-space pair terms inside their cutoffs."""
        out = np.zeros(3, dtype=np.int64)
        self.ctx.check(self.ctx._lib.pmgb_widom_work_counts(self.handle, int(n_per_block), int(n_blocks), int(seed),
                                                            ptr(out, C.c_int64)))
        return {"distances": int(out[0]), "lj_terms": int(out[1]), "es_terms": int(out[2])}

    def energy_grid_work_counts(self, n_pts, repfactors) -> dict:
        """The work the FP32 energy-grid pass does (pmgb_energy_grid_work_counts)."""
        n = np.ascontiguousarray(n_pts, dtype=np.int32)
        r = np.ascontiguousarray(repfactors, dtype=np.int32)
        out = np.zeros(3, dtype=np.int64)
        self.ctx.check(self.ctx._lib.pmgb_energy_grid_work_counts(self.handle, ptr(n, C.c_int32), ptr(r, C.c_int32),
                                                                  ptr(out, C.c_int64)))
        return {"distances": int(out[0]), "lj_terms": int(out[1]), "es_terms": int(out[2])}

    def refined_count(self) -> int:
        """Insertions the last refined Widom run re-evaluated in FP64."""
        out = C.c_int64()
        self.ctx.check(self.ctx._lib.pmgb_system_refined_count(self.handle, C.byref(out)))
        return out.value

    def widom(self, n_per_block: int, n_blocks: int, seed: int, temperature: float, want_energies: bool = False):
        """Per-block (log Σbf, ⟨U_vdw⟩, ⟨U_es⟩, n_inf) and optionally per-insertion (U_vdw, U_es)."""
        block = np.zeros((n_blocks, 4))
        u = np.zeros((n_blocks * n_per_block, 2)) if want_energies else None
        self.ctx.check(self.ctx._lib.pmgb_widom(self.handle, int(n_per_block), int(n_blocks), int(seed),
                                                float(temperature), ptr(block, C.c_double), ptr(u, C.c_double)))
        return block, u

    def widom_adjoint(self, n_per_block: int, n_blocks: int, seed: int, temperature: float,
                      want_energies: bool = False, want_grad: bool = False):
        """Widom block results plus Σ_i w_i ∂U_i/∂θ (see pmgb_widom_adjoint) as a dict:
        log_scale M, sum_w, sum_w_ues, d_eps / d_sig2 (n_species x n_species over self.species,
        row = guest species, column = framework species); optional per-insertion energies and
        dU/dx_COM."""
        ns = len(self.species)
        block = np.zeros((n_blocks, 4))
        dth = np.zeros(3 + 2 * ns * ns)
        u = np.zeros((n_blocks * n_per_block, 2)) if want_energies else None
        g = np.zeros((n_blocks * n_per_block, 3), dtype=np.float32) if want_grad else None
        self.ctx.check(self.ctx._lib.pmgb_widom_adjoint(self.handle, int(n_per_block), int(n_blocks), int(seed),
                                                        float(temperature), ptr(block, C.c_double),
                                                        ptr(dth, C.c_double), ptr(u, C.c_double), ptr(g, C.c_float)))
        pair = dth[3:].reshape(ns, ns, 2)
        return block, {"log_scale": dth[0], "sum_w": dth[1], "sum_w_ues": dth[2], "d_eps": pair[:, :, 0].copy(),
                       "d_sig2": pair[:, :, 1].copy(), "u": u, "grad": g}

    def move_evaluator(self, max_conf: int = 1) -> "MoveEvaluator":
        """A low-latency evaluator of up to max_conf configurations per call (pmgb_move_*)."""
        return MoveEvaluator(self, max_conf)

    def energies_grad(self, site_xf: np.ndarray):
        """((n, 3) energies as in energies(), (n, 3) dU/dx of the rigid configuration, K/Å)."""
        site_xf = np.ascontiguousarray(site_xf, dtype=np.float64).reshape(-1, self.n_sites, 3)
        n = site_xf.shape[0]
        out = np.zeros((n, 3))
        g = np.zeros((n, 3), dtype=np.float32)
        self.ctx.check(self.ctx._lib.pmgb_energies_grad(self.handle, n, ptr(site_xf, C.c_double), ptr(out, C.c_double),
                                                        ptr(g, C.c_float)))
        return out, g

    def energy_grid_adjoint(self, n_pts, repfactors, unit_factor: float, temperature: float):
        n = np.ascontiguousarray(n_pts, dtype=np.int32)
        r = np.ascontiguousarray(repfactors, dtype=np.int32)
        total = int(np.prod(n))
        out = np.zeros(total, dtype=np.float32)
        g = np.zeros((total, 3), dtype=np.float32)
        ns = len(self.species)
        dth = np.zeros(3 + 2 * ns * ns)
        self.ctx.check(self.ctx._lib.pmgb_energy_grid_adjoint(self.handle, ptr(n, C.c_int32), ptr(r, C.c_int32),
                                                              float(unit_factor), float(temperature),
                                                              ptr(out, C.c_float), ptr(g, C.c_float),
                                                              ptr(dth, C.c_double)))
        shape = tuple(int(v) for v in n[::-1])
        data = out.reshape(shape).transpose(2, 1, 0)
        grad = g.reshape(shape + (3,)).transpose(2, 1, 0, 3)
        pair = dth[3:].reshape(ns, ns, 2)
        return data, grad, {"log_scale": dth[0], "sum_w": dth[1], "d_eps": pair[:, :, 0].copy(),
                            "d_sig2": pair[:, :, 1].copy()}

    def energy_grid(self, n_pts, repfactors, unit_factor: float) -> np.ndarray:
        n = np.ascontiguousarray(n_pts, dtype=np.int32)
        r = np.ascontiguousarray(repfactors, dtype=np.int32)
        out = np.zeros(int(np.prod(n)), dtype=np.float32)
        self.ctx.check(self.ctx._lib.pmgb_energy_grid(self.handle, ptr(n, C.c_int32), ptr(r, C.c_int32),
                                                      float(unit_factor), ptr(out, C.c_float)))
        return out.reshape(tuple(int(v) for v in n[::-1])).transpose(2, 1, 0)  # data[i, j, k], i fastest

    def energy_grid_rotational(self, n_pts, repfactors, n_rotations: int, temperature: float, seed: int,
                               unit_factor: float) -> np.ndarray:
        """-T log⟨e^{-U/T}⟩ over n_rotations orientations at each grid point (pmgb_energy_grid_rotational)."""
        n = np.ascontiguousarray(n_pts, dtype=np.int32)
        r = np.ascontiguousarray(repfactors, dtype=np.int32)
        out = np.zeros(int(np.prod(n)), dtype=np.float32)
        self.ctx.check(self.ctx._lib.pmgb_energy_grid_rotational(
            self.handle, ptr(n, C.c_int32), ptr(r, C.c_int32), int(n_rotations), float(temperature), int(seed),
            float(unit_factor), ptr(out, C.c_float)))
        return out.reshape(tuple(int(v) for v in n[::-1])).transpose(2, 1, 0)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.ctx._lib.pmgb_system_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MoveEvaluator:
    """Guest-host energies of a few configurations per call through a captured CUDA graph: the
    per-move energy of a Monte Carlo simulation (src/gcmc.jl:111-124).  energies() takes and
    returns what GPUSystem.energies does."""

    def __init__(self, system: GPUSystem, max_conf: int = 1):
        self.system = system
        self.max_conf = int(max_conf)
        h = C.c_void_p()
        system.ctx.check(system.ctx._lib.pmgb_move_create(system.handle, self.max_conf, C.byref(h)))
        self.handle = h.value
        self._out = np.zeros((self.max_conf, 3))

    def energies(self, site_xf: np.ndarray) -> np.ndarray:
        site_xf = np.ascontiguousarray(site_xf, dtype=np.float64).reshape(-1, self.system.n_sites, 3)
        n = site_xf.shape[0]
        self.system.ctx.check(self.system.ctx._lib.pmgb_move_energies(self.handle, n, ptr(site_xf, C.c_double),
                                                                      ptr(self._out, C.c_double)))
        return self._out[:n].copy()

    def close(self):
        if getattr(self, "handle", None):
            self.system.ctx._lib.pmgb_move_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
