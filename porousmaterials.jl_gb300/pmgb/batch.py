"""Batched Widom screening: many (framework, guest) systems in one persistent launch.

The reference computes one Henry coefficient per henry_coefficient call
(src/henry.jl:34-181); screening a set of frameworks is a loop over those calls.  Here the
systems of a screen are evaluated together by one graph-captured kernel launch whose CTAs
pull insertion units from a work queue, largest frameworks first, so that frameworks of a
few hundred atoms and of a hundred thousand share the GPU without idle SMs.  Every system
sees exactly the insertions and energies pmgb_widom would give it with the seed
`system_seed(seed, s)`; with the adjoint, the parameter derivatives of
henry_coefficient_gradient come out of the same launch.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._lib import Context, ptr
from .crystal import Crystal, has_charges, replicate
from .ewald import setup_Ewald_sum
from .forcefield import LJForceField, replication_factors
from .molecule import Frac, Molecule
from .system import GPUSystem

_GOLDEN = 0x9E3779B97F4A7C15
ORDER_COST = 0      # units by estimated cost, largest first
ORDER_SYSTEM = 1    # units system by system


def system_seed(seed: int, s: int) -> int:
    """Philox key of system s in a batch run with `seed` (seed + s * 0x9E3779B97F4A7C15 mod 2^64)."""
    return (int(seed) + int(s) * _GOLDEN) % (1 << 64)


class BatchScreen:
    """pmgb_batch handle over a list of GPUSystems (kept alive by this object)."""

    def __init__(self, systems: list[GPUSystem], n_per_block, n_blocks: int = 5, with_adjoint: bool = False,
                 ctx: Context | None = None, refine_tail: float = 0.0, cull: bool = True):
        if not systems:
            raise ValueError("BatchScreen needs at least one system")
        self.ctx = ctx or systems[0].ctx
        self.systems = list(systems)
        npb = np.broadcast_to(np.asarray(n_per_block, dtype=np.int64), (len(systems),))
        self.n_per_block = np.ascontiguousarray(npb)
        self.n_blocks = int(n_blocks)
        self.with_adjoint = bool(with_adjoint)
        handles = (C.c_void_p * len(systems))(*[s.handle for s in systems])
        h = C.c_void_p()
        self.ctx.check(self.ctx._lib.pmgb_batch_create(self.ctx.handle, len(systems), handles,
                                                       self.n_per_block.ctypes.data_as(C.POINTER(C.c_int64)),
                                                       self.n_blocks, int(self.with_adjoint), C.byref(h)))
        self.handle = h.value
        self._n_species = [len(s.species) for s in systems]
        self.refine_tail = 0.0
        self.cull = True  # the library's default
        if refine_tail:
            self.set_refine(refine_tail)
        if not cull:
            self.set_cull(False)

    def set_refine(self, tail_fraction: float) -> None:
        """FP64 refinement of the Boltzmann tail of every system (see pmgb_batch_set_refine)."""
        self.ctx.check(self.ctx._lib.pmgb_batch_set_refine(self.handle, float(tail_fraction)))
        self.refine_tail = float(tail_fraction)

    def set_cull(self, on: bool) -> None:
        """Spatially ordered processing with cutoff culling (see pmgb_batch_set_cull)."""
        self.ctx.check(self.ctx._lib.pmgb_batch_set_cull(self.handle, int(bool(on))))
        self.cull = bool(on)

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._lib.pmgb_batch_destroy(self.handle)
            self.handle = None

    __del__ = close

    def info(self) -> dict:
        out = (C.c_int64 * 8)()
        self.ctx.check(self.ctx._lib.pmgb_batch_info(self.handle, out))
        return {"n_units": out[0], "n_ctas": out[1], "order": out[2], "dtheta_len": out[3],
                "device_bytes": out[4], "insertions_per_run": out[5], "n_chunks": out[6], "unit_mflop": out[7]}

    def configure(self, n_ctas: int = 0, order: int = ORDER_COST, unit_mflop: float = 0.0):
        """Launch shape (see pmgb_batch_configure); re-captures the graph."""
        self.ctx.check(self.ctx._lib.pmgb_batch_configure(self.handle, int(n_ctas), int(order), float(unit_mflop)))

    def tune(self, seed: int, temperature: float, repeats: int = 3) -> float:
        """Time every candidate launch shape and keep the fastest; returns its ms per run."""
        ms = C.c_double()
        self.ctx.check(self.ctx._lib.pmgb_batch_tune(self.handle, int(seed) % (1 << 64), float(temperature),
                                                     int(repeats), C.byref(ms)))
        return ms.value

    def refined_counts(self) -> np.ndarray:
        """Insertions of each system the last run re-evaluated in FP64."""
        out = np.zeros(len(self.systems), dtype=np.int64)
        self.ctx.check(self.ctx._lib.pmgb_batch_refined_counts(self.handle, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def energies(self) -> list[np.ndarray]:
        """Per-insertion (U_vdw, U_es) of the last run, one [n_blocks * n_per_block, 2] array per
        system in index order, refined insertions with their FP64 energies (pmgb_batch_energies:
        needs culling or refinement on)."""
        total = int(self.info()["insertions_per_run"])
        u = np.zeros((total, 2))
        self.ctx.check(self.ctx._lib.pmgb_batch_energies(self.handle, ptr(u, C.c_double)))
        out, o = [], 0
        for npb in self.n_per_block:
            n = int(npb) * self.n_blocks
            out.append(u[o:o + n].copy())
            o += n
        return out

    def launch(self, seed: int, temperature: float):
        """Enqueue one run on the context stream (asynchronous)."""
        self.ctx.check(self.ctx._lib.pmgb_batch_launch(self.handle, int(seed) % (1 << 64), float(temperature)))

    def results(self):
        """(blocks [n_systems, n_blocks, 4] as GPUSystem.widom's, list of adjoint dicts or None)."""
        n = len(self.systems)
        blocks = np.zeros((n, self.n_blocks, 4))
        dth = np.zeros(sum(3 + 2 * k * k for k in self._n_species)) if self.with_adjoint else None
        self.ctx.check(self.ctx._lib.pmgb_batch_results(self.handle, ptr(blocks, C.c_double), ptr(dth, C.c_double)))
        if not self.with_adjoint:
            return blocks, None
        adj, o = [], 0
        for k in self._n_species:
            d = dth[o:o + 3 + 2 * k * k]
            pair = d[3:].reshape(k, k, 2)
            adj.append({"log_scale": d[0], "sum_w": d[1], "sum_w_ues": d[2], "d_eps": pair[:, :, 0].copy(),
                        "d_sig2": pair[:, :, 1].copy()})
            o += 3 + 2 * k * k
        return blocks, adj

    def run(self, seed: int, temperature: float):
        self.launch(seed, temperature)
        return self.results()


def build_systems(crystals: list[Crystal], molecule: Molecule | list[Molecule], ljff: LJForceField, *,
                  ewald_precision: float = 1e-6, ctx: Context | None = None, n_threads: int = 0) -> list[GPUSystem]:
    """One GPUSystem per crystal (replicated for the cutoff, Ewald set up when both are charged),
    all built in one native call (pmgb_systems_create_unitcell: host set-up on n_threads threads,
    0 = all; device set-up back to back)."""
    ctx = ctx or Context.default()
    mols = list(molecule) if isinstance(molecule, (list, tuple)) else [molecule] * len(crystals)
    return GPUSystem.many_from_unit_cells(list(crystals), mols, ljff, ewald_precision=ewald_precision, ctx=ctx,
                                          n_threads=n_threads)


def henry_coefficient_screen(crystals: list[Crystal], molecule: Molecule | list[Molecule], temperature: float,
                             ljforcefield: LJForceField, *, insertions: int = 20000, n_blocks: int = 5,
                             seed: int = 0, with_gradient: bool = True, ewald_precision: float = 1e-6,
                             tune: bool = True, systems: list[GPUSystem] | None = None,
                             refine_tail: float = 1e-3) -> list[dict]:
    """K_H (mol/(m³ bar), block mean as henry_coefficient) of every crystal, and with_gradient the
    derivatives of henry_coefficient_gradient, from one batched run."""
    from .adjoint import henry_gradients
    from .henry import UNIV_GAS_CONST

    temperature = float(temperature)
    if systems is None:
        systems = build_systems(crystals, molecule, ljforcefield, ewald_precision=ewald_precision)
    npb = max(1, math.ceil(insertions / n_blocks))
    screen = BatchScreen(systems, npb, n_blocks, with_adjoint=with_gradient, refine_tail=refine_tail)
    if tune:
        screen.tune(seed + 1, temperature)
    blocks, adj = screen.run(seed, temperature)
    out = []
    for s, gs in enumerate(systems):
        kh = np.exp(blocks[s, :, 0] - math.log(UNIV_GAS_CONST * temperature * npb))
        r = {"henry coefficient [mol/(m³-bar)]": float(np.mean(kh)), "blocks": blocks[s],
             "seed": system_seed(seed, s), "n_insertions_per_block": npb}
        if with_gradient:
            d_eps, d_sig, d_lam = henry_gradients(gs, blocks[s], adj[s], temperature, npb)
            r.update({"dKH/d epsilon": d_eps, "dKH/d sigma": d_sig,
                      "dKH/d charge scale": d_lam if gs.charged else 0.0})
        out.append(r)
    screen.close()
    return out
