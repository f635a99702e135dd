#!/usr/bin/env python3
"""Widom-insertion throughput on GB300 (one JSON line on rank 0).

Workload (default): plain Widom K_H with Ewald -- rigid 3-site CO2 in a 600-atom triclinic
cell (13.2 / 18.9 / 9.8 Å, β = 102°, Zn:O:C:H = 32:104:192:96, N(0, 0.4) neutralised
charges) replicated 2x2x3 (7,200 framework sites), 12.5 Å cutoff, Ewald precision 1e-6
(α = 0.24713 / Å, 1,424 k-vectors), 1e6 insertions in 5 blocks at 298 K, seeded synthetic
inputs.  A step is one Widom pass over the 1e6 insertions.

  value : insertions/s of pmgb_widom_device on the resident system with the FP64 refinement
          of the Boltzmann tail (K_H within 1e-6 of FP64), CUDA events on the launching
          stream, L2 flushed before every timed step; the FP32 pass alone is timed too
          (precision.fp32_only_*) and gives the roofline's kernel time
  e2e   : insertions/s of pmgb.henry_coefficient(...) -- the reference-facing call: host
          set-up, host->device copies, S(k), the Widom launch and the device->host read
  --impl reference : the reference's algorithm on the host cores (the FP64 oracle port:
          direct e^{ik.r} Ewald sum, OpenMP over insertions), bounded samples.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "porousmaterials.jl_gb300"))

METRIC = "Widom insertions/s (+grad) on 1 GB300, batched vs plain, at ≤1e-6 rel KH error"
UNIT = "insertions/s"
T = 298.0
N_BLOCKS = 5
N_INS = 1_000_000
# algorithmic flops, fixed counting convention (FMA = 2, MUFU = 1, erfc = 10): every pair counted,
# LJ 28 and real-space Coulomb 40; a reciprocal-space term 17 per (k-vector, guest charge)
F_LJ, F_COUL, F_K = 28, 40, 17
# the same work counted by what the cutoff keeps: the distance of every pair 26; inside the
# cutoff the LJ terms 11 and the real-space terms 30 more
F_DIST, F_LJ_IN, F_ES_IN = 26, 11, 30
# with image lists a distance is an offset from the warp's list: 3 subtractions and r^2 (5); the
# list building (once per warp and image) and the close-pair residual terms are not counted
F_DIST_IMG = 8
# the reciprocal-space loop as the kernels execute it, per evaluated k-vector and guest: 16 flops
# (site 0's phase step and the structure-factor product) and 12 per further guest charge (its
# phase-difference step and the charge sum); 21 in all for mirror-image sites (CO2,
# pmgb_system_kspace_mirror), which step one phase difference and take a real charge sum
F_KROW, F_KROW_SITE, F_KROW_MIRROR = 16, 12, 21
REFINE_TAIL = 1e-3
# DRAM traffic of the config1 image-list pair kernel, from ncu (dram bytes of one launch over 5e5
# insertions: 2.19 MB; profiles/pairs_img_kernel_config1.md), per insertion; a full launch scales
# with the insertions it processes
PAIR_DRAM_BYTES_PER_INSERTION = 2.19e6 / 5e5
# kernels per Widom step: the run's spatial order (count, scan, scatter, per-cell sort), pairs,
# insertion-order partials, block reduction, and the refinement's hist, cut, count, scan, scatter,
# FP64 energies (thread pass, plan, warp pass), and the store, chunk re-form and block
# recombination of the results
LAUNCHES_PER_STEP = 18


ALL_LEGS = ("adjoint", "e2e", "porous", "batched", "config4", "moves", "config2", "cpu")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--insertions", type=int, default=N_INS)
    p.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline leg (profiling runs)")
    p.add_argument("--skip-e2e", action="store_true", help="omit the end-to-end leg (profiling runs)")
    p.add_argument("--batch-frameworks", type=int, default=512,
                   help="frameworks in the batched-screening leg (each with CH4 and CO2; 0 = skip)")
    p.add_argument("--batch-insertions", type=int, default=20000, help="insertions per (framework, guest)")
    p.add_argument("--c4-insertions", type=int, default=10_000_000, help="insertions of the large-cell leg")
    p.add_argument("--skip-configs", action="store_true", help="omit the large-cell and energy-grid legs")
    p.add_argument("--image-lists", default="auto", choices=["auto", "on", "off"],
                   help="image lists in the config1 workload's ordered Widom pass (pmgb_system_set_image_lists)")
    p.add_argument("--legs", default="all",
                   help="comma list of the legs beside the config1 workload to run: " + ",".join(ALL_LEGS) +
                        " (default all; the skip flags remove legs from it)")
    args = p.parse_args()
    legs = set(ALL_LEGS) if args.legs == "all" else {x.strip() for x in args.legs.split(",") if x.strip()}
    unknown = legs - set(ALL_LEGS)
    if unknown:
        p.error(f"unknown legs {sorted(unknown)}")
    if args.skip_cpu:
        legs.discard("cpu")
    if args.skip_e2e:
        legs -= {"e2e", "adjoint"}
    if args.skip_configs:
        legs -= {"porous", "config4", "config2", "moves"}
    if args.batch_frameworks <= 0:
        legs.discard("batched")
    args.legs = legs
    return args


def workload():
    import pmgb
    from pmgb import synthetic

    cr = synthetic.config1()
    ff = synthetic.forcefield(12.5)
    rep = pmgb.replication_factors(cr.box, ff)
    sc = pmgb.replicate(cr, rep)
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    return cr, sc, ff, ep, synthetic.co2(), rep


def flops_per_insertion(sc, mol, ep):
    """Algorithmic FP32 flops of one insertion under the fixed convention: every (framework, guest)
    LJ pair 28, every real-space charge pair 40, every (k-vector, guest charge) term 17."""
    n_lj = mol.n_atoms * sc.atoms.n
    n_q = mol.n_charges * sc.charges.n
    f = F_LJ * n_lj
    if ep is not None and mol.n_charges:
        f += F_COUL * n_q + F_K * mol.n_charges * ep.n_kvecs
    return f


def counted_flops(counts: dict, n_items: int, n_q_sites: int = 0, n_kvecs: int = 0, image_lists: bool = False,
                  mirror: bool = False) -> float:
    """Algorithmic FP32 flops per item of the work a pass did (pmgb_*_work_counts): 26 per
    (guest site, record) distance evaluated (8 per (guest site, list image) distance with image
    lists), 11 more per LJ term and 30 per real-space term inside their cutoffs; per evaluated
    k-vector 16 + 12 (n_q_sites - 1), or 21 with mirror-image sites."""
    fd = F_DIST_IMG if image_lists else F_DIST
    fk = 0 if n_q_sites == 0 else (F_KROW_MIRROR if mirror else F_KROW + F_KROW_SITE * (n_q_sites - 1))
    return (fd * counts["distances"] + F_LJ_IN * counts["lj_terms"] + F_ES_IN * counts["es_terms"]) / n_items + \
        fk * n_kvecs


def flops_inside_cutoff(sc, mol, ff, ep, n_kvecs=None):
    """Algorithmic FP32 flops of one insertion (FMA = 2, MUFU = 1): the minimum-image distance
    of every (framework record, guest site) pair; the LJ and real-space terms of the pairs inside
    their cutoffs -- a uniform insertion has n (4/3) pi rc^3 / V framework sites inside rc on
    average (minimum image, rc at most half the smallest width); reciprocal-space terms of the
    n_kvecs k-vectors evaluated (S(k) vanishes on the others when the cell is a replica)."""
    import numpy as np

    sph = lambda r: 4.0 / 3.0 * math.pi * r ** 3 / sc.box.Omega
    n_rec = len({tuple(np.round(np.mod(x, 1.0), 12)) for x in np.vstack([sc.atoms.xf, sc.charges.xf])}) \
        if sc.charges.n else sc.atoms.n
    sites = max(mol.n_atoms, mol.n_charges)
    f = F_DIST * sites * n_rec + F_LJ_IN * mol.n_atoms * sc.atoms.n * sph(ff.r_cutoff)
    if ep is not None and mol.n_charges:
        f += F_ES_IN * mol.n_charges * sc.charges.n * sph(ep.sr_cutoff_r) + \
            F_K * mol.n_charges * (ep.n_kvecs if n_kvecs is None else n_kvecs)
    return f


# ------------------------------------------------------------------ clocks sampling
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines: list[str] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
            return self
        # nvidia-smi takes a moment to start: wait (bounded) for its first sample, then keep only the
        # samples taken from here on, i.e. during the timed region
        t_end = time.perf_counter() + 5.0
        while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
            time.sleep(0.01)
        self.lines.clear()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = sorted(r[0] for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[2]) if v.lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------------ CPU legs
def oracle_module():
    """The FP64 oracle's Python binding (oracle/oracle.py).  Its folder goes first on the path
    before the first import: with the repository root alone on the path, `import oracle` would
    find the oracle/ folder itself as an empty namespace package."""
    p = str(ROOT / "oracle")
    if p not in sys.path:
        sys.path.insert(0, p)
    mod = sys.modules.get("oracle")
    if mod is not None and not hasattr(mod, "OracleSystem"):
        del sys.modules["oracle"]
    import importlib

    return importlib.import_module("oracle")


def oracle_system(sc, mol, ff, ep):
    """The FP64 oracle (the reference's algorithm restated in C) holding a workload's inputs."""
    oracle = oracle_module()

    species = list(dict.fromkeys(list(sc.atoms.species) + list(mol.atom_species)))
    sid = {s: i for i, s in enumerate(species)}
    eps, sig2 = ff.tables(species)
    o = oracle.OracleSystem(sc.box.f_to_c, sc.atoms.xf, [sid[s] for s in sc.atoms.species], sc.charges.xf,
                            sc.charges.q, eps, sig2, ff.r2_cutoff, [sid[s] for s in mol.atom_species], mol.charge_q)
    if ep is not None:
        o.set_ewald(ep.alpha, ep.sr_cutoff_r, ep.kreps, ep.kvec_abc, ep.kvec_wt)
    return o


def cpu_rate(sc, mol, ep, budget_s: float, seed: int = 99, nthreads: int = 0, use_sk: bool = False, ff=None):
    """Insertions/s of the FP64 oracle (direct e^{ik.r} form unless use_sk, all host threads or
    nthreads) on a bounded sample of the workload's insertions (random poses)."""
    import numpy as np

    oracle = oracle_module()
    from pmgb import synthetic
    from pmgb.molecule import body_offsets

    o = oracle_system(sc, mol, ff or synthetic.forcefield(12.5), ep)
    charged = ep is not None and mol.n_charges > 0
    cores = nthreads if nthreads > 0 else oracle.num_threads()
    rng = np.random.default_rng(seed)
    ax, qx = body_offsets(mol, sc.box)

    def run(n):
        xf = rng.random((n, 3))
        R = np.stack([_rot(rng) for _ in range(n)])
        lj = xf[:, None, :] + np.einsum("ij,njk,lk->nli", sc.box.c_to_f, R, ax)
        q = xf[:, None, :] + np.einsum("ij,njk,lk->nli", sc.box.c_to_f, R, qx) if charged else None
        t0 = time.perf_counter()
        o.energies(lj, q, charged=charged, use_sk=use_sk, nthreads=nthreads)
        return time.perf_counter() - t0

    # calibrate on a few insertions per thread, then sample until the time budget is spent
    per = run(4 * cores) / (4 * cores)
    total_n, total_t = 0, 0.0
    while total_t < 0.9 * budget_s:
        n = max(2 * cores, int((budget_s - total_t) / max(per, 1e-9)))
        dt = run(n)
        total_n += n
        total_t += dt
        per = total_t / total_n
    return total_n / total_t, cores, total_n, total_t


def cpu_legs(sc, mol, ep, ff):
    """The reference's algorithm on the host cores (the FP64 oracle port), beside the GPU:
    config1 (the workload) with the direct e^{ik.r} Ewald form on all threads and on one, and with
    the structure-factor form (the same algorithm the GPU runs, so the two config1 rates split the
    speed-up into algorithm and hardware); config0 in full (1e5 CH4 insertions), config2 in full
    (the 96^3 Xe grid) and a bounded sample of config4 (direct form)."""
    import numpy as np

    oracle = oracle_module()
    import pmgb
    from pmgb import synthetic

    r, cores, n, dt = cpu_rate(sc, mol, ep, budget_s=15.0)
    r1, _, n1, dt1 = cpu_rate(sc, mol, ep, budget_s=4.0, seed=98, nthreads=1)
    rsk, _, nsk, dtsk = cpu_rate(sc, mol, ep, budget_s=5.0, seed=97, use_sk=True)
    out = {"value": r, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{n} insertions of the workload (random poses), FP64 direct e^(ik.r) Ewald sum + LJ "
                     f"(the reference's algorithm), OpenMP over insertions, {dt:.1f} s",
           "single_core": {"value": r1, "unit": UNIT, "cores": 1,
                           "sample": f"{n1} insertions on one thread, {dt1:.1f} s"},
           "sk_form": {"value": rsk, "unit": UNIT, "cores": cores,
                       "sample": f"{nsk} insertions, FP64 structure-factor form of the reciprocal space (every "
                                 f"k-vector, S(k) precomputed) + LJ + real space, {dtsk:.1f} s"}}
    # config0 in full: CH4 (one LJ bead) in the 424-atom cubic cell, 1e5 insertions
    c0 = synthetic.config0()
    rep0 = pmgb.replication_factors(c0.box, ff)
    sc0 = pmgb.replicate(c0, rep0)
    ch4 = synthetic.ch4()
    o0 = oracle_system(sc0, ch4, ff, None)
    rng = np.random.default_rng(11)
    xf = rng.random((100_000, 1, 3))
    t0 = time.perf_counter()
    o0.energies(xf)
    t_c0 = time.perf_counter() - t0
    out["config0_full"] = {"value": 1e5 / t_c0, "unit": UNIT, "cores": cores,
                           "sample": f"all 1e5 insertions of config0 (CH4, 424 atoms, LJ), FP64, {t_c0:.2f} s"}
    # config2 in full: Xe over the 96^3 grid of config0
    ox = oracle_system(sc0, synthetic.xe(), ff, None)
    t0 = time.perf_counter()
    ox.energy_grid((96, 96, 96), rep0)
    t_c2 = time.perf_counter() - t0
    out["config2_full"] = {"value": 96 ** 3 / t_c2, "unit": "grid points/s", "cores": cores,
                           "sample": f"the full 96^3 grid of config2 (Xe in config0), FP64, {t_c2:.2f} s"}
    # config4: a bounded sample with the direct form
    c4 = synthetic.config4()
    sc4 = pmgb.replicate(c4, pmgb.replication_factors(c4.box, ff))
    ep4 = pmgb.setup_Ewald_sum(sc4.box, ff.r_cutoff, eps=1e-6)
    r4, _, n4, dt4 = cpu_rate(sc4, mol, ep4, budget_s=10.0, seed=96, ff=ff)
    out["config4_sample"] = {"value": r4, "unit": UNIT, "cores": cores,
                             "sample": f"{n4} insertions of config4 (CO2, 20,000 atoms, 6,974 k-vectors), FP64 direct "
                                       f"e^(ik.r) form, {dt4:.1f} s"}
    del oracle
    return out


def _rot(rng):
    import pmgb

    return pmgb.random_rotation_matrix(rng)


def reference_arm(args, rank, world):
    if rank != 0:
        return
    cr, sc, ff, ep, mol, rep = workload()
    for _ in range(args.warmup):
        cpu_rate(sc, mol, ep, budget_s=1.0)
    rates, times, ns = [], [], []
    for s in range(args.steps):
        r, cores, n, dt = cpu_rate(sc, mol, ep, budget_s=8.0, seed=1000 + s)
        rates.append(r)
        times.append(dt)
        ns.append(n)
    value = sum(ns) / sum(times)
    sample = (f"{sum(ns)} insertions of the workload (random poses) over {args.steps} steps; FP64 direct "
              f"e^(ik.r) Ewald sum + LJ, OpenMP over insertions")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "widom_co2_ewald_600atom_triclinic_2x2x3_1e6", "insertions_per_step": None,
                      "cpu_sample": True},
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ batched screening leg
def batched_leg(args, ctx, stream, peak=None):
    """Batched vs plain forward + adjoint Widom over uneven synthetic frameworks.

    Frameworks: atoms log-uniform 50-5000, cell lengths U(8, 40) Å, angles U(80, 110)°,
    neutralised N(0, 0.4) charges, replicated for the 12.5 Å cutoff; each with CH4 (LJ) and
    CO2 (LJ + Ewald 1e-6); args.batch_insertions insertions per system in 5 blocks.
      plain   : GPUSystem.widom_adjoint per system, one after another (each call returns its
                results to the host, as henry_coefficient_gradient does per framework)
      batched : BatchScreen.run -- one graph replay of the persistent kernel + per-system
                reduction, then the results copy (the same outputs for every system)
    Systems are built once, outside both timings."""
    import numpy as np
    import torch

    from pmgb import synthetic
    from pmgb.batch import BatchScreen, build_systems, system_seed

    t0 = time.perf_counter()
    fws = synthetic.batch_frameworks(args.batch_frameworks)
    t_gen = time.perf_counter() - t0
    ff = synthetic.forcefield(12.5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    systems = build_systems(fws, synthetic.ch4(), ff, ctx=ctx) + build_systems(fws, synthetic.co2(), ff, ctx=ctx)
    for gs in systems:
        gs.set_refine(REFINE_TAIL)  # as the drop-in calls: K_H within 1e-6 of FP64
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    npb = max(1, args.batch_insertions // N_BLOCKS)
    n_ins = npb * N_BLOCKS * len(systems)
    sizes = np.array([gs.info()["n_records"] for gs in systems[:len(fws)]])

    def plain(adjoint):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for s, gs in enumerate(systems):
            if adjoint:
                gs.widom_adjoint(npb, N_BLOCKS, 900 + s, T)
            else:
                gs.widom(npb, N_BLOCKS, 900 + s, T)
        return time.perf_counter() - t

    def dropin(adjoint):
        """The drop-in call per (framework, guest), set-up included, as a screening loop over
        henry_coefficient / henry_coefficient_gradient would run it."""
        import pmgb

        torch.cuda.synchronize()
        t = time.perf_counter()
        s = 0
        for mol in (synthetic.ch4(), synthetic.co2()):
            for cr in fws:
                ipv = npb * N_BLOCKS / cr.box.Omega
                if adjoint:
                    pmgb.henry_coefficient_gradient(cr, mol, T, ff, insertions_per_volume=ipv, seed=700 + s)
                else:
                    pmgb.henry_coefficient(cr, mol, T, ff, insertions_per_volume=ipv, seed=700 + s, verbose=False,
                                           autosave=False)
                s += 1
        return time.perf_counter() - t

    out = {}
    for adjoint in (False, True):
        t_dropin = dropin(adjoint)
        plain(adjoint)  # warm-up: per-system scratch allocations
        t_plain = min(plain(adjoint) for _ in range(2))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        screen = BatchScreen(systems, npb, N_BLOCKS, with_adjoint=adjoint, ctx=ctx, refine_tail=REFINE_TAIL)
        torch.cuda.synchronize()
        t_create = time.perf_counter() - t0
        tuned_ms = screen.tune(1, T, repeats=2)
        info = screen.info()
        for w in range(args.warmup):
            screen.run(2 + w, T)
        k = max(3, args.steps // 2)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        torch.cuda.synchronize()
        t = time.perf_counter()
        for i in range(k):
            ev[i][0].record(stream)
            screen.launch(100 + i, T)
            ev[i][1].record(stream)
            screen.results()
        t_batched = (time.perf_counter() - t) / k
        ms_dev = sum(a.elapsed_time(b) for a, b in ev) / k
        refined = int(screen.refined_counts().sum())
        screen.close()
        key = "forward_plus_adjoint" if adjoint else "forward"
        out[key] = {"plain_dropin_insertions_per_s": n_ins / t_dropin, "plain_dropin_s": t_dropin,
                    "speedup_vs_plain_dropin": t_dropin / t_batched,
                    "plain_insertions_per_s": n_ins / t_plain, "plain_s": t_plain,
                    "batched_insertions_per_s": n_ins / t_batched, "batched_s": t_batched,
                    "batched_device_ms": ms_dev, "batched_device_insertions_per_s": n_ins / (ms_dev * 1e-3),
                    "speedup_vs_plain": t_plain / t_batched,
                    "batch_create_s": t_create,
                    "speedup_with_setup_both_sides": t_dropin / (t_setup + t_create + t_batched),
                    "refined_insertions_per_run": refined, "refined_fraction": refined / n_ins,
                    "tuned": {"n_ctas": info["n_ctas"],
                    "order": ["cost-descending", "by-system"][info["order"]], "ms": tuned_ms},
                    "work_units": info["n_units"], "gpu_launches_per_run": 17}
        # spatial order (3), batch kernel, insertion-order partials, per-system reduction, 11 refinement kernels
    # counted-work roofline of the batch kernel: its FP32 pass (refinement off) over insertions of
    # the same kind, against the work the counting pass reports for each system
    screen = BatchScreen(systems, npb, N_BLOCKS, with_adjoint=False, ctx=ctx, refine_tail=0.0)
    screen.tune(1, T, repeats=2)
    for w in range(args.warmup):
        screen.run(2 + w, T)
    k = max(3, args.steps // 2)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    torch.cuda.synchronize()
    for i in range(k):
        ev[i][0].record(stream)
        screen.launch(100 + i, T)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms_fp32 = sum(a.elapsed_time(b) for a, b in ev) / k
    screen.close()
    flops = 0.0
    for s_, gs in enumerate(systems):
        c = gs.widom_work_counts(npb, N_BLOCKS, system_seed(100, s_))
        nq = int((gs.site_charge >= 0).sum()) if gs.charged else 0
        nk = gs.info()["n_kvecs_evaluated"] if gs.charged else 0
        flops += counted_flops(c, npb * N_BLOCKS, nq, nk, gs.image_lists(npb * N_BLOCKS),
                               gs.info()["kspace_mirror"]) * npb * N_BLOCKS
    tf = flops / (ms_fp32 * 1e-3) / 1e12
    out["roofline"] = {"bound": "fp32", "achieved": tf, "unit": "TFLOP/s", "frac": tf / peak if peak else None,
                       "flops_per_run": flops, "fp32_pass_ms": ms_fp32,
                       "kernel": "the batch's forward FP32 pass (refinement off: the spatial order, the persistent "
                                 "batch kernel, partials and per-system reduction), CUDA events around the graph "
                                 "replay",
                       "counting": "pmgb_widom_work_counts of each system over its insertions of one run (26 / 11 / "
                                   "30 flops per distance, LJ term, real-space term; 8 per distance from an image "
                                   "list, the lists' building not counted; per evaluated k-vector 16 + 12 per "
                                   "further guest charge, 21 with mirror-image sites)"}
    assert ctx.device_status() == 0
    out["refined_fraction"] = out["forward_plus_adjoint"]["refined_fraction"]
    out.update({"systems": len(systems), "frameworks": len(fws), "guests": ["CH4", "CO2"],
                "insertions_per_system": npb * N_BLOCKS, "insertions_per_run": n_ins,
                "framework_sites": {"min": int(sizes.min()), "median": float(np.median(sizes)),
                                    "max": int(sizes.max()), "total": int(sizes.sum())},
                "setup_s": t_setup, "framework_generation_s": t_gen,
                "timing": "plain_dropin: wall clock of henry_coefficient(_gradient) per (framework, guest), "
                          "set-up included (one pass); plain: wall clock of the per-system loop over pre-built "
                          "systems (best of 2); batched: wall clock of launch + results per run over the same "
                          "pre-built systems, and CUDA events around the graph replay; setup_s: building the "
                          "batch's systems once (replication, Ewald parameters, pmgb_system_create, S(k)); "
                          "speedup_with_setup_both_sides: the drop-in loop (which builds every system) over "
                          "setup_s + batch_create_s + one batched run; framework_generation_s (the synthetic "
                          "crystals themselves) is charged to neither side"})
    return out


# ------------------------------------------------------------------ error against the FP64 oracle
def widom_error(gs, ff, n_per_block: int, seed: int):
    """A Widom run of gs (its refinement setting) against the FP64 oracle (structure-factor form)
    on the exact device poses: the largest relative error of a block's K_H (sum of e^{-U/T}) and of
    its <U>, and the fraction of insertions whose energy is within 1e-5 relative or 1e-4 K."""
    import numpy as np

    from pmgb.molecule import body_offsets

    blocks, u = gs.widom(n_per_block, N_BLOCKS, seed, T, want_energies=True)
    xf, rot = gs.ctx.sample_poses(seed, 0, N_BLOCKS * n_per_block)
    body = np.zeros((gs.n_sites, 3))
    ax, qx = body_offsets(gs.molecule, gs.crystal.box)
    for k in range(gs.n_sites):
        body[k] = ax[gs.site_atom[k]] if gs.site_atom[k] >= 0 else qx[gs.site_charge[k]]
    o = oracle_system(gs.crystal, gs.molecule, ff, gs.eparams)
    sites = o.sites_from_poses(xf.astype(np.float64), rot.astype(np.float64), body)
    n = sites.shape[0]
    lj = np.zeros((n, gs.molecule.n_atoms, 3))
    q = np.zeros((n, gs.molecule.n_charges, 3))
    for k in range(gs.n_sites):
        if gs.site_atom[k] >= 0:
            lj[:, gs.site_atom[k]] = sites[:, k]
        if gs.site_charge[k] >= 0:
            q[:, gs.site_charge[k]] = sites[:, k]
    v, sr, lr = o.energies(lj, q, charged=gs.charged, use_sk=True)
    u_ref = v + sr + lr
    ug = u.sum(axis=1)
    both_inf = np.isinf(ug) & np.isinf(u_ref)
    with np.errstate(invalid="ignore"):  # inf - inf where both are infinite
        ok = both_inf | (np.abs(ug - u_ref) <= np.maximum(1e-5 * np.abs(u_ref), 1e-4))
    x = np.where(np.isfinite(u_ref), -u_ref / T, -np.inf).reshape(N_BLOCKS, n_per_block)
    m = x.max(axis=1, keepdims=True)
    w = np.exp(x - m)
    log_ref = m[:, 0] + np.log(w.sum(axis=1))
    u_mean = (np.where(np.isfinite(u_ref), u_ref, 0.0).reshape(N_BLOCKS, -1) * w).sum(axis=1) / w.sum(axis=1)
    kh_rel = np.abs(np.expm1(blocks[:, 0] - log_ref))
    u_rel = np.abs(blocks[:, 1] + blocks[:, 2] - u_mean) / np.abs(u_mean)
    return {"insertions": n, "kh_max_rel_error": float(kh_rel.max()), "u_mean_max_rel_error": float(u_rel.max()),
            "insertion_energies_within_tolerance": float(ok.mean()),
            "oracle": "FP64 structure-factor form of the reference's algorithm on the device's own poses"}


def grid_error(gs, ff, n_pts, rep, grid, n_sample: int = 20000, seed: int = 3):
    """Grid values (K) at a random sample of points against the FP64 oracle: the largest relative
    error and the fraction within 1e-5 relative or 1e-4 K."""
    import numpy as np

    o = oracle_system(gs.crystal, gs.molecule, ff, None)
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, int(np.prod(n_pts)), n_sample)
    i, j, k = idx % n_pts[0], (idx // n_pts[0]) % n_pts[1], idx // (n_pts[0] * n_pts[1])
    f = [np.where(a / (n - 1) >= 1.0, 0.0, a / (n - 1)) / r for a, n, r in zip((i, j, k), n_pts, rep)]
    pts = np.stack(f, axis=1)[:, None, :]
    ref = o.energies(pts)[0]
    got = grid[i, j, k].astype(np.float64)
    fin = np.isfinite(ref)
    with np.errstate(invalid="ignore"):  # inf - inf where both are infinite
        ok = (np.isinf(got) & ~fin) | (np.abs(got - ref) <= np.maximum(1e-5 * np.abs(ref), 1e-4))
    rel = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-300)
    return {"points_checked": n_sample, "within_tolerance": float(ok.mean()), "max_rel_error": float(rel.max())}


# ------------------------------------------------------------------ porous cell
def porous_leg(args, ctx, stream, flush):
    """The bench workload's guest and Ewald set-up in a porous variant of the config1 cell (the
    same lattice and species mix at a quarter of the atoms; synthetic.config1_porous), where the
    Boltzmann weight spreads over many insertions: the refined pass with its refined count and the
    refinement's share of the step, and the FP32 pass alone.  CUDA events on the launching stream,
    L2 flushed before every timed step."""
    import torch

    import pmgb
    from pmgb import synthetic

    cr = synthetic.config1_porous()
    ff = synthetic.forcefield(12.5)
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.co2(), sc.box), ff, ep, ctx=ctx, refine_tail=REFINE_TAIL)
    npb = args.insertions // N_BLOCKS
    n = npb * N_BLOCKS
    dev = torch.device("cuda", torch.cuda.current_device())
    block_out = torch.zeros(N_BLOCKS * 4, dtype=torch.float64, device=dev)
    lib = ctx._lib

    def run(seed0, k):
        for w in range(2):
            ctx.check(lib.pmgb_widom_device(gs.handle, npb, N_BLOCKS, seed0 + 100 + w, T, block_out.data_ptr(), None))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        refined = []
        ctx.set_kernel_timing(True)
        for i in range(k):
            flush.zero_()
            ev[i][0].record(stream)
            ctx.check(lib.pmgb_widom_device(gs.handle, npb, N_BLOCKS, seed0 + i, T, block_out.data_ptr(), None))
            ev[i][1].record(stream)
            refined.append(gs.refined_count())
        torch.cuda.synchronize()
        k_ms, k_n = ctx.kernel_timing()
        ctx.set_kernel_timing(False)
        return sum(a.elapsed_time(b) for a, b in ev) / k, k_ms / max(k_n, 1), refined

    k = max(3, min(args.steps, 10))
    ms_ref, kern_ref, refined = run(5000, k)
    err = widom_error(gs, ff, 20000, 5099)
    gs.set_refine(0.0)
    ms32, kern32, _ = run(6000, k)
    assert ctx.device_status() == 0
    return {"workload": "CO2 + Ewald 1e-6 in the porous config1 cell (150 atoms per 13.2 x 18.9 x 9.8 A cell, "
                        "replicated 2x2x3), 1e6 insertions in 5 blocks, 298 K",
            "framework_sites": sc.atoms.n, "insertions": n,
            "insertions_per_s": n / (ms_ref * 1e-3), "ms_per_step": ms_ref,
            "refined_per_step": {"mean": sum(refined) / len(refined), "max": max(refined)},
            "pair_kernel_ms": kern_ref, "refinement_share_of_step": 1.0 - kern_ref / ms_ref,
            "fp32_only_insertions_per_s": n / (ms32 * 1e-3), "fp32_only_ms_per_step": ms32,
            "error_vs_fp64_oracle": err,
            "note": "refined steps: the pair kernel without the box-matrix residual, then the FP64 re-evaluation "
                    "of the insertions that carry all but 1e-3 of each block's Boltzmann weight (K_H within 1e-6); "
                    "refinement_share_of_step = 1 - pair-kernel time / step time (the spatial order, partials and "
                    "block reduction, ~2% of a step, count with the refinement)"}


# ------------------------------------------------------------------ the other configurations
def other_configs(args, ctx, stream, peak=None):
    """The large Ewald cell (config4) and the energy grid (config2), one timed pass each after a
    warm-up, CUDA events on the launching stream.

    config4: CO2 in an orthorhombic 52 x 52 x 52 A cell of 20,000 atoms (same species mix and
      charges), Ewald precision 1e-6, 1e7 insertions in 5 blocks; forward with the FP64 tail
      refinement, forward FP32 only, and forward + adjoint.
    config2: Xe over a 96^3 fractional grid of config0's framework (FP32 output), and the grid
      adjoint (dU/dr per point and dK_H/d(eps, sigma^2)) at 298 K."""
    import ctypes as C

    import torch

    import pmgb
    from pmgb import synthetic

    out = {}

    def timed(fn, reps=1, warm=1):
        for _ in range(warm):
            fn()  # warm-up (allocates scratch)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ff = synthetic.forcefield(12.5)
    mol = synthetic.co2()
    if "config4" in args.legs:
        out["config4_large_ewald"] = config4_leg(args, ctx, ff, mol, timed, peak)
    if "moves" in args.legs:
        out["monte_carlo_move"] = moves_leg(ctx, ff, mol)
    if "config2" in args.legs:
        out["config2_energy_grid"] = config2_leg(ctx, ff, timed, peak)
    assert ctx.device_status() == 0
    return out


def config4_leg(args, ctx, ff, mol, timed, peak):
    """config4: refined, FP32-only and forward + adjoint Widom runs and the error against the oracle."""
    import pmgb
    from pmgb import synthetic

    cr = synthetic.config4()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    gs = pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep, ctx=ctx, refine_tail=REFINE_TAIL)
    npb = args.c4_insertions // N_BLOCKS
    n = npb * N_BLOCKS
    ms_ref = timed(lambda: gs.widom(npb, N_BLOCKS, 41, T))
    refined = gs.refined_count()
    gs.set_refine(0.0)
    ms32 = timed(lambda: gs.widom(npb, N_BLOCKS, 42, T))
    ms_adj = timed(lambda: gs.widom_adjoint(npb, N_BLOCKS, 43, T))
    gs.set_refine(REFINE_TAIL)
    err4 = widom_error(gs, ff, 4000, 44)
    fpi = flops_per_insertion(sc, mol, ep)
    work4 = gs.widom_work_counts(npb, N_BLOCKS, 42)   # the FP32-only run's insertions
    fpc = counted_flops(work4, n, mol.n_charges, gs.info()["n_kvecs_evaluated"], gs.image_lists(n),
                        gs.info()["kspace_mirror"])
    tf4 = fpc * n / (ms32 * 1e-3) / 1e12
    return {
        "workload": "CO2 in a 20,000-atom 52x52x52 A cell, Ewald 1e-6", "framework_sites": sc.atoms.n,
        "kvectors": ep.n_kvecs, "insertions": n,
        "insertions_per_s": n / (ms_ref * 1e-3), "refined_insertions": refined,
        "fp32_only_insertions_per_s": n / (ms32 * 1e-3),
        "forward_plus_adjoint_insertions_per_s": n / (ms_adj * 1e-3),
        "roofline": {"bound": "fp32", "flops_per_insertion": fpc, "achieved": tf4, "unit": "TFLOP/s",
                     "frac": tf4 / peak if peak else None, "work_counts": work4,
                     "kernel": "the FP32-only Widom pass (image-list pair kernel + partials), CUDA events",
                     "counting": "counted by pmgb_widom_work_counts over the same insertions: distances "
                                 "evaluated (8 flops each from an image list, the lists' building not counted), "
                                 "LJ and real-space terms inside their cutoffs (11 / 30 flops), the evaluated "
                                 "k-vectors (21 flops each: CO2's mirror-image sites)"},
        "every_pair_flops_per_insertion": fpi,
        "every_pair_tflops": fpi * n / (ms32 * 1e-3) / 1e12,
        "note": "every_pair_tflops counts every pair and k-vector; in this 52 A cell the kernel skips whole "
                "sub-chunks of records beyond every lane's cutoff, distances included, and the energy terms of "
                "most remaining groups, so that figure exceeds the FP32 peak; the roofline counts the work done",
        "error_vs_fp64_oracle": err4,
        "centre_image": gs.info()["centre_image"],
        "distances": "with centre_image, each record's minimum image is taken from the pose centre once and the "
                     "three sites subtract their offsets (every width of this cell exceeds 2 (cutoff + 1.16 A); "
                     "pmgb_system_set_centre_image; the per-site form differs by FP32 rounding only)"}


def moves_leg(ctx, ff, mol):
    """Monte Carlo move latency: one configuration per call through the captured graph, with exact
    energies (the default) and with the FP32 latency kernel."""
    import numpy as np

    import pmgb
    from pmgb import synthetic

    c1 = synthetic.config1()
    sc1 = pmgb.replicate(c1, pmgb.replication_factors(c1.box, ff))
    g1 = pmgb.GPUSystem(sc1, pmgb.Frac(mol, sc1.box), ff, pmgb.setup_Ewald_sum(sc1.box, ff.r_cutoff, eps=1e-6),
                        ctx=ctx)
    rng = np.random.default_rng(5)
    confs = rng.random((64, 1, 3)) + np.zeros((64, g1.n_sites, 3))  # rigid shifts of all sites

    def latency():
        ev = g1.move_evaluator(1)
        for c in confs[:16]:
            ev.energies(c)
        t0 = time.perf_counter()
        for i in range(500):
            ev.energies(confs[i % 64])
        dt = (time.perf_counter() - t0) / 500 * 1e6
        ev.close()
        return dt

    exact_us = latency()
    g1.set_exact(False)
    fp32_us = latency()
    return {
        "workload": "guest-host energy of one CO2 configuration in the config1 supercell (7,200 sites, Ewald)",
        "us_per_call": exact_us, "fp32_us_per_call": fp32_us,
        "call": "GPUSystem.move_evaluator(1).energies (pmgb_move_energies: pinned staging, one graph replay, "
                "synchronous); us_per_call: exact energies (double-float, the default), fp32: the FP32 latency "
                "kernel"}


def config2_leg(ctx, ff, timed, peak):
    """config2: the 96^3 Xe grid, exact and FP32-only, its counted-work roofline and its error."""
    import ctypes as C

    import torch

    import pmgb
    from pmgb import synthetic

    c0 = synthetic.config0()
    rep = pmgb.replication_factors(c0.box, ff)
    sc0 = pmgb.replicate(c0, rep)
    gx = pmgb.GPUSystem(sc0, pmgb.Frac(synthetic.xe(), sc0.box), ff, ctx=ctx)
    pts = (96, 96, 96)
    n_pts = 96 ** 3
    dev = torch.device("cuda", torch.cuda.current_device())
    grid_dev = torch.empty(n_pts, dtype=torch.float32, device=dev)
    n3 = (C.c_int32 * 3)(*pts)
    r3 = (C.c_int32 * 3)(*rep)

    def grid_device():
        ctx.check(ctx._lib.pmgb_energy_grid_device(gx.handle, n3, r3, 1.0, grid_dev.data_ptr()))

    ms_exact = timed(grid_device, reps=20, warm=3)      # FP32 pass with error estimates + re-evaluation
    refined = gx.refined_count()
    grid_exact = gx.energy_grid(pts, rep, 1.0)
    ms_g = timed(lambda: gx.energy_grid(pts, rep, 1.0), reps=20, warm=3)
    ms_ga = timed(lambda: gx.energy_grid_adjoint(pts, rep, 1.0, T), reps=10, warm=3)
    gx.set_exact(False)
    ms_fp32 = timed(grid_device, reps=20, warm=3)       # the FP32 grid kernel alone
    grid_fp32 = gx.energy_grid(pts, rep, 1.0)
    gx.set_exact(True)
    # counted work of the FP32 grid kernel (pmgb_energy_grid_work_counts): the distances it evaluates
    # and the LJ terms inside the cutoff
    gwork = gx.energy_grid_work_counts(pts, rep)
    fpp = counted_flops(gwork, n_pts)
    tf = fpp * n_pts / (ms_fp32 * 1e-3) / 1e12
    return {
        "workload": "Xe over a 96^3 grid of config0 (424 atoms, 25.832 A cubic)", "points": n_pts,
        "points_per_s": n_pts / (ms_exact * 1e-3),
        "exact": "every point within 1e-5 relative or 1e-4 K of FP64: the FP32 pass with a per-point error "
                 "estimate, then the points it cannot clear re-evaluated in double-float",
        "refined_points": refined, "refined_fraction": refined / n_pts,
        "fp32_only_points_per_s": n_pts / (ms_fp32 * 1e-3),
        "host_call_points_per_s": n_pts / (ms_g * 1e-3), "adjoint_points_per_s": n_pts / (ms_ga * 1e-3),
        "roofline": {"bound": "fp32", "flops_per_point": fpp, "achieved": tf, "unit": "TFLOP/s",
                     "frac": tf / peak if peak else None, "work_counts": gwork,
                     "kernel": "pairs_kernel<1,false,...> (FP32 grid, exact energies off), CUDA events around "
                               "pmgb_energy_grid_device",
                     "counting": "counted by pmgb_energy_grid_work_counts: 26 flops per (record, probe) distance "
                                 "evaluated, 11 more per LJ term inside the cutoff (FMA = 2, MUFU = 1)"},
        "error_vs_fp64_oracle": {"exact": grid_error(gx, ff, pts, rep, grid_exact),
                                 "fp32_only": grid_error(gx, ff, pts, rep, grid_fp32)},
        "timing": "points_per_s and fp32_only: CUDA events around the device call (grid left on the device); "
                  "host_call and adjoint: the host call including the device-to-host copy of the grid (and "
                  "gradients)"}


def job_rate(ms_total: float, n_per_rank_step: int, steps: int, world: int, device="cpu"):
    """The slowest rank bounds the job: (max over ranks of the timed ms, whole-job units/s with
    every rank processing n_per_rank_step units per step).  Ranks are independent replicas; the
    one collective is this max."""
    import torch

    t = torch.tensor([ms_total], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    return ms_max, world * n_per_rank_step * steps / (ms_max * 1e-3)


# ------------------------------------------------------------------ GPU arm
def ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import pmgb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    cr, sc, ff, ep, mol, rep = workload()
    ctx = pmgb.Context(local_rank)
    stream = torch.cuda.Stream(dev)          # a real (non-legacy) stream shared with the library
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    # FP32 pair pass + FP64 refinement of the Boltzmann tail: K_H within 1e-6 of FP64
    system = pmgb.GPUSystem(sc, pmgb.Frac(mol, sc.box), ff, ep, ctx=ctx, refine_tail=REFINE_TAIL)
    system.set_image_lists({"auto": "auto", "on": True, "off": False}[args.image_lists])
    n_ins = args.insertions
    npb = n_ins // N_BLOCKS
    n_ins = npb * N_BLOCKS
    block_out = torch.zeros(N_BLOCKS * 4, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    lib = ctx._lib

    def step(seed):
        ctx.check(lib.pmgb_widom_device(system.handle, npb, N_BLOCKS, seed, T, block_out.data_ptr(), None))

    fp32_peak, peak_clocks = None, None
    if rank == 0:
        # the roofline denominator: the FFMA probe, best of three, with the SM clock it ran at
        with ClockSampler(local_rank) as pclk:  # ~0.5 s of probes, so the sampler sees their clock
            fp32_peak = max(ctx.fp32_peak_tflops(iters=65536) for _ in range(3))
        peak_clocks = pclk.summary()
    for w in range(args.warmup):
        step(10_000 + w)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ctx.set_kernel_timing(True)  # CUDA events around each step's pair-kernel launch, on its stream
    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize()
        t_wall0 = time.perf_counter()
        for s in range(args.steps):
            flush.zero_()
            starts[s].record(stream)
            step(s + 1)
            ends[s].record(stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    k_ms, k_n = ctx.kernel_timing()
    ctx.set_kernel_timing(False)
    kernel_ms = k_ms / max(k_n, 1)  # the dominant kernel of the timed steps, per launch
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    ms_total = sum(ms)
    assert ctx.device_status() == 0
    blocks = block_out.cpu().numpy().reshape(N_BLOCKS, 4)
    assert np.all(np.isfinite(blocks[:, 0])), blocks

    ms_max, value = job_rate(ms_total, n_ins, args.steps, world, dev)

    # the FP32 pair pass alone (pairs_kernel + block reduction): the roofline's kernel time
    system.set_refine(0.0)
    for w in range(2):
        step(20_000 + w)
    ev32 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s_ in range(args.steps):
        flush.zero_()
        ev32[s_][0].record(stream)
        step(30_000 + s_)
        ev32[s_][1].record(stream)
    torch.cuda.synchronize()
    ms32 = sum(a.elapsed_time(b) for a, b in ev32) / args.steps
    system.set_refine(REFINE_TAIL)
    err1 = widom_error(system, ff, 4000, 77) if rank == 0 else None

    # forward + adjoint in one pass (pmgb_widom_adjoint: energies, dK_H/d(eps, sigma, lambda))
    adj = None
    if "adjoint" in args.legs:
        system.widom_adjoint(npb, N_BLOCKS, 7, T)  # warm-up (allocates its scratch)
        a_times = []
        for s in range(max(3, args.steps // 2)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            system.widom_adjoint(npb, N_BLOCKS, 100 + s, T)
            a_times.append(time.perf_counter() - t0)
        adj = {"value": n_ins * len(a_times) / sum(a_times), "unit": UNIT,
               "ms_per_step": 1e3 * sum(a_times) / len(a_times),
               "what": "pmgb_widom_adjoint: forward energies + dK_H/d(epsilon, sigma^2) per species pair + "
                       "dK_H/d(charge scale), pair terms recomputed (host call, includes the D2H of the sums)"}

    # end to end through the reference-facing call (host buffers, copies inside)
    e2e = None
    if "e2e" in args.legs:
        ipv = n_ins / cr.box.Omega
        e_times = []
        ctx_default = pmgb.Context.default(local_rank)
        ctx_default.set_stream(stream.cuda_stream)
        holder = []
        for s in range(2 + args.steps):
            holder.clear()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = pmgb.henry_coefficient(cr, mol, T, ff, insertions_per_volume=ipv, verbose=False, autosave=False,
                                         seed=500 + s, system_out=holder)
            t1 = time.perf_counter()
            if s >= 2:
                e_times.append(t1 - t0)
        n_e2e = res.n_insertions_per_block * N_BLOCKS
        h2d = holder[0].info()["h2d_bytes"] + 0
        e2e = {"value": n_e2e * len(e_times) / sum(e_times), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": N_BLOCKS * 4 * 8, "call": "pmgb.henry_coefficient (host set-up + "
               "pmgb_system_create + pmgb_system_set_ewald + pmgb_widom)"}

    batched = None
    if "batched" in args.legs and rank == 0:
        batched = batched_leg(args, ctx, stream, fp32_peak)
    others = None
    if args.legs & {"config4", "moves", "config2"} and rank == 0:
        others = other_configs(args, ctx, stream, fp32_peak)

    porous = None
    if "porous" in args.legs and rank == 0:
        porous = porous_leg(args, ctx, stream, flush)

    if rank != 0:
        return
    fpi = flops_per_insertion(sc, mol, ep)
    achieved_every = fpi * n_ins / (kernel_ms * 1e-3) / 1e12
    n_kev = system.info()["n_kvecs_evaluated"]
    work = system.widom_work_counts(npb, N_BLOCKS, 1)   # the insertions of the first timed step
    img = system.image_lists(n_ins)
    mirror = system.info()["kspace_mirror"]
    fpi_in = counted_flops(work, n_ins, mol.n_charges, n_kev, img, mirror)
    per_site_eq = None
    if img:  # the same insertions' counted work in the per-site form, completed in the lists' time
        system.set_image_lists(False)
        work_ps = system.widom_work_counts(npb, N_BLOCKS, 1)
        system.set_image_lists({"auto": "auto", "on": True, "off": False}[args.image_lists])
        fpi_ps = counted_flops(work_ps, n_ins, mol.n_charges, n_kev, False, mirror)
        ach_ps = fpi_ps * n_ins / (kernel_ms * 1e-3) / 1e12
        per_site_eq = {"flops_per_insertion": fpi_ps, "work_counts": work_ps, "achieved": ach_ps,
                       "frac": ach_ps / fp32_peak if fp32_peak else None,
                       "meaning": "the per-site pass's counted work for the same insertions (26 flops per "
                                  "(site, record) distance) over the image-list kernel's time: the rate at which "
                                  "the per-site form's work is completed, not a rate of executed flops"}
    fpi_est = flops_inside_cutoff(sc, mol, ff, ep, n_kev)
    achieved = fpi_in * n_ins / (kernel_ms * 1e-3) / 1e12
    cpu = None
    if "cpu" in args.legs:
        cpu = cpu_legs(sc, mol, ep, ff)
    summary = {"kh_max_rel_error": err1["kh_max_rel_error"] if err1 else None,
               "pair_kernel_frac_of_fp32_peak": achieved / fp32_peak if fp32_peak else None,
               "e2e_insertions_per_s": e2e["value"] if e2e else None,
               "cpu_direct_insertions_per_s": cpu["value"] if cpu else None,
               "cpu_sk_form_insertions_per_s": cpu["sk_form"]["value"] if cpu else None,
               "fwd_adj_insertions_per_s": adj["value"] if adj else None}
    if porous:
        summary.update({"porous_insertions_per_s": porous["insertions_per_s"],
                        "porous_refinement_share": porous["refinement_share_of_step"],
                        "porous_kh_max_rel_error": porous["error_vs_fp64_oracle"]["kh_max_rel_error"]})
    if batched:
        fa = batched["forward_plus_adjoint"]
        summary.update({"batched_fwd_adj_insertions_per_s": fa["batched_insertions_per_s"],
                        "batched_vs_plain_prebuilt": fa["speedup_vs_plain"],
                        "batched_vs_plain_with_setup": fa.get("speedup_with_setup_both_sides"),
                        "batched_refined_fraction": batched.get("refined_fraction"),
                        "batched_fp32_pass_frac_of_fp32_peak": batched["roofline"]["frac"]})
    if others and "config4_large_ewald" in others:
        summary["config4_insertions_per_s"] = others["config4_large_ewald"]["insertions_per_s"]
    if others and "config2_energy_grid" in others:
        summary["config2_points_per_s"] = others["config2_energy_grid"]["points_per_s"]
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "summary": summary,
           "config": {"workload": "widom_co2_ewald_600atom_triclinic_2x2x3_1e6",
                      "insertions_per_step": n_ins, "framework_sites": sc.atoms.n, "kvectors": ep.n_kvecs,
                      "guest": "CO2 (3 LJ sites, 3 charges)", "temperature_K": T, "blocks": N_BLOCKS,
                      "l2": "flushed (256 MB write) before every timed step",
                      "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
           "gpu_launches": LAUNCHES_PER_STEP * args.steps,
           "precision": {"pairs": "FP32 (compensated per-site sums)", "accumulation": "FP64 log-sum-exp",
                         "refine_tail": REFINE_TAIL,
                         "kh_error": "insertions carrying all but 1e-3 of each block's Boltzmann weight "
                                     "re-evaluated in FP64 from exact positions: K_H within 1e-6 relative of "
                                     "the FP64 oracle",
                         "error_vs_fp64_oracle": err1,
                         "fp32_only_insertions_per_s": n_ins / (ms32 * 1e-3),
                         "fp32_only_ms_per_step": ms32,
                         "fp32_only": "refinement off: the same pass without the FP64 re-evaluation of the "
                                      "Boltzmann tail"},
           "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": achieved / fp32_peak if fp32_peak else None,
                        "traffic": PAIR_DRAM_BYTES_PER_INSERTION * n_ins,
                        "traffic_source": "ncu DRAM bytes of one image-list pair-kernel launch over 5e5 insertions "
                                          "(2.19 MB), scaled to this launch's insertions "
                                          "(profiles/pairs_img_kernel_config1.md); the framework lives in L2 and "
                                          "the CTAs' shared-memory lists, so the kernel is compute-bound",
                        "peak_source": "in-run FFMA probe (pmgb_fp32_peak, best of 3); MEASURED_PEAKS.json has no "
                                       "FP32 figure",
                        "peak_clocks": peak_clocks,
                        "flops_per_insertion": fpi_in,
                        "work_counts": work,
                        "counting": "the work the kernel does, counted by its work-counting pass "
                                    "(pmgb_widom_work_counts) over the first timed step's insertions: 8 flops per "
                                    "(guest site, list image) distance (3 subtractions and r^2 from the CTA's image "
                                    "list; building the lists, once per CTA and record, is not counted) or 26 per "
                                    "(guest site, record) distance in the per-site form, 11 more per LJ and 30 per "
                                    "real-space term inside their cutoffs; per evaluated k-vector the loop as "
                                    "executed: 21 for CO2's mirror-image sites (16 + 12 per further guest charge "
                                    "in the general loop); FMA = 2, MUFU = 1",
                        "per_site_equivalent": per_site_eq,
                        "flops_per_insertion_uniform_estimate": fpi_est,
                        "kvectors_evaluated": system.info()["n_kvecs_evaluated"],
                        "every_pair": {"flops_per_insertion": fpi, "achieved": achieved_every,
                                       "frac": achieved_every / fp32_peak if fp32_peak else None,
                                       "convention": "every pair and every k-vector counted: LJ 28, real-space 40, "
                                                     "k-term 17 flops; credits the energy terms culling skips and "
                                                     "the k-vectors whose S(k) vanishes"},
                        "kernel": ("pairs_img_kernel<3,true> (CO2, Ewald, forward, image lists over the run's "
                                   "order)" if system.image_lists(n_ins) else
                                   "pairs_kernel<3,true,false,false> (CO2, Ewald, forward, per site, no box residual)")
                                  + ": CUDA events around each of its launches inside the timed refined steps, on the "
                                    "launching stream",
                        "kernel_ms_per_launch": kernel_ms, "kernel_share_of_step": kernel_ms * args.steps / ms_total},
           "forward_plus_adjoint": adj,
           "porous_cell": porous,
           "batched": batched,
           "other_configs": others,
           "clocks": clk.summary(),
           "wall_s_timed_region": t_wall,
           "e2e": e2e,
           "cpu_baseline": cpu}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    try:
        ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
