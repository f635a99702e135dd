"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 CPU oracle (oracle/pm_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / --impl reference legs
may import this module, and only as the checker.  The product path never loads it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libpmoracle.so"

_dp, _ip, _up, _vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_uint32), C.c_void_p
_SIGS = [
    ("or_eps0", C.c_double, []),
    ("or_four_pi_eps0", C.c_double, []),
    ("or_box", None, [C.c_double] * 6 + [_dp, _dp, _dp, _dp]),
    ("or_replication_factors", None, [_dp, C.c_double, _ip]),
    ("or_lennard_jones", C.c_double, [C.c_double, C.c_double, C.c_double]),
    ("or_determine_ewald_params", None, [C.c_double, C.c_double, _dp, _dp]),
    ("or_required_kreps", None, [_dp, C.c_double, _ip]),
    ("or_precompute_kvec_wts", C.c_int, [_ip, _dp, C.c_double, C.c_double, C.c_double, C.c_int, _ip, _dp]),
    ("or_system_create", _vp, [_dp, C.c_int, _dp, _ip, C.c_int, _dp, _dp, C.c_int, _dp, _dp, C.c_double,
                               C.c_int, _ip, C.c_int, _dp]),
    ("or_system_set_ewald", None, [_vp, C.c_double, C.c_double, _ip, C.c_int, _ip, _dp]),
    ("or_system_destroy", None, [_vp]),
    ("or_structure_factor", None, [_vp]),
    ("or_get_structure_factor", None, [_vp, _dp, _dp]),
    ("or_energies", None, [_vp, C.c_int64, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]),
    ("or_energies_scaled", None, [_vp, C.c_int64, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    ("or_widom_blocks", None, [_dp, _dp, C.c_int64, C.c_double, C.c_int, C.c_int64, _dp]),
    ("or_sites_from_poses", None, [_vp, C.c_int64, _dp, _dp, C.c_int, _dp, _dp]),
    ("or_energy_grid", None, [_vp, _ip, _ip, C.c_int, _dp]),
    ("or_philox4x32_10", None, [_up, _up, _up]),
    ("or_num_threads", C.c_int, []),
]
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        h = C.CDLL(str(LIB))
        for n, r, a in _SIGS:
            f = getattr(h, n)
            f.restype = r
            f.argtypes = a
        _lib = h
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def eps0() -> float:
    return lib().or_eps0()


def four_pi_eps0() -> float:
    return lib().or_four_pi_eps0()


def box(a, b, c, alpha, beta, gamma):
    """(f_to_c, c_to_f, reciprocal, Ω) with 3x3 numpy matrices (row i, column j)."""
    f, cf, r = np.zeros(9), np.zeros(9), np.zeros(9)
    om = C.c_double()
    lib().or_box(a, b, c, alpha, beta, gamma, _p(f, C.c_double), _p(cf, C.c_double), _p(r, C.c_double), C.byref(om))
    return f.reshape(3, 3).T, cf.reshape(3, 3).T, r.reshape(3, 3).T, om.value


def _colmajor(m):
    return _d(np.asarray(m, dtype=np.float64).T.reshape(-1))


def replication_factors(f_to_c, r_cutoff):
    rep = np.zeros(3, dtype=np.int32)
    lib().or_replication_factors(_p(_colmajor(f_to_c), C.c_double), r_cutoff, _p(rep, C.c_int))
    return tuple(int(x) for x in rep)


def lennard_jones(r2, sig2, eps):
    return lib().or_lennard_jones(r2, sig2, eps)


def determine_ewald_params(sr_cutoff, eps):
    a, k = C.c_double(), C.c_double()
    lib().or_determine_ewald_params(sr_cutoff, eps, C.byref(a), C.byref(k))
    return a.value, k.value


def required_kreps(recip, max_k2):
    k = np.zeros(3, dtype=np.int32)
    lib().or_required_kreps(_p(_colmajor(recip), C.c_double), max_k2, _p(k, C.c_int))
    return tuple(int(x) for x in k)


def precompute_kvec_wts(kreps, recip, alpha, omega, max_k2=np.inf):
    kr = _i(kreps)
    n = lib().or_precompute_kvec_wts(_p(kr, C.c_int), _p(_colmajor(recip), C.c_double), alpha, omega, max_k2, 0,
                                     None, None)
    abc = np.zeros((n, 3), dtype=np.int32)
    wt = np.zeros(n)
    lib().or_precompute_kvec_wts(_p(kr, C.c_int), _p(_colmajor(recip), C.c_double), alpha, omega, max_k2, n,
                                 _p(abc, C.c_int), _p(wt, C.c_double))
    return abc, wt


def philox4x32_10(ctr, key):
    ctr = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
    key = np.ascontiguousarray(key, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros_like(ctr)
    for i in range(ctr.shape[0]):
        lib().or_philox4x32_10(_p(ctr[i], C.c_uint32), _p(key[i], C.c_uint32), _p(out[i], C.c_uint32))
    return out


def num_threads() -> int:
    return lib().or_num_threads()


def widom_blocks(u_vdw, u_es, temperature, n_blocks, n_per_block):
    """Per-block (Σbf, ΣU_vdw bf, ΣU_es bf) in insertion order (src/henry.jl:212-244)."""
    uv, ue = _d(u_vdw), _d(u_es)
    out = np.zeros(3 * n_blocks)
    lib().or_widom_blocks(_p(uv, C.c_double), _p(ue, C.c_double), uv.shape[0], temperature, n_blocks, n_per_block,
                          _p(out, C.c_double))
    return out.reshape(n_blocks, 3)


def widom_blocks_log(u_vdw, u_es, temperature, n_blocks, n_per_block):
    """The same per-block sums in log space: (log Σbf, ΣU_vdw bf / Σbf, ΣU_es bf / Σbf, #U=+Inf),
    for blocks whose plain FP64 Σ e^{-U/T} underflows."""
    uv = np.asarray(u_vdw, dtype=np.float64).reshape(n_blocks, n_per_block)
    ue = np.asarray(u_es, dtype=np.float64).reshape(n_blocks, n_per_block)
    out = np.zeros((n_blocks, 4))
    for b in range(n_blocks):
        u = uv[b] + ue[b]
        fin = np.isfinite(u)
        out[b, 3] = (~fin).sum()
        if not fin.any():
            out[b, :3] = (-np.inf, np.nan, np.nan)
            continue
        x = -u[fin] / temperature
        m = x.max()
        w = np.exp(x - m)
        s = w.sum()
        out[b, 0] = m + np.log(s)
        out[b, 1] = (w * uv[b][fin]).sum() / s
        out[b, 2] = (w * ue[b][fin]).sum() / s
    return out


class OracleSystem:
    """Replicated crystal + force-field tables + guest description, FP64 on the CPU."""

    def __init__(self, f_to_c, fw_xf, fw_sp, q_xf, q, eps, sig2, r2_cut, g_sp, g_q):
        self.f_to_c = np.asarray(f_to_c, dtype=np.float64)
        self._keep = [_colmajor(f_to_c), _d(fw_xf).reshape(-1, 3), _i(fw_sp), _d(q_xf).reshape(-1, 3), _d(q),
                      _d(eps), _d(sig2), _i(g_sp), _d(g_q)]
        f, fx, fs, qx, qq, e, s2, gs, gq = self._keep
        self.n_species = int(round(np.sqrt(e.size)))
        self.n_glj, self.n_gq = gs.shape[0], gq.shape[0]
        self.h = lib().or_system_create(_p(f, C.c_double), fs.shape[0], _p(fx, C.c_double), _p(fs, C.c_int),
                                        qq.shape[0], _p(qx, C.c_double), _p(qq, C.c_double), self.n_species,
                                        _p(e, C.c_double), _p(s2, C.c_double), r2_cut, self.n_glj, _p(gs, C.c_int),
                                        self.n_gq, _p(gq, C.c_double))
        self.n_k = 0

    def set_ewald(self, alpha, sr_cut, kreps, abc, wt):
        kr, a, w = _i(kreps), _i(abc), _d(wt)
        self.n_k = w.shape[0]
        lib().or_system_set_ewald(self.h, alpha, sr_cut, _p(kr, C.c_int), self.n_k, _p(a, C.c_int),
                                  _p(w, C.c_double))

    def structure_factor(self):
        lib().or_structure_factor(self.h)
        re, im = np.zeros(self.n_k), np.zeros(self.n_k)
        lib().or_get_structure_factor(self.h, _p(re, C.c_double), _p(im, C.c_double))
        return re + 1j * im

    def energies(self, lj_xf, q_xf=None, charged=False, use_sk=False, nthreads=0, scales=False):
        """(vdw, sr, lr) arrays for configurations (n, n_glj, 3) / (n, n_gq, 3); with
        scales=True also (Σ|LJ parts|, Σ|q_g| Σ|real-space terms|) per configuration."""
        lx = _d(lj_xf).reshape(-1, max(self.n_glj, 1) * 3) if self.n_glj else None
        n = lx.shape[0] if lx is not None else _d(q_xf).reshape(-1, self.n_gq * 3).shape[0]
        if lx is None:
            lx = np.zeros((n, 3))
        qx = _d(q_xf).reshape(n, -1) if (charged and self.n_gq) else np.zeros((n, 3))
        vdw, sr, lr = np.zeros(n), np.zeros(n), np.zeros(n)
        sv, ss = np.zeros(n), np.zeros(n)
        lib().or_energies_scaled(self.h, n, _p(lx, C.c_double), _p(qx, C.c_double), int(charged), int(use_sk),
                                 int(nthreads), _p(vdw, C.c_double), _p(sr, C.c_double), _p(lr, C.c_double),
                                 _p(sv, C.c_double), _p(ss, C.c_double))
        if scales:
            return vdw, sr, lr, sv, ss
        return vdw, sr, lr

    def sites_from_poses(self, xf_com, rot, body):
        xf, R, b = _d(xf_com).reshape(-1, 3), _d(rot).reshape(-1, 9), _d(body).reshape(-1, 3)
        n = xf.shape[0]
        out = np.zeros((n, b.shape[0], 3))
        lib().or_sites_from_poses(self.h, n, _p(xf, C.c_double), _p(R, C.c_double), b.shape[0], _p(b, C.c_double),
                                  _p(out, C.c_double))
        return out

    def energy_grid(self, n_pts, rep, nthreads=0):
        n, r = _i(n_pts), _i(rep)
        out = np.zeros(int(np.prod(n)))
        lib().or_energy_grid(self.h, _p(n, C.c_int), _p(r, C.c_int), int(nthreads), _p(out, C.c_double))
        return out.reshape(tuple(int(v) for v in n[::-1])).transpose(2, 1, 0)

    def __del__(self):
        try:
            lib().or_system_destroy(self.h)
        except Exception:
            pass


def accessible(grid_data, xf, repfactors):
    """Vectorised restatement of the accessibility gate (src/grid.jl:778-836; henry.jl:225).

    grid_data: Bool array (n1, n2, n3) over the unit cell; xf: (n, 3) supercell fractional
    centres of mass; repfactors: the supercell's replication.  The point scaled into the unit
    cell, mod 1, has nearest node 1 + round(x (n - 1)) (ties to even, as Julia's round); it is
    accessible iff that node or any of its 26 neighbours is (index 0 -> n, n + 1 -> 1)."""
    g = np.asarray(grid_data, dtype=bool)
    n = np.array(g.shape)
    x = np.mod(np.asarray(xf, dtype=np.float64) * np.asarray(repfactors), 1.0)
    nn = 1 + np.rint(x * (n - 1)).astype(np.int64)      # numpy rint: ties to even
    out = np.zeros(x.shape[0], dtype=bool)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                v = nn + np.array([i, j, k])
                v = np.where(v == 0, n, v)
                v = np.where(v == n + 1, 1, v)
                out |= g[v[:, 0] - 1, v[:, 1] - 1, v[:, 2] - 1]
    return out
