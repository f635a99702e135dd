"""ctypes binding of libpmgb.so (declared in include/pmgb.h).

The library is the only compute path: if it is missing or no CUDA device is present the
calls raise; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpmgb.so"

PMGB_OK = 0
ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "out of device memory",
    -4: "kernel-side failure",
    -5: "unsupported",
    -6: "not ready",
}

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint32)
_vp = C.c_void_p

# (name, restype, argtypes) of every entry point of include/pmgb.h
SIGNATURES = [
    ("pmgb_abi_version", C.c_int, []),
    ("pmgb_create", C.c_int, [C.c_int, C.POINTER(_vp)]),
    ("pmgb_destroy", None, [_vp]),
    ("pmgb_last_error", C.c_char_p, [_vp]),
    ("pmgb_set_stream", C.c_int, [_vp, _vp]),
    ("pmgb_synchronize", C.c_int, [_vp]),
    ("pmgb_system_create", C.c_int,
     [_vp, _dp, C.c_int32, _dp, _ip, C.c_int32, _dp, _dp, C.c_int32, _dp, _dp, C.c_double,
      C.c_int32, _dp, _ip, C.c_int32, _dp, _dp, C.POINTER(_vp)]),
    ("pmgb_system_set_ewald", C.c_int, [_vp, C.c_double, C.c_double, C.c_int32, _ip, _dp]),
    ("pmgb_replication_factors", C.c_int, [_dp, C.c_double, _ip]),
    ("pmgb_ewald_setup", C.c_int, [_dp, C.c_double, C.c_double, C.c_int64, _dp, _dp, _ip, C.POINTER(C.c_int64),
                                   _ip, _dp]),
    ("pmgb_system_create_unitcell", C.c_int,
     [_vp, _dp, C.c_int32, _dp, _ip, C.c_int32, _dp, _dp, C.c_int32, _dp, _dp, C.c_double,
      C.c_int32, _dp, _ip, C.c_int32, _dp, _dp, C.c_double, _ip, C.POINTER(_vp)]),
    ("pmgb_systems_create_unitcell", C.c_int,
     [_vp, C.c_int32, C.POINTER(_dp), _ip, C.POINTER(_dp), C.POINTER(_ip), _ip, C.POINTER(_dp), C.POINTER(_dp), _ip,
      C.POINTER(_dp), C.POINTER(_dp), C.c_double, _ip, C.POINTER(_dp), C.POINTER(_ip), _ip, C.POINTER(_dp),
      C.POINTER(_dp), C.c_double, C.c_int32, _ip, C.POINTER(_vp)]),
    ("pmgb_system_destroy", None, [_vp]),
    ("pmgb_system_info", C.c_int, [_vp, C.POINTER(C.c_int64)]),
    ("pmgb_system_n_sites", C.c_int, [_vp]),
    ("pmgb_system_sites", C.c_int, [_vp, _ip, _ip]),
    ("pmgb_structure_factor", C.c_int, [_vp, _dp]),
    ("pmgb_energies", C.c_int, [_vp, C.c_int64, _dp, _dp]),
    ("pmgb_system_set_cull", C.c_int, [_vp, C.c_int32]),
    ("pmgb_system_set_image_lists", C.c_int, [_vp, C.c_int32]),
    ("pmgb_system_image_lists", C.c_int, [_vp, C.c_int64, _ip]),
    ("pmgb_hilbert_cell", C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32]),
    ("pmgb_system_set_centre_image", C.c_int, [_vp, C.c_int32]),
    ("pmgb_system_centre_image", C.c_int, [_vp, C.POINTER(C.c_int32)]),
    ("pmgb_system_kspace_mirror", C.c_int, [_vp, C.POINTER(C.c_int32)]),
    ("pmgb_system_set_accessibility", C.c_int, [_vp, _ip, _ip, C.POINTER(C.c_uint8)]),
    ("pmgb_system_set_refine", C.c_int, [_vp, C.c_double]),
    ("pmgb_system_set_exact", C.c_int, [_vp, C.c_int32]),
    ("pmgb_system_refined_count", C.c_int, [_vp, C.POINTER(C.c_int64)]),
    ("pmgb_widom", C.c_int, [_vp, C.c_int64, C.c_int32, C.c_uint64, C.c_double, _dp, _dp]),
    ("pmgb_widom_device", C.c_int, [_vp, C.c_int64, C.c_int32, C.c_uint64, C.c_double, _vp, _vp]),
    ("pmgb_widom_noalloc", C.c_int, [_vp, C.c_int64, C.c_int32, C.c_uint64, C.c_double, _vp, _vp]),
    ("pmgb_widom_adjoint", C.c_int, [_vp, C.c_int64, C.c_int32, C.c_uint64, C.c_double, _dp, _dp, _dp, _fp]),
    ("pmgb_energies_grad", C.c_int, [_vp, C.c_int64, _dp, _dp, _fp]),
    ("pmgb_move_create", C.c_int, [_vp, C.c_int32, C.POINTER(_vp)]),
    ("pmgb_move_energies", C.c_int, [_vp, C.c_int32, _dp, _dp]),
    ("pmgb_move_destroy", None, [_vp]),
    ("pmgb_energy_grid_adjoint", C.c_int, [_vp, _ip, _ip, C.c_double, C.c_double, _fp, _fp, _dp]),
    ("pmgb_sample_poses", C.c_int, [_vp, C.c_uint64, C.c_int64, C.c_int64, _fp, _fp]),
    ("pmgb_energy_grid", C.c_int, [_vp, _ip, _ip, C.c_double, _fp]),
    ("pmgb_energy_grid_device", C.c_int, [_vp, _ip, _ip, C.c_double, _vp]),
    ("pmgb_energy_grid_rotational", C.c_int, [_vp, _ip, _ip, C.c_int32, C.c_double, C.c_uint64, C.c_double, _fp]),
    ("pmgb_batch_create", C.c_int, [_vp, C.c_int32, C.POINTER(_vp), C.POINTER(C.c_int64), C.c_int32, C.c_int32,
                                     C.POINTER(_vp)]),
    ("pmgb_batch_destroy", None, [_vp]),
    ("pmgb_batch_configure", C.c_int, [_vp, C.c_int32, C.c_int32, C.c_double]),
    ("pmgb_batch_tune", C.c_int, [_vp, C.c_uint64, C.c_double, C.c_int32, _dp]),
    ("pmgb_batch_set_refine", C.c_int, [_vp, C.c_double]),
    ("pmgb_batch_set_cull", C.c_int, [_vp, C.c_int32]),
    ("pmgb_batch_energies", C.c_int, [_vp, _dp]),
    ("pmgb_widom_work_counts", C.c_int, [_vp, C.c_int64, C.c_int32, C.c_uint64, C.POINTER(C.c_int64)]),
    ("pmgb_energy_grid_work_counts", C.c_int, [_vp, _ip, _ip, C.POINTER(C.c_int64)]),
    ("pmgb_set_kernel_timing", C.c_int, [_vp, C.c_int32]),
    ("pmgb_kernel_timing", C.c_int, [_vp, _dp, C.POINTER(C.c_int64)]),
    ("pmgb_batch_refined_counts", C.c_int, [_vp, C.POINTER(C.c_int64)]),
    ("pmgb_batch_launch", C.c_int, [_vp, C.c_uint64, C.c_double]),
    ("pmgb_batch_results", C.c_int, [_vp, _dp, _dp]),
    ("pmgb_batch_info", C.c_int, [_vp, C.POINTER(C.c_int64)]),
    ("pmgb_philox4x32_10", C.c_int, [_vp, C.c_int64, _up, _up, _up]),
    ("pmgb_vdw_energy_ordered", C.c_int, [_vp, _dp, C.c_int32, _dp, _ip, C.c_int32, _dp, _dp, C.c_double,
                                          C.c_int64, C.c_int32, _ip, _dp, _dp]),
    ("pmgb_fp32_peak", C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    ("pmgb_device_status", C.c_int, [_vp, _up]),
    ("pmgb_test_bounded_wait", C.c_int, [_vp, C.c_int64, C.c_int32]),
]


class PMGBError(RuntimeError):
    """A libpmgb call returned a nonzero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"libpmgb: {ERRORS.get(code, 'error')} ({code}): {message}")
        self.code = code


_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """Load libpmgb.so once (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"libpmgb.so not found at {LIB_PATH}: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` (the CUDA path has no fallback)")
            handle = C.CDLL(str(LIB_PATH))
            for name, res, args in SIGNATURES:
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def ptr(arr, ctype):
    """Pointer to a C-contiguous numpy array (None for None)."""
    if arr is None:
        return None
    assert isinstance(arr, np.ndarray) and arr.flags["C_CONTIGUOUS"], "expected a C-contiguous numpy array"
    return arr.ctypes.data_as(C.POINTER(ctype))


class Context:
    """A libpmgb context: one CUDA device, one stream."""

    _default: dict[int, "Context"] = {}

    def __init__(self, device: int = 0):
        self._lib = lib()
        h = _vp()
        rc = self._lib.pmgb_create(int(device), C.byref(h))
        if rc != PMGB_OK:
            raise PMGBError(rc, self._lib.pmgb_last_error(None).decode())
        self.handle = h
        self.device = device

    @classmethod
    def default(cls, device: int = 0) -> "Context":
        if device not in cls._default:
            cls._default[device] = Context(device)
        return cls._default[device]

    def check(self, rc: int) -> None:
        if rc != PMGB_OK:
            raise PMGBError(rc, self._lib.pmgb_last_error(self.handle).decode())

    def set_stream(self, stream_handle: int | None) -> None:
        self.check(self._lib.pmgb_set_stream(self.handle, _vp(stream_handle) if stream_handle else None))

    def synchronize(self) -> None:
        self.check(self._lib.pmgb_synchronize(self.handle))

    def set_kernel_timing(self, on: bool) -> None:
        """Record CUDA events around every Widom pass's pair-kernel launch (pmgb_set_kernel_timing)."""
        self.check(self._lib.pmgb_set_kernel_timing(self.handle, int(bool(on))))

    def kernel_timing(self) -> tuple[float, int]:
        """(summed pair-kernel ms, launches) recorded since the last read; synchronises and clears."""
        ms, n = C.c_double(0.0), C.c_int64(0)
        self.check(self._lib.pmgb_kernel_timing(self.handle, C.byref(ms), C.byref(n)))
        return ms.value, int(n.value)

    def device_status(self) -> int:
        st = C.c_uint32(0)
        self.check(self._lib.pmgb_device_status(self.handle, C.byref(st)))
        return int(st.value)

    def test_bounded_wait(self, limit_ns: int, arm: bool) -> None:
        """Run the self-test of the kernels' bounded mbarrier wait (pmgb_test_bounded_wait);
        raises PMGBError (kernel-side failure) when the wait gave up."""
        self.check(self._lib.pmgb_test_bounded_wait(self.handle, int(limit_ns), int(bool(arm))))

    def philox4x32_10(self, ctr: np.ndarray, key: np.ndarray) -> np.ndarray:
        ctr = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
        key = np.ascontiguousarray(key, dtype=np.uint32).reshape(-1, 2)
        assert ctr.shape[0] == key.shape[0]
        out = np.zeros_like(ctr)
        self.check(self._lib.pmgb_philox4x32_10(self.handle, ctr.shape[0], ptr(ctr, C.c_uint32),
                                                ptr(key, C.c_uint32), ptr(out, C.c_uint32)))
        return out

    def vdw_energy_ordered(self, f_to_c, atom_xf, atom_species, eps, sigma2, r2_cutoff: float, site_species,
                           site_xf) -> np.ndarray:
        """FP64 guest-host van der Waals energies (K) in the reference's operation order
        (pmgb_vdw_energy_ordered).  atom_xf (n_atoms, 3) in the crystal's atom order; eps and
        sigma2 (n_species, n_species) indexed [guest species, atom species]; site_xf
        (n_conf, n_sites, 3)."""
        f2c = np.ascontiguousarray(np.asarray(f_to_c, dtype=np.float64).reshape(3, 3).T)  # column-major
        axf = np.ascontiguousarray(atom_xf, dtype=np.float64).reshape(-1, 3)
        asp = np.ascontiguousarray(atom_species, dtype=np.int32)
        e = np.ascontiguousarray(eps, dtype=np.float64)
        s2 = np.ascontiguousarray(sigma2, dtype=np.float64)
        ssp = np.ascontiguousarray(site_species, dtype=np.int32)
        sxf = np.ascontiguousarray(site_xf, dtype=np.float64).reshape(-1, ssp.shape[0], 3)
        assert asp.shape[0] == axf.shape[0] and e.shape == s2.shape and e.shape[0] == e.shape[1]
        out = np.zeros(sxf.shape[0], dtype=np.float64)
        self.check(self._lib.pmgb_vdw_energy_ordered(
            self.handle, ptr(f2c, C.c_double), axf.shape[0], ptr(axf, C.c_double), ptr(asp, C.c_int32),
            e.shape[0], ptr(e, C.c_double), ptr(s2, C.c_double), float(r2_cutoff), sxf.shape[0], ssp.shape[0],
            ptr(ssp, C.c_int32), ptr(sxf, C.c_double), ptr(out, C.c_double)))
        return out

    def sample_poses(self, seed: int, start: int, n: int):
        xf = np.zeros((n, 3), dtype=np.float32)
        rot = np.zeros((n, 9), dtype=np.float32)
        self.check(self._lib.pmgb_sample_poses(self.handle, int(seed), int(start), int(n),
                                               ptr(xf, C.c_float), ptr(rot, C.c_float)))
        return xf, rot

    def fp32_peak_tflops(self, n_ctas: int = 152 * 8, iters: int = 4096) -> float:
        out = C.c_double(0.0)
        self.check(self._lib.pmgb_fp32_peak(self.handle, int(n_ctas), int(iters), C.byref(out)))
        return float(out.value)

    def __del__(self):
        try:
            if getattr(self, "handle", None) and _lib is not None:
                _lib.pmgb_destroy(self.handle)
                self.handle = None
        except Exception:
            pass
