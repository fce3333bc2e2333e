"""ctypes binding of libcsp_gb300.so (the C ABI declared in include/csp_c_api.h).

There is no fallback: if the native library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .scenes import ELEMENT_DTYPE

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libcsp_gb300.so")
MAX_DEPTH = 5
NO_ELEMENT = 0xFFFFFFFF

STATUS = {
    0: "CSP_OK",
    -1: "CSP_ERR_INVALID_ARGUMENT",
    -2: "CSP_ERR_CUDA",
    -3: "CSP_ERR_OUT_OF_MEMORY",
    -4: "CSP_ERR_BAD_SCENE",
    -5: "CSP_ERR_TIMEOUT",
    -6: "CSP_ERR_STATE",
    -7: "CSP_ERR_IO",
    -8: "CSP_ERR_PARSE",
}

# every entry point of include/csp_c_api.h: name -> (restype, argtypes)
_H = ctypes.c_void_p
_P = ctypes.c_void_p
SIGNATURES = {
    "csp_last_error": (ctypes.c_char_p, []),
    "csp_abi_version": (ctypes.c_int, []),
    "csp_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_uint64]),
    "csp_destroy": (ctypes.c_int, [_H]),
    "csp_set_num_rays": (ctypes.c_int, [_H, ctypes.c_uint64]),
    "csp_add_element": (ctypes.c_int, [_H, _P]),
    "csp_set_elements": (ctypes.c_int, [_H, _P, ctypes.c_uint32]),
    "csp_get_num_elements": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint32)]),
    "csp_get_elements": (ctypes.c_int, [_H, _P, ctypes.c_uint32]),
    "csp_set_sun_vector": (ctypes.c_int, [_H, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "csp_set_sun_shape": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_double]),
    "csp_set_seed": (ctypes.c_int, [_H, ctypes.c_uint64, ctypes.c_uint32]),
    "csp_set_record_ids": (ctypes.c_int, [_H, ctypes.c_int]),
    "csp_initialize": (ctypes.c_int, [_H]),
    "csp_run": (ctypes.c_int, [_H]),
    "csp_trace_async": (ctypes.c_int, [_H, _P]),
    "csp_update": (ctypes.c_int, [_H]),
    "csp_copy_hits": (ctypes.c_int, [_H, _P, _P, ctypes.c_uint64, ctypes.c_uint64]),
    "csp_run_to_host": (ctypes.c_int, [_H, _P, _P]),
    "csp_get_device_buffers": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]),
    "csp_get_timing": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "csp_get_sun_plane": (ctypes.c_int, [_H, _P]),
    "csp_parse_stinput": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), _P, _P,
                                         ctypes.c_int]),
    "csp_read_stinput": (ctypes.c_int, [_H, ctypes.c_char_p, ctypes.c_int]),
    "csp_write_hits_csv": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_char_p]),
    "csp_write_output": (ctypes.c_int, [_H, ctypes.c_char_p]),
    "csp_write_hits_csv_ex": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int]),
    "csp_write_output_ex": (ctypes.c_int, [_H, ctypes.c_char_p, ctypes.c_int]),
    "csp_element_frame": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "csp_trace_into": (ctypes.c_int, [_H, _P, _P, ctypes.c_uint64, ctypes.c_uint64, _P]),
    "csp_trace_noalloc": (ctypes.c_int, [ctypes.c_int, _P, ctypes.c_uint32, _P, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, _P, _P,
                                         _P]),
    "csp_set_accel": (ctypes.c_int, [_H, ctypes.c_int]),
    "csp_get_accel": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_int)]),
    "csp_flux_map": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_double, _P]),
    "csp_flux_map_ex": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _P, ctypes.c_double, _P]),
    "csp_batch_set_output": (ctypes.c_int, [_H, ctypes.c_int]),
    "csp_server_set_output": (ctypes.c_int, [_H, ctypes.c_int]),
    "csp_flux_target": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, _P]),
    "csp_batch_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "csp_batch_destroy": (ctypes.c_int, [_H]),
    "csp_batch_set_flux_grid": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.c_uint32]),
    "csp_batch_add_scene": (ctypes.c_int, [_H, _P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]),
    "csp_batch_add_instance": (ctypes.c_int, [_H, ctypes.c_uint32, _P, _P, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                              ctypes.POINTER(ctypes.c_uint32)]),
    "csp_batch_clear_instances": (ctypes.c_int, [_H]),
    "csp_batch_num_instances": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint32)]),
    "csp_batch_set_tuning": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "csp_batch_get_tuning": (ctypes.c_int, [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "csp_batch_run": (ctypes.c_int, [_H]),
    "csp_batch_run_async": (ctypes.c_int, [_H]),
    "csp_batch_wait": (ctypes.c_int, [_H]),
    "csp_batch_get_flux": (ctypes.c_int, [_H, ctypes.c_uint32, _P, ctypes.c_double, _P]),
    "csp_batch_get_stats": (ctypes.c_int, [_H, ctypes.c_uint32, _P]),
    "csp_batch_get_sun_plane": (ctypes.c_int, [_H, ctypes.c_uint32, _P]),
    "csp_batch_get_timing": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "csp_batch_get_transfer": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "csp_server_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_uint64,
                                         ctypes.c_uint32, ctypes.c_uint64]),
    "csp_server_destroy": (ctypes.c_int, [_H]),
    "csp_server_add_scene": (ctypes.c_int, [_H, _P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]),
    "csp_server_submit": (ctypes.c_int, [_H, ctypes.c_uint32, _P, _P, ctypes.c_int, ctypes.c_double, ctypes.c_uint64,
                                         ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]),
    "csp_server_wait": (ctypes.c_int, [_H, ctypes.c_uint64, ctypes.c_double, _P, _P, _P]),
    "csp_server_hold": (ctypes.c_int, [_H, ctypes.c_int]),
    "csp_server_stats": (ctypes.c_int, [_H, _P]),
    "csp_run_to_host_compact": (ctypes.c_int, [_H, _P, _P, _P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    "csp_write_compact_csv": (ctypes.c_int, [_P, _P, _P, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int]),
    "csp_debug_fail_allocation": (ctypes.c_int, [ctypes.c_int64]),
    "csp_set_tune_cache": (ctypes.c_int, [ctypes.c_char_p]),
    "csp_tune_cache_entries": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint32)]),
    "csp_bounds_check_status": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]),
}
STINPUT_APPLY_OPTICS = 1
OUT_STAGED = 1  # staged results: rays straight from the sun to the receiver left out
ACCEL_AUTO, ACCEL_BVH, ACCEL_GRID, ACCEL_LIST = 0, 1, 2, 3
GROUP_LIST, GROUP_BVH, GROUP_GRID = 0, 1, 2  # batch kernel groups

_lib = None
_lock = threading.Lock()


class CspError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the native library (no fallback): `path`, else the file CSP_NATIVE_LIB names (the
    bounds-check build, for instance), else the in-tree build."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or os.environ.get("CSP_NATIVE_LIB") or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(f"native library {p} is missing: run optixsoltracedemos_gb300.build.build()")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise CspError(rc, load().csp_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Tracer:
    """One csp_handle: scene, sun, device buffers."""

    def __init__(self, device: int = 0, num_rays: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.csp_create(ctypes.byref(h), int(device), int(num_rays)))
        self.h = h
        self.num_rays = int(num_rays)
        self.record_ids = False

    # ---- configuration
    def set_num_rays(self, n: int):
        _check(self.lib.csp_set_num_rays(self.h, int(n)))
        self.num_rays = int(n)

    def set_elements(self, elements: np.ndarray):
        e = np.ascontiguousarray(elements)
        if e.dtype != ELEMENT_DTYPE:
            raise TypeError("elements must use scenes.ELEMENT_DTYPE")
        _check(self.lib.csp_set_elements(self.h, _ptr(e), len(e)))

    def add_element(self, element: np.ndarray):
        e = np.ascontiguousarray(element.reshape(1))
        _check(self.lib.csp_add_element(self.h, _ptr(e)))

    def get_elements(self) -> np.ndarray:
        n = ctypes.c_uint32()
        _check(self.lib.csp_get_num_elements(self.h, ctypes.byref(n)))
        out = np.zeros(n.value, ELEMENT_DTYPE)
        if n.value:
            _check(self.lib.csp_get_elements(self.h, _ptr(out), n.value))
        return out

    def set_sun_vector(self, x, y=None, z=None):
        if y is None:
            x, y, z = x
        _check(self.lib.csp_set_sun_vector(self.h, float(x), float(y), float(z)))

    def set_sun_shape(self, shape: int, param: float):
        _check(self.lib.csp_set_sun_shape(self.h, int(shape), float(param)))

    def set_seed(self, seed: int, instance: int = 0):
        _check(self.lib.csp_set_seed(self.h, int(seed), int(instance)))

    def set_record_ids(self, enable: bool = True):
        _check(self.lib.csp_set_record_ids(self.h, 1 if enable else 0))
        self.record_ids = bool(enable)

    def set_accel(self, mode: int):
        """ACCEL_AUTO / ACCEL_BVH / ACCEL_GRID (next initialize())."""
        _check(self.lib.csp_set_accel(self.h, int(mode)))

    def accel(self) -> int:
        m = ctypes.c_int()
        _check(self.lib.csp_get_accel(self.h, ctypes.byref(m)))
        return m.value

    # ---- lifecycle
    def initialize(self):
        _check(self.lib.csp_initialize(self.h))

    def run(self):
        _check(self.lib.csp_run(self.h))

    def trace_async(self, stream: int | None = None):
        _check(self.lib.csp_trace_async(self.h, ctypes.c_void_p(stream or 0)))

    def update(self):
        _check(self.lib.csp_update(self.h))

    def copy_hits(self, first: int = 0, count: int | None = None, with_ids: bool | None = None):
        count = self.num_rays - first if count is None else count
        hits = np.empty((count, MAX_DEPTH, 4), np.float32)
        with_ids = self.record_ids if with_ids is None else with_ids
        ids = np.empty((count, MAX_DEPTH), np.uint32) if with_ids else None
        _check(self.lib.csp_copy_hits(self.h, _ptr(hits), _ptr(ids), int(first), int(count)))
        return hits, ids

    def run_to_host(self, hits: np.ndarray, ids: np.ndarray | None = None):
        """hits: float32 array with num_rays*5*4 elements (page-locked for full speed)."""
        if hits.dtype != np.float32 or hits.size != self.num_rays * MAX_DEPTH * 4 or not hits.flags.c_contiguous:
            raise ValueError("hits must be a contiguous float32 array of num_rays*5*4 elements")
        _check(self.lib.csp_run_to_host(self.h, _ptr(hits), _ptr(ids)))

    def trace_into(self, hits_ptr: int, ids_ptr: int | None = None, first: int = 0, count: int | None = None,
                   stream: int | None = None):
        count = self.num_rays - first if count is None else count
        _check(self.lib.csp_trace_into(self.h, ctypes.c_void_p(hits_ptr), ctypes.c_void_p(ids_ptr or 0), int(first),
                                       int(count), ctypes.c_void_p(stream or 0)))

    def run_to_host_compact(self, points: np.ndarray | None = None, counts: np.ndarray | None = None,
                            records: np.ndarray | None = None):
        """Trace and copy the records in compact form: (points [N, 3] float32, counts [N] uint8,
        records [R, 4] float32).  Arrays given are filled (records sized for 4 N)."""
        n = self.num_rays
        points = np.empty((n, 3), np.float32) if points is None else points
        counts = np.empty(n, np.uint8) if counts is None else counts
        records = np.empty((4 * n, 4), np.float32) if records is None else records
        nr = ctypes.c_uint64()
        _check(self.lib.csp_run_to_host_compact(self.h, _ptr(points), _ptr(counts), _ptr(records), records.shape[0],
                                                ctypes.byref(nr)))
        return points, counts, records[:nr.value]

    def run_to_host_compact_ptr(self, points_ptr: int, counts_ptr: int, records_ptr: int, capacity: int) -> int:
        """run_to_host_compact into caller memory (pinned host memory for full link speed); returns
        the number of records."""
        nr = ctypes.c_uint64()
        _check(self.lib.csp_run_to_host_compact(self.h, ctypes.c_void_p(points_ptr), ctypes.c_void_p(counts_ptr),
                                                ctypes.c_void_p(records_ptr), int(capacity), ctypes.byref(nr)))
        return nr.value

    def run_to_host_ptr(self, hits_ptr: int, ids_ptr: int | None = None):
        _check(self.lib.csp_run_to_host(self.h, ctypes.c_void_p(hits_ptr), ctypes.c_void_p(ids_ptr or 0)))

    def device_buffers(self):
        a, b = ctypes.c_void_p(), ctypes.c_void_p()
        _check(self.lib.csp_get_device_buffers(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def timing(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(self.lib.csp_get_timing(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def sun_plane(self) -> np.ndarray:
        out = np.zeros(16, np.float32)
        _check(self.lib.csp_get_sun_plane(self.h, _ptr(out)))
        return out

    def flux_map(self, nx: int = 100, ny: int = 100, dni: float = 1000.0, staged: bool = False):
        """(counts [nx, ny] uint32, flux [nx, ny] W/m^2) of the last run, binned on the device;
        staged: without the receiver records of rays straight from the sun."""
        counts = np.zeros((nx, ny), np.uint32)
        flux = np.zeros((nx, ny), np.float64)
        _check(self.lib.csp_flux_map_ex(self.h, int(nx), int(ny), OUT_STAGED if staged else 0, _ptr(counts),
                                        float(dni), _ptr(flux)))
        return counts, flux

    def read_stinput(self, path: str, apply_optics: bool = False):
        _check(self.lib.csp_read_stinput(self.h, path.encode(), STINPUT_APPLY_OPTICS if apply_optics else 0))

    def write_output(self, path: str, staged: bool = False):
        """The reference's CSV of the last run; staged: without the rows of rays straight from the
        sun to the receiver (clean_direct_sun.py's output)."""
        _check(self.lib.csp_write_output_ex(self.h, path.encode(), OUT_STAGED if staged else 0))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            _check(self.lib.csp_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """One csp_batch: many scene instances traced in one persistent launch, flux maps out."""

    def __init__(self, device: int = 0, nx: int = 100, ny: int = 100):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.csp_batch_create(ctypes.byref(h), int(device)))
        self.h = h
        self.nx, self.ny = int(nx), int(ny)
        _check(self.lib.csp_batch_set_flux_grid(self.h, self.nx, self.ny))

    def add_scene(self, elements: np.ndarray) -> int:
        e = np.ascontiguousarray(elements)
        if e.dtype != ELEMENT_DTYPE:
            raise TypeError("elements must use scenes.ELEMENT_DTYPE")
        sid = ctypes.c_uint32()
        _check(self.lib.csp_batch_add_scene(self.h, _ptr(e), len(e), ctypes.byref(sid)))
        return sid.value

    def add_instance(self, scene: int, sun_dir, sun_shape: int, sun_param: float, num_rays: int, seed: int = 0,
                     instance: int = 0, poses: np.ndarray | None = None) -> int:
        p = None
        if poses is not None:
            p = np.ascontiguousarray(poses)
            if p.dtype != ELEMENT_DTYPE:
                raise TypeError("poses must use scenes.ELEMENT_DTYPE")
        sd = np.ascontiguousarray(sun_dir, np.float64)
        idx = ctypes.c_uint32()
        _check(self.lib.csp_batch_add_instance(self.h, int(scene), _ptr(p), _ptr(sd), int(sun_shape),
                                               float(sun_param), int(num_rays), int(seed), int(instance),
                                               ctypes.byref(idx)))
        return idx.value

    def clear_instances(self):
        _check(self.lib.csp_batch_clear_instances(self.h))

    def __len__(self) -> int:
        n = ctypes.c_uint32()
        _check(self.lib.csp_batch_num_instances(self.h, ctypes.byref(n)))
        return n.value

    def set_tuning(self, block: int = 0, ctas_per_sm: int = 0, chunk: int = 0):
        _check(self.lib.csp_batch_set_tuning(self.h, int(block), int(ctas_per_sm), int(chunk)))

    def tuning(self, group: int) -> tuple[int, int, int]:
        """(block, ctas_per_sm, chunk) of the last run for a kernel group: GROUP_LIST (<= 8 elements),
        GROUP_BVH or GROUP_GRID."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(self.lib.csp_batch_get_tuning(self.h, int(group), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def run(self):
        _check(self.lib.csp_batch_run(self.h))

    def set_output(self, staged: bool = False):
        """Staged flux maps (no receiver records of rays straight from the sun) from the next run on."""
        _check(self.lib.csp_batch_set_output(self.h, OUT_STAGED if staged else 0))

    def run_async(self):
        """Build the current instances and queue their run behind the one in flight (at most two)."""
        _check(self.lib.csp_batch_run_async(self.h))

    def wait(self):
        """Complete the oldest run in flight; its results become the current ones."""
        _check(self.lib.csp_batch_wait(self.h))

    def counts(self, index: int) -> np.ndarray:
        out = np.zeros((self.nx, self.ny), np.uint32)
        _check(self.lib.csp_batch_get_flux(self.h, int(index), _ptr(out), 0.0, None))
        return out

    def flux(self, index: int, dni: float = 1000.0) -> np.ndarray:
        out = np.zeros((self.nx, self.ny), np.float64)
        _check(self.lib.csp_batch_get_flux(self.h, int(index), None, float(dni), _ptr(out)))
        return out

    def stats(self, index: int) -> np.ndarray:
        out = np.zeros(4, np.uint64)
        _check(self.lib.csp_batch_get_stats(self.h, int(index), _ptr(out)))
        return out

    def sun_plane(self, index: int) -> np.ndarray:
        out = np.zeros(16, np.float32)
        _check(self.lib.csp_batch_get_sun_plane(self.h, int(index), _ptr(out)))
        return out

    def timing(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(self.lib.csp_batch_get_timing(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def transfer(self):
        """(host-to-device bytes, device-to-host bytes) of the last completed run."""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib.csp_batch_get_transfer(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            _check(self.lib.csp_batch_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """One csp_server: a request loop with continuous batching over resident scenes."""

    def __init__(self, device: int = 0, memory_budget: int = 0, max_active: int = 64, step_rays: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.csp_server_create(ctypes.byref(h), int(device), int(memory_budget), int(max_active),
                                          int(step_rays)))
        self.h = h

    def add_scene(self, elements: np.ndarray) -> int:
        e = np.ascontiguousarray(elements)
        if e.dtype != ELEMENT_DTYPE:
            raise TypeError("elements must use scenes.ELEMENT_DTYPE")
        sid = ctypes.c_uint32()
        _check(self.lib.csp_server_add_scene(self.h, _ptr(e), len(e), ctypes.byref(sid)))
        return sid.value

    def submit(self, scene: int, sun_dir, sun_shape: int, sun_param: float, num_rays: int, seed: int = 0,
               instance: int = 0, poses: np.ndarray | None = None) -> int:
        p = None
        if poses is not None:
            p = np.ascontiguousarray(poses)
            if p.dtype != ELEMENT_DTYPE:
                raise TypeError("poses must use scenes.ELEMENT_DTYPE")
        sd = np.ascontiguousarray(sun_dir, np.float64)
        rid = ctypes.c_uint64()
        _check(self.lib.csp_server_submit(self.h, int(scene), _ptr(p), _ptr(sd), int(sun_shape), float(sun_param),
                                          int(num_rays), int(seed), int(instance), ctypes.byref(rid)))
        return rid.value

    def hold(self, on: bool = True):
        """Pause (True) or resume (False) admission of queued requests."""
        _check(self.lib.csp_server_hold(self.h, 1 if on else 0))

    def set_output(self, staged: bool = False):
        """Staged flux maps for the requests submitted from now on."""
        _check(self.lib.csp_server_set_output(self.h, OUT_STAGED if staged else 0))

    def wait(self, request: int, timeout: float = -1.0):
        """(counts [100, 100] uint32, stats [4] uint64, (latency s, queueing s))."""
        counts = np.zeros((100, 100), np.uint32)
        stats = np.zeros(4, np.uint64)
        lat = np.zeros(2, np.float64)
        _check(self.lib.csp_server_wait(self.h, int(request), float(timeout), _ptr(counts), _ptr(stats), _ptr(lat)))
        return counts, stats, (float(lat[0]), float(lat[1]))

    def stats(self) -> dict:
        out = np.zeros(8, np.float64)
        _check(self.lib.csp_server_stats(self.h, _ptr(out)))
        keys = ["completed", "rays", "p50_s", "p99_s", "rays_per_s", "peak_active", "peak_arena_bytes", "steps"]
        return dict(zip(keys, out.tolist()))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            _check(self.lib.csp_server_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def write_compact_csv(points: np.ndarray, counts: np.ndarray, records: np.ndarray, path: str,
                      staged: bool = False) -> None:
    """The reference CSV (write_output) of compact records, host only."""
    p = np.ascontiguousarray(points, np.float32)
    c = np.ascontiguousarray(counts, np.uint8)
    r = np.ascontiguousarray(records, np.float32)
    _check(load().csp_write_compact_csv(_ptr(p), _ptr(c), _ptr(r), len(c), path.encode(),
                                        OUT_STAGED if staged else 0))


def debug_fail_allocation(after: int) -> None:
    """Make the library's allocation after `after` further successful ones fail (out of memory),
    once; -1 cancels."""
    _check(load().csp_debug_fail_allocation(int(after)))


def set_tune_cache(path: str | None) -> int:
    """Use `path` as the batched autotuner's persistent cache (None: this process only); returns the
    tunings known after reading it."""
    lib = load()
    _check(lib.csp_set_tune_cache(path.encode() if path else None))
    return tune_cache_entries()


def tune_cache_entries() -> int:
    n = ctypes.c_uint32()
    _check(load().csp_tune_cache_entries(ctypes.byref(n)))
    return n.value


def bounds_check_status(device: int = 0) -> int:
    """Bit mask of the index checks that failed on the device since the last call (bounds-check
    builds only; CspError otherwise)."""
    v = ctypes.c_uint32()
    _check(load().csp_bounds_check_status(int(device), ctypes.byref(v)))
    return v.value


def flux_target(receiver: np.ndarray, nx: int = 100, ny: int = 100) -> np.ndarray:
    """Host-only: the float binning parameters of a receiver element (csp_flux_target, 20 floats)."""
    e = np.ascontiguousarray(np.asarray(receiver).reshape(1))
    if e.dtype != ELEMENT_DTYPE:
        raise TypeError("receiver must use scenes.ELEMENT_DTYPE")
    out = np.zeros(20, np.float32)
    _check(load().csp_flux_target(_ptr(e), int(nx), int(ny), _ptr(out)))
    return out


def parse_stinput(path: str, apply_optics: bool = False):
    """Host-only .stinput parse: (elements, sun_dir, sun_angle)."""
    lib = load()
    n = ctypes.c_uint32()
    sun = np.zeros(3, np.float64)
    ang = np.zeros(1, np.float64)
    fl = STINPUT_APPLY_OPTICS if apply_optics else 0
    _check(lib.csp_parse_stinput(path.encode(), None, 0, ctypes.byref(n), _ptr(sun), _ptr(ang), fl))
    out = np.zeros(n.value, ELEMENT_DTYPE)
    _check(lib.csp_parse_stinput(path.encode(), _ptr(out), n.value, ctypes.byref(n), _ptr(sun), _ptr(ang), fl))
    return out, sun, float(ang[0])


def trace_noalloc(elements: np.ndarray, sun_dir, sun_shape: int, sun_param: float, hits_ptr: int,
                  ids_ptr: int | None = None, first_ray: int = 0, num_rays: int = 0, seed: int = 0,
                  instance: int = 0, device: int = 0, stream: int | None = None) -> None:
    """csp_trace_noalloc: trace into caller-owned device buffers without any allocation (<= 8 elements)."""
    e = np.ascontiguousarray(elements)
    if e.dtype != ELEMENT_DTYPE:
        raise TypeError("elements must use scenes.ELEMENT_DTYPE")
    sd = np.ascontiguousarray(sun_dir, np.float64)
    _check(load().csp_trace_noalloc(int(device), _ptr(e), len(e), _ptr(sd), int(sun_shape), float(sun_param),
                                    int(seed), int(instance), int(first_ray), int(num_rays),
                                    ctypes.c_void_p(hits_ptr), ctypes.c_void_p(ids_ptr or 0),
                                    ctypes.c_void_p(stream or 0)))


def write_hits_csv(hits: np.ndarray, path: str, staged: bool = False) -> None:
    """Host-only CSV writer of [N, 5, 4] float32 hit records (the reference's write_output format);
    staged: without the rows of rays straight from the sun to the receiver."""
    h = np.ascontiguousarray(hits, np.float32)
    _check(load().csp_write_hits_csv_ex(_ptr(h), h.shape[0], path.encode(), OUT_STAGED if staged else 0))


def tracer_for(scene, device: int = 0, seed: int = 0, instance: int = 0, record_ids: bool = True,
               num_rays: int | None = None, accel: int = ACCEL_AUTO) -> Tracer:
    """Tracer configured and initialized for a scenes.Scene."""
    t = Tracer(device, scene.num_rays if num_rays is None else num_rays)
    t.set_accel(accel)
    t.set_elements(scene.elements)
    t.set_sun_vector(scene.sun_dir)
    t.set_sun_shape(scene.sun_shape, scene.sun_param)
    t.set_seed(seed, instance)
    t.set_record_ids(record_ids)
    t.initialize()
    return t
