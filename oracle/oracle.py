"""TEST INFRASTRUCTURE: ctypes access to the checkers built by oracle/Makefile.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, and only to
check or time the reference algorithm on the CPU.  The product package never imports it.

  Oracle(precision="f32")   C restatement of the reference's hot path (csp_oracle.c), float
  Oracle(precision="f64")   the same restatement in double (FP64 oracle for flux-map L2)
  RefHost()                 the reference's own device programs built on the host (_ref), when
                            the reference sources were present at build time
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

ELEMENT_DTYPE = np.dtype(
    [
        ("origin", "<f8", 3),
        ("aim_point", "<f8", 3),
        ("zrot_deg", "<f8"),
        ("width", "<f8"),
        ("height", "<f8"),
        ("curv_x", "<f8"),
        ("curv_y", "<f8"),
        ("reflectivity", "<f8"),
        ("slope_error", "<f8"),
        ("specularity_error", "<f8"),
        ("surface", "<i4"),
        ("aperture", "<i4"),
    ],
    align=True,
)
assert ELEMENT_DTYPE.itemsize == 120

MAX_DEPTH = 5


def reference_dir() -> str | None:
    """The reference checkout named by CSP_REFERENCE_DIR, or None when unset or absent."""
    d = os.environ.get("CSP_REFERENCE_DIR", "")
    return d if d and os.path.isdir(os.path.join(d, "cuda")) else None


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle libraries, and _ref (the reference's own programs on the host) when
    with_ref is True, or None and CSP_REFERENCE_DIR names the reference checkout."""
    ref_dir = reference_dir()
    if with_ref is None:
        with_ref = ref_dir is not None
    if with_ref and ref_dir is None:
        raise RuntimeError("building the reference host build needs CSP_REFERENCE_DIR=<reference checkout>")
    cmd = ["make", "-s", "-C", HERE, "ref" if with_ref else "all"]
    if with_ref:
        cmd.append(f"REF_DIR={ref_dir}")
    subprocess.run(cmd, check=True)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def as_elements(elements) -> np.ndarray:
    if isinstance(elements, np.ndarray) and elements.dtype == ELEMENT_DTYPE:
        return np.ascontiguousarray(elements)
    raise TypeError("elements must be a numpy array of ELEMENT_DTYPE")


class Oracle:
    def __init__(self, precision: str = "f32"):
        path = os.path.join(HERE, f"liboracle_{precision}.so")
        if not os.path.exists(path):
            build(with_ref=False)
        self.lib = ctypes.CDLL(path)
        self.precision = precision
        L = self.lib
        L.orc_trace.restype = ctypes.c_int
        L.orc_trace.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_scene_info.restype = ctypes.c_int
        L.orc_scene_info.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_philox.argtypes = [ctypes.c_void_p] * 3
        for f in ("orc_sincos_batch", "orc_sincos2pi_batch"):
            getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_log_batch.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.orc_atan2_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.orc_flux_counts.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_void_p]

    def trace(self, elements, sun_dir, sun_shape=0, sun_param=0.0, first_ray=0, count=1000, seed=0,
              instance=0, max_depth=MAX_DEPTH, nthreads=0, with_ids=True):
        el = as_elements(elements)
        sd = np.ascontiguousarray(sun_dir, dtype=np.float64)
        hits = np.zeros((count, max_depth, 4), np.float64)
        ids = np.zeros((count, max_depth), np.uint32) if with_ids else None
        rc = self.lib.orc_trace(_p(el), len(el), _p(sd), int(sun_shape), float(sun_param), int(first_ray), int(count),
                                int(seed), int(instance), int(max_depth), _p(hits),
                                _p(ids) if ids is not None else None, int(nthreads))
        if rc != 0:
            raise RuntimeError(self.lib.orc_last_error().decode())
        return hits, ids

    def scene_info(self, elements, sun_dir, sun_shape=0, sun_param=0.0):
        el = as_elements(elements)
        sd = np.ascontiguousarray(sun_dir, dtype=np.float64)
        prims = np.zeros((len(el), 32), np.float64)
        sun = np.zeros(32, np.float64)
        rc = self.lib.orc_scene_info(_p(el), len(el), _p(sd), int(sun_shape), float(sun_param), _p(prims), _p(sun))
        if rc != 0:
            raise RuntimeError(self.lib.orc_last_error().decode())
        return prims, sun

    def philox(self, ctr, key):
        c = np.ascontiguousarray(ctr, np.uint32)
        k = np.ascontiguousarray(key, np.uint32)
        o = np.zeros(4, np.uint32)
        self.lib.orc_philox(_p(c), _p(k), _p(o))
        return o

    def sincos(self, x):
        x = np.ascontiguousarray(x, np.float32)
        s = np.empty_like(x)
        c = np.empty_like(x)
        self.lib.orc_sincos_batch(_p(x), x.size, _p(s), _p(c))
        return s, c

    def sincos2pi(self, u):
        u = np.ascontiguousarray(u, np.float32)
        s = np.empty_like(u)
        c = np.empty_like(u)
        self.lib.orc_sincos2pi_batch(_p(u), u.size, _p(s), _p(c))
        return s, c

    def log(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty_like(x)
        self.lib.orc_log_batch(_p(x), x.size, _p(y))
        return y

    def atan2(self, y, x):
        y = np.ascontiguousarray(y, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty_like(y)
        self.lib.orc_atan2_batch(_p(y), _p(x), y.size, _p(out))
        return out

    def flux_counts(self, hits, target, nx=100, ny=100):
        """(counts [nx, ny] uint32, stats [4] uint64) of float records [..., 4] for the receiver
        parameters `target` (20 floats, as csp_flux_target returns them)."""
        rec = np.ascontiguousarray(np.asarray(hits).reshape(-1, 4), np.float32)
        t = np.ascontiguousarray(target, np.float32)
        counts = np.zeros((nx, ny), np.uint32)
        stats = np.zeros(4, np.uint64)
        self.lib.orc_flux_counts(_p(rec), rec.shape[0], _p(t), int(nx), int(ny), _p(counts), _p(stats))
        return counts, stats


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libref_host.so"))


class RefHost:
    """The reference's own programs built on the host (pillbox sun, no optical errors)."""

    def __init__(self):
        path = os.path.join(HERE, "_ref", "libref_host.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ref_trace.restype = ctypes.c_int
        L.ref_trace.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64,
                                ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_int]
        L.ref_scene_info.restype = ctypes.c_int
        L.ref_scene_info.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_double,
                                     ctypes.c_void_p, ctypes.c_void_p]
        L.ref_last_error.restype = ctypes.c_char_p

    def trace(self, elements, sun_dir, sun_angle, first_ray=0, count=1000, seed=0, instance=0, nthreads=0):
        el = as_elements(elements)
        sd = np.ascontiguousarray(sun_dir, dtype=np.float64)
        hits = np.zeros((count, MAX_DEPTH, 4), np.float64)
        ids = np.zeros((count, MAX_DEPTH), np.uint32)
        rc = self.lib.ref_trace(_p(el), len(el), _p(sd), float(sun_angle), int(first_ray), int(count), int(seed),
                                int(instance), _p(hits), _p(ids), int(nthreads))
        if rc != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return hits, ids

    def scene_info(self, elements, sun_dir, sun_angle):
        el = as_elements(elements)
        sd = np.ascontiguousarray(sun_dir, dtype=np.float64)
        prims = np.zeros((len(el), 32), np.float64)
        sun = np.zeros(32, np.float64)
        rc = self.lib.ref_scene_info(_p(el), len(el), _p(sd), float(sun_angle), _p(prims), _p(sun))
        if rc != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return prims, sun
