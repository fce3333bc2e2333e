"""The C-ABI library builds, loads without a GPU and exports exactly what include/*.h declares."""
import ctypes
import glob
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        for m in re.finditer(r"CSP_API\s+[^;(]*?\b(csp_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"csp_create", "csp_destroy", "csp_initialize", "csp_run", "csp_copy_hits"} <= names


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(native_lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(native_lib):
    from optixsoltracedemos_gb300 import native
    assert declared_symbols() == set(native.SIGNATURES)


def test_element_struct_layout_matches_header():
    from optixsoltracedemos_gb300.scenes import ELEMENT_DTYPE

    class CElement(ctypes.Structure):
        _fields_ = [("origin", ctypes.c_double * 3), ("aim_point", ctypes.c_double * 3), ("zrot_deg", ctypes.c_double),
                    ("width", ctypes.c_double), ("height", ctypes.c_double), ("curv_x", ctypes.c_double),
                    ("curv_y", ctypes.c_double), ("reflectivity", ctypes.c_double), ("slope_error", ctypes.c_double),
                    ("specularity_error", ctypes.c_double), ("surface", ctypes.c_int32), ("aperture", ctypes.c_int32)]

    assert ctypes.sizeof(CElement) == ELEMENT_DTYPE.itemsize
    for name, _ in CElement._fields_:
        assert getattr(CElement, name).offset == ELEMENT_DTYPE.fields[name][1]


def test_abi_version_and_errors_without_gpu(native_lib):
    assert native_lib.csp_abi_version() == 1
    # argument errors are reported without touching CUDA
    from optixsoltracedemos_gb300 import native
    assert native_lib.csp_destroy(None) == -1
    assert b"null handle" in native_lib.csp_last_error()
    assert native_lib.csp_create(None, 0, 10) == -1
    _ = native, np
