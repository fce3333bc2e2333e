"""The reference's C++ API (drop-in headers + libcsp_gb300.so): a demo compiles and links without a
GPU; on the GPU its records and CSV equal the oracle's trace of the same scene."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from optixsoltracedemos_gb300 import scenes
from tests.test_io import _write_stinput, reference_csv_rows

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "optixsoltracedemos_gb300")


def compile_demo(out_dir):
    from optixsoltracedemos_gb300 import build
    lib = build.build()
    exe = os.path.join(out_dir, "demo_heliostats")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(PKG, "cpp", "include"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "demo_heliostats.cpp"), "-o", exe, "-L", os.path.dirname(lib),
           "-lcsp_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True)
    return exe


def test_demo_compiles_against_dropin_headers(native_lib, tmp_path):
    exe = compile_demo(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_demo_runs_and_matches_oracle(gpu, oracle32, tmp_path):
    exe = compile_demo(str(tmp_path))
    n = 50000
    csv, raw = str(tmp_path / "out.csv"), str(tmp_path / "out.raw")
    subprocess.run([exe, csv, raw, str(n)], check=True, timeout=300)
    hits = np.fromfile(raw, np.float32).reshape(n, 5, 4)
    el = np.fromfile(raw + ".elements", scenes.ELEMENT_DTYPE)
    assert len(el) == 4 and np.all(el["reflectivity"] == 1.0)
    oh, _ = oracle32.trace(el, np.array([0.0, -1.0, 1.0]), 0, 4.65e-3, count=n)
    np.testing.assert_array_equal(hits, oh.astype(np.float32))
    lines = open(csv).read().splitlines()
    assert lines[0] == "number,stage,loc_x,loc_y,loc_z"
    assert lines[1:] == reference_csv_rows(oh.astype(np.float32))


@pytest.mark.gpu
def test_demo_stinput_and_facade(gpu, oracle32, tmp_path):
    exe = compile_demo(str(tmp_path))
    sc = scenes.single_parabolic(sun_shape=scenes.SUN_PILLBOX, sun_sigma=4.65e-3, slope_error=0.0)
    st = str(tmp_path / "scene.stinput")
    _write_stinput(st, sc.elements, sc.sun_dir, 4.65)
    n = 20000
    csv, raw = str(tmp_path / "out.csv"), str(tmp_path / "out.raw")
    subprocess.run([exe, csv, raw, str(n), st], check=True, timeout=300)
    hits = np.fromfile(raw, np.float32).reshape(n, 5, 4)
    from optixsoltracedemos_gb300 import native
    _, sun, ang = native.parse_stinput(st)
    el = np.fromfile(raw + ".elements", scenes.ELEMENT_DTYPE)
    oh, _ = oracle32.trace(el, sun, 0, ang, count=n)
    np.testing.assert_array_equal(hits, oh.astype(np.float32))
    facade = open(csv + ".facade.csv").read().splitlines()
    oh1000, _ = oracle32.trace(el, sun, 0, ang, count=1000)
    assert facade[1:] == reference_csv_rows(oh1000.astype(np.float32))
