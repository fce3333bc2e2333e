"""The reference's own demo programs against the drop-in C++ API.

Where CSP_REFERENCE_DIR names the reference checkout, its three built demos (demos/CMakeLists.txt:
demo_three_heliostats, demo_large_scene, demo_dynamic_scene) compile unchanged against the drop-in
headers and link against libcsp_gb300.so; the only header supplied besides the drop-in is an empty
stand-in for the OptiX SDK's optix_function_table_definition.h, which the demos include and the
drop-in does not need.  No GPU is needed for that.

On the GPU, the frame loop of demos/demo_dynamic_scene.cpp:82-97 -- run, write_output, move the sun,
update -- runs through the drop-in (tests/cpp/demo_frames.cpp, the project's program with the demo's
scene) and every frame's CSV equals the oracle's trace of that frame's sun.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from optixsoltracedemos_gb300 import scenes
from tests.test_io import reference_csv_rows

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "optixsoltracedemos_gb300")
REF = os.environ.get("CSP_REFERENCE_DIR", "")
REF_DEMOS = ["demo_three_heliostats", "demo_large_scene", "demo_dynamic_scene"]


def _compile(src, exe, extra_inc=()):
    from optixsoltracedemos_gb300 import build
    lib = build.build()
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2"]
    for inc in extra_inc:
        cmd += ["-I", inc]
    cmd += ["-I", os.path.join(PKG, "cpp", "include"), "-I", os.path.join(ROOT, "include"), src, "-o", exe,
            "-L", os.path.dirname(lib), "-lcsp_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "demos")),
                    reason="CSP_REFERENCE_DIR does not name the reference checkout")
@pytest.mark.parametrize("demo", REF_DEMOS)
def test_reference_demo_compiles_unchanged(native_lib, tmp_path, demo):
    stub = tmp_path / "stub"
    stub.mkdir()
    (stub / "optix_function_table_definition.h").write_text("/* the drop-in needs no OptiX function table */\n")
    exe = _compile(os.path.join(REF, "demos", demo + ".cpp"), str(tmp_path / demo), extra_inc=[str(stub)])
    assert os.path.exists(exe)


def test_frame_loop_program_compiles(native_lib, tmp_path):
    exe = _compile(os.path.join(ROOT, "tests", "cpp", "demo_frames.cpp"), str(tmp_path / "demo_frames"))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_dynamic_frame_loop_matches_oracle(gpu, oracle32, tmp_path):
    """Five frames of 20,000 rays: after each run the CSV is written, the sun vector's y grows by 1
    and update() re-computes the sun plane; every frame's CSV equals the reference CSV format of the
    oracle's trace with that frame's sun (collimated: sun angle 0)."""
    exe = _compile(os.path.join(ROOT, "tests", "cpp", "demo_frames.cpp"), str(tmp_path / "demo_frames"))
    n, frames = 20000, 5
    prefix = str(tmp_path / "frame")
    subprocess.run([exe, prefix, str(n), str(frames)], check=True, timeout=300)
    el = np.fromfile(prefix + ".elements", scenes.ELEMENT_DTYPE)
    assert len(el) == 2 and int(el["surface"][0]) == scenes.SURFACE_PARABOLIC
    stages = set()
    for f in range(frames):
        sun = np.array([0.0, -20.0 + f, 100.0])
        oh, _ = oracle32.trace(el, sun, 0, 0.0, count=n)
        rows = open(f"{prefix}_{f}.csv").read().splitlines()
        assert rows[0] == "number,stage,loc_x,loc_y,loc_z"
        assert rows[1:] == reference_csv_rows(oh.astype(np.float32)), f"frame {f}"
        stages |= set(np.unique(oh[:, :, 0]).tolist())
    assert {1.0, 2.0} <= stages
