"""Host-side auxiliaries that need no GPU: the autotuner's persistent cache file and the switches
of the allocation-failure injection and the bounds-check status, and the element records built in
ranges on several threads."""
import json
import os

import pytest

from optixsoltracedemos_gb300 import native


def test_tune_cache_file_read_and_malformed_entries_skipped(native_lib, tmp_path):
    path = tmp_path / "tune.json"
    path.write_text(
        '{"format": "csp_gb300 batch tuning cache", "version": 1, "entries": [\n'
        '  {"device": "test device cc0.0 sm1", "build": 7, "group": 2, "ray_class": 10, "block": 256, '
        '"ctas_per_sm": 4, "chunk": 16},\n'
        '  {"device": "test device cc0.0 sm1", "build": 7, "group": 0, "ray_class": 10, "block": 128, '
        '"ctas_per_sm": 9, "chunk": 4},\n'
        '  {"device": "test device cc0.0 sm1", "build": 7, "group": 2, "ray_class": 11, "block": 96, '
        '"ctas_per_sm": 4, "chunk": 16},\n'
        '  {"device": "test device cc0.0 sm1", "group": 1}\n'
        ']}\n')
    try:
        before = native.set_tune_cache(None)
        after = native.set_tune_cache(str(path))
        # the two well-formed entries; a block size the kernels do not have and a line without its
        # fields are skipped
        assert after == before + 2
        # reading the same file again adds nothing
        assert native.set_tune_cache(str(path)) == after
        json.loads(path.read_text())  # the format is JSON
    finally:
        native.set_tune_cache(None)


def test_tune_cache_missing_file_is_empty(native_lib, tmp_path):
    try:
        before = native.set_tune_cache(None)
        assert native.set_tune_cache(str(tmp_path / "absent.json")) == before
    finally:
        native.set_tune_cache(None)


def test_fail_allocation_argument_checked(native_lib):
    with pytest.raises(native.CspError) as e:
        native.debug_fail_allocation(-2)
    assert e.value.status == -1
    native.debug_fail_allocation(-1)  # cancelling with nothing pending is fine


def test_bounds_check_status_in_a_normal_build(native_lib):
    # the in-tree library is built without the checks
    with pytest.raises(native.CspError) as e:
        native.bounds_check_status(0)
    assert e.value.status == -6


def test_element_records_built_in_ranges_equal_serial(tmp_path):
    """The server builds the element records of large submissions in ranges on its host threads:
    the same records and the same error as the serial build (a host program compiled from the scene
    builder's source)."""
    import shutil
    import subprocess
    from optixsoltracedemos_gb300 import scenes
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    csrc = os.path.join(root, "optixsoltracedemos_gb300", "csrc")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    exe = str(tmp_path / "scene_build_ranges")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", "-I", csrc, "-I",
           os.path.join(root, "include"), "-I", cuda_inc, os.path.join(root, "tests", "cpp", "scene_build_ranges.cpp"),
           os.path.join(csrc, "csp_scene.cpp"), "-o", exe]
    subprocess.run(cmd, check=True)
    field = str(tmp_path / "field.bin")
    scenes.large_field(n_heliostats=10000, num_rays=1).elements.tofile(field)
    r = subprocess.run([exe, field], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK 10001 elements, error 'element 1031:"), r.stdout
