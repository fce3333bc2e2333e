"""Host-side auxiliaries that need no GPU: the autotuner's persistent cache file and the switches
of the allocation-failure injection and the bounds-check status."""
import json

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
