"""The CSV of compact records (csp_write_compact_csv) is the CSV of the dense records
(csp_write_hits_csv, the reference's write_output format), on records of the oracle's trace."""
import numpy as np
import pytest

from optixsoltracedemos_gb300 import native, scenes


def to_compact(hits):
    """Dense [N, 5, 4] rows -> (points [N, 3], counts [N], records [R, 4]) as the device compaction
    makes them: slot 0's point, then the slots after it whose stage is not 0."""
    points = hits[:, 0, 1:].copy()
    present = hits[:, 1:, 0] != 0
    counts = present.sum(axis=1).astype(np.uint8)
    records = hits[:, 1:][present]
    return points, counts, records


@pytest.mark.parametrize("name,staged", [("three_heliostats", False), ("three_heliostats", True),
                                         ("corridor", False), ("single_parabolic", True)])
def test_compact_csv_equals_dense_csv(native_lib, oracle32, tmp_path, name, staged):
    sc = getattr(scenes, name)(num_rays=40000)
    hits, _ = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=40000, seed=3)
    hits = hits.astype(np.float32)
    points, counts, records = to_compact(hits)
    assert counts.max() >= 1
    dense_csv, compact_csv = tmp_path / "dense.csv", tmp_path / "compact.csv"
    native.write_hits_csv(hits, str(dense_csv), staged=staged)
    native.write_compact_csv(points, counts, records, str(compact_csv), staged=staged)
    assert compact_csv.read_bytes() == dense_csv.read_bytes()


def test_compact_csv_rejects_bad_counts(native_lib, tmp_path):
    points = np.zeros((2, 3), np.float32)
    counts = np.array([1, 7], np.uint8)
    records = np.zeros((8, 4), np.float32)
    with pytest.raises(native.CspError) as e:
        native.write_compact_csv(points, counts, records, str(tmp_path / "x.csv"))
    assert e.value.status == -1


def _synthetic_hits(n, seed=11):
    """[n, 5, 4] records shaped like a trace's: every ray a sun-plane point, some rays 1 to 4 more
    records, the rest of each row zero (the writer's ray-end markers)."""
    rs = np.random.default_rng(seed)
    hits = np.zeros((n, 5, 4), np.float32)
    hits[:, 0, 1:] = rs.uniform(-900.0, 900.0, (n, 3))
    extra = rs.choice([0, 0, 0, 0, 0, 0, 1, 2, 3, 4], n)
    for s in range(1, 5):
        m = extra >= s
        hits[m, s, 0] = np.where(s == extra[m], 2.0, 1.0)
        hits[m, s, 1:] = rs.uniform(-50.0, 250.0, (int(m.sum()), 3))
    return hits


def test_writers_agree_across_pipelined_batches(native_lib, tmp_path):
    """4.5M rays: several pipelined batches of either writer (dense blocks of 2^18 rays and compact
    blocks of 2^16, one per host thread per batch) give the same file."""
    hits = _synthetic_hits(4_500_000)
    points, counts, records = to_compact(hits)
    dense_csv, compact_csv = tmp_path / "dense.csv", tmp_path / "compact.csv"
    native.write_hits_csv(hits, str(dense_csv))
    native.write_compact_csv(points, counts, records, str(compact_csv))
    assert compact_csv.stat().st_size == dense_csv.stat().st_size
    assert compact_csv.read_bytes() == dense_csv.read_bytes()
    with open(dense_csv, "rb") as f:
        lines = f.read().split(b"\n")
    # rows numbered by ray from 1, one per record (markers write nothing)
    assert lines[0] == b"number,stage,loc_x,loc_y,loc_z"
    assert len(lines) - 2 == int((hits[:, :, 1:] != 0).any(axis=2).sum())
    assert lines[-2].split(b",")[0] == str(hits.shape[0]).encode()


def test_writers_report_a_full_disk(native_lib):
    """A write that fails (/dev/full) is CSP_ERR_IO from either writer, with the formatting threads
    and the writer thread joined."""
    import os
    if not os.path.exists("/dev/full"):
        pytest.skip("no /dev/full")
    hits = _synthetic_hits(600_000, seed=12)
    points, counts, records = to_compact(hits)
    for fn in (lambda: native.write_hits_csv(hits, "/dev/full"),
               lambda: native.write_compact_csv(points, counts, records, "/dev/full")):
        with pytest.raises(native.CspError) as e:
            fn()
        assert e.value.status == -7  # CSP_ERR_IO
