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
