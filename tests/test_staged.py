"""Staged results (SolTrace's stage order, scripts/post_processing/clean_direct_sun.py:6-18): rays
whose first interaction is the receiver -- straight from the sun -- are left out of the CSV and of
the flux maps.

CPU: on the oracle's records of the parabolic scene (its cylinder receiver is lit directly by the
sun), the staged CSV writer equals the plain CSV after `clean_receiver_direct_sun_hits`, byte for
byte, and the ray numbers it keeps are those of the script's group rule (a number is kept if its
rows include stage 1 or exclude stage 2), restated here from the records.
GPU: staged device flux maps equal the oracle's binning of the kept rays; the staged write_output
equals the cleaned plain one; staged batch and served flux maps equal staged plain ones.
"""
import os

import numpy as np
import pytest

from optixsoltracedemos_gb300 import native, post, scenes


def _records(oracle32, sc, n, seed=0):
    hits, ids = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, seed=seed, nthreads=0)
    return hits.astype(np.float32), ids


def test_staged_csv_equals_cleaned_csv(tmp_path, oracle32):
    sc = scenes.single_parabolic()
    hits, _ = _records(oracle32, sc, 60000)
    direct = post.direct_sun_rays(hits)
    assert direct.sum() > 100 and (hits[:, 1, 0] == 1).sum() > 100  # both kinds present
    plain, staged, cleaned = (str(tmp_path / f) for f in ("plain.csv", "staged.csv", "cleaned.csv"))
    native.write_hits_csv(hits, plain)
    native.write_hits_csv(hits, staged, staged=True)
    post.clean_receiver_direct_sun_hits(plain, cleaned)
    assert open(staged, "rb").read() == open(cleaned, "rb").read()
    # the script's group rule, restated from the records: ray r is number r + 1 (every ray has its
    # stage-0 row); keep it if any record has stage 1 or none has stage 2
    stages = hits[:, :, 0]
    keep = (stages == 1).any(axis=1) | ~(stages == 2).any(axis=1)
    nums = np.loadtxt(staged, delimiter=",", skiprows=1, usecols=0, dtype=np.int64)
    np.testing.assert_array_equal(np.unique(nums), np.nonzero(keep)[0] + 1)
    np.testing.assert_array_equal(keep, ~direct)
    assert os.path.getsize(staged) < os.path.getsize(plain)


def test_clean_csv_group_rule(tmp_path):
    """Hand-made file: ray numbers with stages {0}, {0,1}, {0,1,2}, {0,2}, {0,1,1,2}, {2} (no stage 0)
    and {0,1,1}; the script's rule keeps a number with a stage-1 row or without a stage-2 row, so
    numbers 4 and 6 go; kept rows are copied byte for byte."""
    rows = {1: [0], 2: [0, 1], 3: [0, 1, 2], 4: [0, 2], 5: [0, 1, 1, 2], 6: [2], 7: [0, 1, 1]}
    lines = ["number,stage,loc_x,loc_y,loc_z\n"]
    for num, stages in rows.items():
        for k, st in enumerate(stages):
            lines.append(f"{num},{st},{k}.5,-{num}e-05,{num * 10 + k}\n")
    src, dst = str(tmp_path / "in.csv"), str(tmp_path / "out.csv")
    open(src, "w").write("".join(lines))
    post.clean_receiver_direct_sun_hits(src, dst)
    want = [lines[0]] + [l for l in lines[1:] if int(l.split(",")[0]) not in (4, 6)]
    assert open(dst).read() == "".join(want)


def test_staged_flag_validation(tmp_path):
    hits = np.zeros((1, 5, 4), np.float32)
    rc = native.load().csp_write_hits_csv_ex(hits.ctypes.data, 1, str(tmp_path / "x.csv").encode(), 2)
    assert rc != 0  # unknown flag
    assert native.load().csp_write_hits_csv_ex(hits.ctypes.data, 1, str(tmp_path / "x.csv").encode(), 1) == 0


@pytest.mark.gpu
def test_staged_device_outputs(gpu, oracle32, tmp_path):
    sc = scenes.single_parabolic()
    n = 200000
    t = native.tracer_for(sc, seed=3, num_rays=n)
    try:
        t.run()
        hits, _ = t.copy_hits(0, n)
        oh, _ = _records(oracle32, sc, n, seed=3)
        np.testing.assert_array_equal(hits, oh)
        target = native.flux_target(sc.elements[-1])
        kept = oh[~post.direct_sun_rays(oh)]
        want_staged, _ = oracle32.flux_counts(kept, target)
        want_plain, _ = oracle32.flux_counts(oh, target)
        got_staged, _ = t.flux_map(staged=True)
        got_plain, _ = t.flux_map()
        np.testing.assert_array_equal(got_staged, want_staged)
        np.testing.assert_array_equal(got_plain, want_plain)
        assert got_staged.sum() < got_plain.sum()
        plain, staged, cleaned = (str(tmp_path / f) for f in ("plain.csv", "staged.csv", "cleaned.csv"))
        t.write_output(plain)
        t.write_output(staged, staged=True)
        post.clean_receiver_direct_sun_hits(plain, cleaned)
        assert open(staged, "rb").read() == open(cleaned, "rb").read()
    finally:
        t.close()
    # batch instances with staged flux maps equal staged plain runs
    b = native.Batch(0)
    try:
        sid = b.add_scene(sc.elements)
        b.add_instance(sid, sc.sun_dir, sc.sun_shape, sc.sun_param, n, seed=3, instance=0)
        b.add_instance(sid, sc.sun_dir, sc.sun_shape, sc.sun_param, 90001, seed=8, instance=4)
        b.set_output(staged=True)
        b.run()
        np.testing.assert_array_equal(b.counts(0), want_staged)
        t2 = native.tracer_for(sc, seed=8, instance=4, num_rays=90001)
        try:
            t2.run()
            np.testing.assert_array_equal(b.counts(1), t2.flux_map(staged=True)[0])
        finally:
            t2.close()
        b.set_output(staged=False)
        b.run()
        np.testing.assert_array_equal(b.counts(0), want_plain)
    finally:
        b.close()
    # served requests: the setting at submission applies
    srv = native.Server(0, memory_budget=1 << 30, max_active=8)
    try:
        sid = srv.add_scene(sc.elements)
        srv.set_output(staged=True)
        a = srv.submit(sid, sc.sun_dir, sc.sun_shape, sc.sun_param, n, seed=3, instance=0)
        srv.set_output(staged=False)
        c = srv.submit(sid, sc.sun_dir, sc.sun_shape, sc.sun_param, n, seed=3, instance=0)
        np.testing.assert_array_equal(srv.wait(a)[0], want_staged)
        np.testing.assert_array_equal(srv.wait(c)[0], want_plain)
    finally:
        srv.close()


@pytest.mark.gpu
def test_compact_transfer_matches_dense(gpu, tmp_path):
    """csp_run_to_host_compact moves the same records as the dense copy (points, counts and records
    expand back to the dense rows, bit for bit), fewer bytes, and its CSV is the dense CSV."""
    from optixsoltracedemos_gb300 import native
    from tests.test_compact_cpu import to_compact
    for sc in (scenes.three_heliostats(num_rays=300000),
               scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(35.0, 20.0), num_rays=200000)):
        t = native.tracer_for(sc, device=0, seed=4, record_ids=False)
        try:
            dense = np.zeros((sc.num_rays, 5, 4), np.float32)
            t.run_to_host(dense.reshape(-1))
            points, counts, records = t.run_to_host_compact()
        finally:
            t.close()
        p2, c2, r2 = to_compact(dense)
        assert np.array_equal(points, p2) and np.array_equal(counts, c2) and np.array_equal(records, r2)
        assert records.shape[0] > 0
        # compact bytes: 13 per ray + 16 per record, against 80 per ray
        assert 13 * sc.num_rays + 16 * records.shape[0] < 0.5 * 80 * sc.num_rays
        a, b = tmp_path / "dense.csv", tmp_path / "compact.csv"
        native.write_hits_csv(dense, str(a))
        native.write_compact_csv(points, counts, records, str(b))
        assert a.read_bytes() == b.read_bytes()
