"""Error paths and persistence on the GPU.

  * Allocation failures, injected on the host (csp_debug_fail_allocation makes one device or
    pinned-host allocation of the library report out-of-memory): csp_initialize, csp_batch_run and a
    served request fail with CSP_ERR_OUT_OF_MEMORY, and the same handle then works and gives the
    oracle's / the plain path's results.  No GPU fault is involved: the failing call never reaches
    the driver.
  * The batched autotuner's persistent cache: a run writes its tuning to the file, and another
    process reading the file uses it without tuning again.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from optixsoltracedemos_gb300 import scenes

pytestmark = pytest.mark.gpu

OOM = -3
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_initialize_out_of_memory_then_usable(gpu, oracle32):
    from optixsoltracedemos_gb300 import native
    field = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(40.0, 30.0))
    n = 20000
    oh, oi = oracle32.trace(field.elements, field.sun_dir, field.sun_shape, field.sun_param, count=n, seed=3)
    failures = 0
    for k in range(64):
        t = native.Tracer(0, n)
        try:
            t.set_elements(field.elements)
            t.set_sun_vector(field.sun_dir)
            t.set_sun_shape(field.sun_shape, field.sun_param)
            t.set_seed(3)
            t.set_record_ids(True)
            native.debug_fail_allocation(k)
            try:
                t.initialize()
                injected = False
            except native.CspError as e:
                assert e.status == OOM, str(e)
                injected = True
                failures += 1
            native.debug_fail_allocation(-1)
            if injected:
                t.initialize()  # the same handle, now with memory
            t.run()
            hits, ids = t.copy_hits()
            assert np.array_equal(ids, oi) and np.array_equal(hits, oh.astype(np.float32)), f"after failure {k}"
        finally:
            native.debug_fail_allocation(-1)
            t.close()
        if not injected:
            break  # k is past the last allocation of initialize
    assert failures >= 5  # every allocation of the set-up was exercised


def test_batch_run_out_of_memory_then_usable(gpu, oracle32):
    from optixsoltracedemos_gb300 import native
    field = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(40.0, 30.0), num_rays=1)
    suns = [scenes.sun_vector(40.0, 30.0), scenes.sun_vector(25.0, -60.0)]
    poses = [scenes.reaim(field.elements, s) for s in suns]
    tgt = native.flux_target(field.elements[-1])
    ref = []
    for i, s in enumerate(suns):
        oh, _ = oracle32.trace(poses[i], s, scenes.SUN_PILLBOX, 4.65e-3, count=40000, seed=i, instance=i)
        ref.append(oracle32.flux_counts(oh.astype(np.float32), tgt)[0])
    # a fresh batch's first run allocates its arena, then its staging and result buffers: each of the
    # three fails in turn
    for k in (0, 1, 2):
        b = native.Batch(0)
        try:
            sid = b.add_scene(field.elements)
            for i, s in enumerate(suns):
                b.add_instance(sid, s, scenes.SUN_PILLBOX, 4.65e-3, 40000, seed=i, instance=i, poses=poses[i])
            b.set_tuning(128, 0, 4)
            native.debug_fail_allocation(k)
            with pytest.raises(native.CspError) as e:
                b.run()
            assert e.value.status == OOM, k
            native.debug_fail_allocation(-1)
            b.run()  # the same batch, now with memory
            for i in range(len(suns)):
                np.testing.assert_array_equal(b.counts(i), ref[i])
        finally:
            native.debug_fail_allocation(-1)
            b.close()


def test_served_request_out_of_memory_then_usable(gpu, oracle32):
    from optixsoltracedemos_gb300 import native
    sc = scenes.three_heliostats()
    srv = native.Server(0, memory_budget=64 << 20, max_active=4)
    try:
        sid = srv.add_scene(sc.elements)
        # the next allocation is the first admission's pinned staging
        native.debug_fail_allocation(0)
        rid = srv.submit(sid, sc.sun_dir, sc.sun_shape, sc.sun_param, 50000, seed=2, instance=1)
        with pytest.raises(native.CspError) as e:
            srv.wait(rid, timeout=60.0)
        assert e.value.status == OOM
        native.debug_fail_allocation(-1)
        rid = srv.submit(sid, sc.sun_dir, sc.sun_shape, sc.sun_param, 50000, seed=2, instance=1)
        counts, _, _ = srv.wait(rid, timeout=60.0)
        oh, _ = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=50000, seed=2, instance=1)
        oc, _ = oracle32.flux_counts(oh.astype(np.float32), native.flux_target(sc.elements[-1]))
        np.testing.assert_array_equal(counts, oc)
    finally:
        native.debug_fail_allocation(-1)
        srv.close()


_TUNE_RUN = """
import sys, numpy as np
sys.path.insert(0, {root!r})
from optixsoltracedemos_gb300 import native, scenes
native.set_tune_cache({path!r})
field = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(40.0, 30.0), num_rays=1)
b = native.Batch(0)
sid = b.add_scene(field.elements)
for i in range(2):
    b.add_instance(sid, scenes.sun_vector(40.0 - 10 * i, 30.0), scenes.SUN_PILLBOX, 4.65e-3, 1 << 20, seed=i,
                   instance=i)
b.run()
print("TUNING", *b.tuning(native.GROUP_GRID))
b.close()
"""


def test_tune_cache_persists_across_processes(gpu, tmp_path):
    path = str(tmp_path / "tune.json")
    code = _TUNE_RUN.format(root=ROOT, path=path)
    r1 = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r1.returncode == 0, r1.stderr[-2000:]
    tuned = [ln for ln in r1.stdout.splitlines() if ln.startswith("TUNING")][0].split()[1:]
    text = open(path).read()
    assert '"group": 2' in text
    assert f'"block": {tuned[0]}, "ctas_per_sm": {tuned[1]}, "chunk": {tuned[2]}' in text
    mtime = os.path.getmtime(path)
    r2 = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r2.returncode == 0, r2.stderr[-2000:]
    again = [ln for ln in r2.stdout.splitlines() if ln.startswith("TUNING")][0].split()[1:]
    assert again == tuned
    assert os.path.getmtime(path) == mtime  # the second process tuned nothing (no rewrite)
