"""The bounds-check build (-DCSP_BOUNDS_CHECK) on small cases of every launch kind.

The library is built a second time with the index checks on (queue appends, record rows, flux
bins, field-grid and sun-grid cells, sun-grid build, Halton table); a failed check sets a bit of a
device word and skips its access, so an out-of-range index can neither fault nor hang.  A child
process loads that build (CSP_NATIVE_LIB) and runs the element-list, field-grid and BVH traces, a
two-instance batch and a served request on small cases: every result equals the oracle and no check
fails.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
from optixsoltracedemos_gb300 import native, scenes
from oracle import oracle
lib = native.load()
assert native.LIB_PATH not in str(lib._name), lib._name
o32 = oracle.Oracle("f32")
assert native.bounds_check_status(0) == 0

def plain(sc, n, seed, accel=native.ACCEL_AUTO):
    t = native.Tracer(0, n)
    t.set_elements(sc.elements); t.set_sun_vector(sc.sun_dir); t.set_sun_shape(sc.sun_shape, sc.sun_param)
    t.set_seed(seed); t.set_record_ids(True); t.set_accel(accel); t.initialize(); t.run()
    h, i = t.copy_hits(); t.close()
    oh, oi = o32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, seed=seed)
    assert np.array_equal(i, oi) and np.array_equal(h, oh.astype(np.float32)), sc.name

plain(scenes.three_heliostats(), 1 << 16, 1)
field = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(35.0, 20.0))
plain(field, 20000, 2)
plain(field, 20000, 2, native.ACCEL_BVH)
b = native.Batch(0)
s0 = b.add_scene(scenes.three_heliostats().elements)
s1 = b.add_scene(field.elements)
jobs = [(s0, scenes.three_heliostats().elements, scenes.three_heliostats().sun_dir),
        (s1, field.elements, scenes.sun_vector(50.0, -40.0))]
for i, (sid, el, sun) in enumerate(jobs):
    b.add_instance(sid, sun, scenes.SUN_PILLBOX, 4.65e-3, 30000, seed=i, instance=i, poses=scenes.reaim(el, sun))
b.set_tuning(128, 0, 4)
b.run()
for i, (sid, el, sun) in enumerate(jobs):
    p = scenes.reaim(el, sun)
    oh, _ = o32.trace(p, sun, scenes.SUN_PILLBOX, 4.65e-3, count=30000, seed=i, instance=i)
    oc, _ = o32.flux_counts(oh.astype(np.float32), native.flux_target(p[-1]))
    assert np.array_equal(b.counts(i), oc), i
b.close()
srv = native.Server(0, memory_budget=256 << 20, max_active=4)
sid = srv.add_scene(field.elements)
sun = scenes.sun_vector(60.0, 10.0)
p = scenes.reaim(field.elements, sun)
c, _, _ = srv.wait(srv.submit(sid, sun, scenes.SUN_PILLBOX, 4.65e-3, 30000, seed=5, instance=3, poses=p), 120.0)
oh, _ = o32.trace(p, sun, scenes.SUN_PILLBOX, 4.65e-3, count=30000, seed=5, instance=3)
oc, _ = o32.flux_counts(oh.astype(np.float32), native.flux_target(p[-1]))
assert np.array_equal(c, oc)
srv.close()
print("SITES", native.bounds_check_status(0))
"""


def test_bounds_checked_build_small_cases(gpu):
    from optixsoltracedemos_gb300 import build
    from oracle import oracle
    oracle.build(with_ref=None)
    lib = build.build(bounds_check=True)
    env = dict(os.environ, CSP_NATIVE_LIB=lib)
    r = subprocess.run([sys.executable, "-c", _CHILD.format(root=ROOT)], capture_output=True, text=True, timeout=900,
                       env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    sites = [ln for ln in r.stdout.splitlines() if ln.startswith("SITES")]
    assert sites == ["SITES 0"], r.stdout[-2000:]
