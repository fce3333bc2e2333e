"""Device flux maps and batched tracing on the GPU.

  * csp_flux_map (device binning of the dense hit buffer) equals the oracle's binning of the same
    records, and of the oracle's own records, count for count;
  * every instance of a batch (one persistent launch, flux binned in the shading stage, per-instance
    BVH refit on the device) equals a plain single-scene run of the same scene, sun, rays, seed and
    instance id, count for count, whatever the launch parameters;
  * re-running a batch (CUDA graph replay) reproduces it, and a changed layout re-captures;
  * pipelined runs (run_async / wait, two in flight) give each run its own instances' results.
"""
import numpy as np
import pytest

from optixsoltracedemos_gb300 import scenes

pytestmark = pytest.mark.gpu


def _plain_counts(native, elements, sun, shape, param, rays, seed, instance, nx=100, ny=100):
    t = native.Tracer(0, rays)
    try:
        t.set_elements(elements)
        t.set_sun_vector(sun)
        t.set_sun_shape(shape, param)
        t.set_seed(seed, instance)
        t.initialize()
        t.run()
        counts, flux = t.flux_map(nx, ny)
        hits, _ = t.copy_hits()
        return counts, flux, hits
    finally:
        t.close()


@pytest.mark.parametrize("name,n", [("three_heliostats", 300000), ("single_parabolic", 300000),
                                    ("corridor", 100000)])
def test_flux_map_matches_oracle_binning(gpu, oracle32, name, n):
    from optixsoltracedemos_gb300 import native
    sc = getattr(scenes, name)(num_rays=n)
    counts, flux, hits = _plain_counts(native, sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, n, 5, 1)
    t = native.flux_target(sc.elements[-1])
    ref_counts, ref_stats = oracle32.flux_counts(hits, t)
    np.testing.assert_array_equal(counts, ref_counts)
    ohits, _ = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, 0, n, seed=5, instance=1)
    ocounts, _ = oracle32.flux_counts(ohits.astype(np.float32), t)
    np.testing.assert_array_equal(counts, ocounts)
    assert int(counts.sum()) == int(ref_stats[3])
    if name != "corridor":
        assert counts.sum() > 0
    # W/m^2 = counts * dni * sun-plane area / rays / bin area
    from optixsoltracedemos_gb300 import flux as fx
    t2 = native.Tracer(0, n)
    t2.set_elements(sc.elements)
    t2.set_sun_vector(sc.sun_dir)
    t2.set_sun_shape(sc.sun_shape, sc.sun_param)
    t2.initialize()
    area = fx.sun_plane_area(t2.sun_plane())
    t2.close()
    rcv = sc.elements[-1]
    w, h = float(rcv["width"]), float(rcv["height"])
    cyl = int(rcv["surface"]) == scenes.SURFACE_CYLINDER
    bin_area = (2 * np.pi * 0.5 * w / 100) * (h / 100) if cyl else (w / 100) * (h / 100)
    np.testing.assert_allclose(flux, counts * 1000.0 * area / n / bin_area, rtol=1e-12)


def _field(n_heliostats, sun):
    sc = scenes.large_field(n_heliostats=n_heliostats, sun=sun, num_rays=1)
    return sc.elements


def _mixed_batch(native):
    """Small-scene instances (3 heliostats, re-aimed per sun) and BVH instances (a 600-heliostat
    field re-aimed per sun), uneven ray counts, distinct seeds and instance ids."""
    b = native.Batch(0)
    th = scenes.three_heliostats()
    s_small = b.add_scene(th.elements)
    base = _field(600, scenes.sun_vector(45.0, 0.0))
    s_field = b.add_scene(base)
    jobs = []
    suns_small = [np.array([0.0, -1.0, 1.0]), np.array([0.3, -1.0, 1.2]), np.array([-0.2, -0.8, 1.0])]
    for k, sun in enumerate(suns_small):
        poses = th.elements.copy()
        poses["aim_point"][:3] = scenes.bisector_aim(poses["origin"][:3], sun, [0.0, 0.0, 10.0])
        rays = [70001, 131072, 5][k]
        jobs.append((s_small, poses, sun, scenes.SUN_PILLBOX, 4.65e-3, rays, 11 + k, k))
    for k, (el, az) in enumerate([(30.0, -60.0), (70.0, 100.0)]):
        sun = scenes.sun_vector(el, az)
        poses = scenes.reaim(base, sun)
        rays = [200000, 99999][k]
        jobs.append((s_field, poses, sun, scenes.SUN_PILLBOX, 4.65e-3, rays, 21 + k, 7 + k))
    # an instance with the scene's own poses and a Gaussian sun
    jobs.append((s_small, None, th.sun_dir, scenes.SUN_GAUSSIAN, 2.5e-3, 50000, 99, 3))
    for j in jobs:
        b.add_instance(j[0], j[2], j[3], j[4], j[5], seed=j[6], instance=j[7], poses=j[1])
    scene_el = {s_small: th.elements, s_field: base}
    return b, jobs, scene_el


def test_batch_instances_equal_plain_runs(gpu):
    from optixsoltracedemos_gb300 import native
    b, jobs, scene_el = _mixed_batch(native)
    try:
        b.run()
        for i, (sid, poses, sun, shape, param, rays, seed, inst) in enumerate(jobs):
            el = scene_el[sid] if poses is None else poses
            counts, flux, hits = _plain_counts(native, el, sun, shape, param, rays, seed, inst)
            np.testing.assert_array_equal(b.counts(i), counts, err_msg=f"instance {i}")
            np.testing.assert_allclose(b.flux(i), flux, rtol=1e-12, err_msg=f"instance {i}")
            st = b.stats(i)
            assert st[0] == rays
            assert st[1] == int((hits[..., 0] == 1.0).sum())
            assert st[2] == int((hits[..., 0] == 2.0).sum())
            assert st[3] == int(counts.sum())
        assert b.stats(1)[3] > 0 and b.stats(3)[3] > 0
    finally:
        b.close()


def test_batch_groups(gpu):
    """Field instances with their own poses (re-aimed, and one with a moved heliostat) run in the grid
    group, each with the grid of its poses; both equal plain runs."""
    from optixsoltracedemos_gb300 import native
    b = native.Batch(0)
    try:
        base = _field(800, scenes.sun_vector(45.0, 0.0))
        sid = b.add_scene(base)
        sun = scenes.sun_vector(20.0, 60.0)
        reaimed = scenes.reaim(base, sun)
        moved = reaimed.copy()
        moved["origin"][5] += [3.0, -2.0, 0.0]
        rays = 1990656 + 331776 + 999  # both coherent block sizes and a tail
        b.add_instance(sid, sun, scenes.SUN_PILLBOX, 4.65e-3, rays, seed=1, instance=1, poses=reaimed)
        b.add_instance(sid, sun, scenes.SUN_PILLBOX, 4.65e-3, 150000, seed=1, instance=1, poses=moved)
        b.run()
        assert b.tuning(native.GROUP_GRID)[0] in (128, 256)
        assert b.tuning(native.GROUP_BVH)[0] in (128, 256)
        for i, (poses, n) in enumerate(((reaimed, rays), (moved, 150000))):
            counts, _, _ = _plain_counts(native, poses, sun, scenes.SUN_PILLBOX, 4.65e-3, n, 1, 1)
            np.testing.assert_array_equal(b.counts(i), counts)
    finally:
        b.close()


def test_batch_independent_of_launch_parameters(gpu):
    from optixsoltracedemos_gb300 import native
    results = []
    for tune in [(128, 0, 1), (256, 0, 16), (128, 2, 3), (0, 0, 0)]:
        b, jobs, _ = _mixed_batch(native)
        try:
            b.set_tuning(*tune)
            b.run()
            results.append([b.counts(i).copy() for i in range(len(jobs))])
            groups = (native.GROUP_LIST, native.GROUP_GRID)
            for g in groups:
                assert b.tuning(g)[0] == (tune[0] if tune[0] else b.tuning(g)[0]) and b.tuning(g)[0] in (128, 256)
        finally:
            b.close()
    for r in results[1:]:
        for a, c in zip(results[0], r):
            np.testing.assert_array_equal(a, c)


def test_batch_rerun_and_relayout(gpu):
    from optixsoltracedemos_gb300 import native
    b, jobs, scene_el = _mixed_batch(native)
    try:
        b.run()
        first = [b.counts(i).copy() for i in range(len(jobs))]
        _, trace_s = b.timing()
        assert trace_s > 0
        b.run()  # graph replay
        for i in range(len(jobs)):
            np.testing.assert_array_equal(b.counts(i), first[i])
        # change the layout: drop to one instance with more rays
        b.clear_instances()
        th = scenes.three_heliostats()
        b.add_instance(0, th.sun_dir, th.sun_shape, th.sun_param, 400000, seed=4, instance=2)
        b.run()
        counts, _, _ = _plain_counts(native, th.elements, th.sun_dir, th.sun_shape, th.sun_param, 400000, 4, 2)
        np.testing.assert_array_equal(b.counts(0), counts)
    finally:
        b.close()


def test_batch_pipelined_runs(gpu):
    """run_async / wait: two runs in flight with different instance sets (the second built while
    the first executes) give each set's own results, equal to synchronous runs; a third run_async
    and a wait with nothing in flight are refused; results survive a change of the instance list."""
    from optixsoltracedemos_gb300 import native
    b, jobs, scene_el = _mixed_batch(native)
    th = scenes.three_heliostats()
    try:
        b.run()
        ref_a = [b.counts(i).copy() for i in range(len(jobs))]
        ref_a_stats = [b.stats(i).copy() for i in range(len(jobs))]
        counts_b, _, _ = _plain_counts(native, th.elements, th.sun_dir, th.sun_shape, th.sun_param, 400000, 4, 2)
        for _ in range(2):
            b.run_async()  # set A
            b.clear_instances()
            b.add_instance(0, th.sun_dir, th.sun_shape, th.sun_param, 400000, seed=4, instance=2)
            b.run_async()  # set B, built while A runs
            with pytest.raises(native.CspError):
                b.run_async()
            b.wait()
            assert len(b) == 1
            for i in range(len(jobs)):
                np.testing.assert_array_equal(b.counts(i), ref_a[i])
                np.testing.assert_array_equal(b.stats(i), ref_a_stats[i])
            b.wait()
            np.testing.assert_array_equal(b.counts(0), counts_b)
            with pytest.raises(native.CspError):
                b.counts(1)  # set B has one instance
            with pytest.raises(native.CspError):
                b.wait()
            b.clear_instances()
            for j in jobs:
                b.add_instance(j[0], j[2], j[3], j[4], j[5], seed=j[6], instance=j[7], poses=j[1])
        # a run that needs a larger arena than the one in flight (reallocation behind it)
        b.clear_instances()
        b.add_instance(0, th.sun_dir, th.sun_shape, th.sun_param, 400000, seed=4, instance=2)
        b.run_async()  # small layout in flight
        b.clear_instances()
        for j in jobs * 3:
            b.add_instance(j[0], j[2], j[3], j[4], j[5], seed=j[6], instance=j[7], poses=j[1])
        b.run_async()  # three times the instances: the arena grows
        b.wait()
        np.testing.assert_array_equal(b.counts(0), counts_b)
        b.wait()
        for i in range(3 * len(jobs)):
            np.testing.assert_array_equal(b.counts(i), ref_a[i % len(jobs)])
        b.clear_instances()
        for j in jobs:
            b.add_instance(j[0], j[2], j[3], j[4], j[5], seed=j[6], instance=j[7], poses=j[1])
        # synchronous run after pipelined ones, and a run_async left in flight at close
        b.run()
        for i in range(len(jobs)):
            np.testing.assert_array_equal(b.counts(i), ref_a[i])
        b.run_async()
    finally:
        b.close()


def test_batch_fine_coherent_level(gpu):
    """An instance of more than 32 * 2^9 * 3^6 = 11,943,936 rays (the first coherent-order level of
    the launches without dense records) gives the plain run's flux map, count for count."""
    from optixsoltracedemos_gb300 import native
    sun = scenes.sun_vector(35.0, 20.0)
    el = scenes.reaim(_field(600, sun), sun)
    n = 11943936 + 1234567
    b = native.Batch(0)
    try:
        sid = b.add_scene(el)
        b.add_instance(sid, sun, scenes.SUN_PILLBOX, 4.65e-3, n, seed=6, instance=3)
        b.run()
        t = native.Tracer(0, n)
        try:
            t.set_elements(el)
            t.set_sun_vector(sun)
            t.set_sun_shape(scenes.SUN_PILLBOX, 4.65e-3)
            t.set_seed(6, 3)
            t.initialize()
            t.run()
            counts, _ = t.flux_map()
        finally:
            t.close()
        assert counts.sum() > 10000
        np.testing.assert_array_equal(b.counts(0), counts)
    finally:
        b.close()


def test_batch_empty_instances(gpu):
    """Instances with no rays trace nothing and leave empty flux maps; the others are unaffected."""
    from optixsoltracedemos_gb300 import native
    th = scenes.three_heliostats()
    b = native.Batch(0)
    try:
        sid = b.add_scene(th.elements)
        b.add_instance(sid, th.sun_dir, th.sun_shape, th.sun_param, 0, seed=1, instance=0)
        b.add_instance(sid, th.sun_dir, th.sun_shape, th.sun_param, 77777, seed=1, instance=1)
        b.add_instance(sid, th.sun_dir, th.sun_shape, th.sun_param, 0, seed=1, instance=2)
        b.run()
        assert b.counts(0).sum() == 0 and b.counts(2).sum() == 0
        assert list(b.stats(0)) == [0, 0, 0, 0]
        counts, _, _ = _plain_counts(native, th.elements, th.sun_dir, th.sun_shape, th.sun_param, 77777, 1, 1)
        np.testing.assert_array_equal(b.counts(1), counts)
    finally:
        b.close()


def test_batch_rejects_bad_instances(gpu):
    from optixsoltracedemos_gb300 import native
    b = native.Batch(0)
    try:
        th = scenes.three_heliostats()
        sid = b.add_scene(th.elements)
        bad = th.elements.copy()
        bad["surface"][0] = scenes.SURFACE_PARABOLIC
        with pytest.raises(native.CspError):
            b.add_instance(sid, th.sun_dir, 0, 4.65e-3, 1000, poses=bad)
        with pytest.raises(native.CspError):
            b.add_instance(sid + 5, th.sun_dir, 0, 4.65e-3, 1000)
        with pytest.raises(native.CspError):
            b.run()  # no instances
        with pytest.raises(native.CspError):
            b.counts(0)
    finally:
        b.close()
