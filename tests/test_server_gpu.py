"""Serving (continuous batching) on the GPU: every request's flux map is the same alone and in a
mix of concurrent requests of different scenes, sizes and ray counts (sliced over several steps),
equals the plain single-scene result, and admission respects the memory budget."""
import threading

import numpy as np
import pytest

from optixsoltracedemos_gb300 import scenes

pytestmark = pytest.mark.gpu


def _plain_counts(native, elements, sun, shape, param, rays, seed, instance):
    t = native.Tracer(0, rays)
    try:
        t.set_elements(elements)
        t.set_sun_vector(sun)
        t.set_sun_shape(shape, param)
        t.set_seed(seed, instance)
        t.initialize()
        t.run()
        return t.flux_map()[0]
    finally:
        t.close()


def _workload():
    th = scenes.three_heliostats()
    pb = scenes.single_parabolic()
    field = scenes.large_field(n_heliostats=600, num_rays=1).elements
    scene_list = [th.elements, pb.elements, field]
    reqs = []
    rs = np.random.default_rng(5)
    for k in range(10):
        sid = k % 3
        if sid == 0:
            sun = np.array([rs.uniform(-0.3, 0.3), -1.0, 1.0])
            poses = th.elements.copy()
            poses["aim_point"][:3] = scenes.bisector_aim(poses["origin"][:3], sun, [0.0, 0.0, 10.0])
            req = (sid, poses, sun, scenes.SUN_PILLBOX, 4.65e-3)
        elif sid == 1:
            req = (sid, None, pb.sun_dir, scenes.SUN_GAUSSIAN, 2.5e-3)
        else:
            sun = scenes.sun_vector(rs.uniform(15, 80), rs.uniform(-120, 120))
            poses = scenes.reaim(field, sun)
            if k == 5:
                poses["origin"][3] += [1.5, 0.0, 0.0]  # a moved heliostat: BVH group
            req = (sid, poses, sun, scenes.SUN_PILLBOX, 4.65e-3)
        rays = int(rs.integers(200_000, 3_500_000))
        reqs.append(req + (rays, 100 + k, k))
    return scene_list, reqs


def _submit(srv, req):
    sid, poses, sun, shape, param, rays, seed, inst = req
    return srv.submit(sid, sun, shape, param, rays, seed=seed, instance=inst, poses=poses)


def test_server_results_same_alone_and_in_mix(gpu):
    from optixsoltracedemos_gb300 import native
    scene_list, reqs = _workload()
    # step_rays small: each request (at most 3.5M rays, below the 2^24-ray minimum slice) is traced
    # in one slice, several requests per step
    srv = native.Server(0, memory_budget=256 << 20, max_active=8, step_rays=4 << 20)
    try:
        sids = [srv.add_scene(e) for e in scene_list]
        assert sids == [0, 1, 2]
        alone = []
        for r in reqs:
            rid = _submit(srv, r)
            c, st, lat = srv.wait(rid, timeout=120)
            alone.append((c, st))
            assert lat[0] >= lat[1] >= 0
        # the mix: all requests submitted from four threads while admission is held, then admitted
        # together (8 slots for 10 requests: the last two join while the first ones run)
        ids = [None] * len(reqs)
        srv.hold(True)

        def sub(k):
            for i in range(k, len(reqs), 4):
                ids[i] = _submit(srv, reqs[i])
        th = [threading.Thread(target=sub, args=(k,)) for k in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        srv.hold(False)
        for i, rid in enumerate(ids):
            c, st, _ = srv.wait(rid, timeout=120)
            np.testing.assert_array_equal(c, alone[i][0], err_msg=f"request {i}")
            np.testing.assert_array_equal(st, alone[i][1])
        stats = srv.stats()
        assert stats["completed"] == 2 * len(reqs)
        assert stats["peak_active"] > 1  # the mix really ran concurrently
        assert 0 < stats["p50_s"] <= stats["p99_s"]
        assert stats["rays"] == 2 * sum(r[5] for r in reqs)
    finally:
        srv.close()
    # and equal to the plain single-scene path
    for i in (0, 1, 2, 5):
        sid, poses, sun, shape, param, rays, seed, inst = reqs[i]
        el = scene_list[sid] if poses is None else poses
        np.testing.assert_array_equal(alone[i][0], _plain_counts(native, el, sun, shape, param, rays, seed, inst))


def test_server_admission_by_memory(gpu):
    """A budget that holds three field requests with their own poses: ten such requests queue, are
    admitted as memory frees up, and all complete."""
    from optixsoltracedemos_gb300 import native
    field = scenes.large_field(n_heliostats=2000, num_rays=1).elements
    rs = np.random.default_rng(1)
    suns = [scenes.sun_vector(rs.uniform(20, 70), rs.uniform(-90, 90)) for _ in range(10)]
    poses = [scenes.reaim(field, s) for s in suns]
    # a request's device block (records, grids, candidate lists, flux map), measured on one alone;
    # the poses change its grids by a few per cent, so 3.5 blocks hold three requests, never four
    probe = native.Server(0, memory_budget=256 << 20, max_active=4)
    try:
        sid = probe.add_scene(field)
        probe.wait(probe.submit(sid, suns[0], 0, 4.65e-3, 1 << 20, poses=poses[0]), timeout=120)
        per_request = int(probe.stats()["peak_arena_bytes"])
    finally:
        probe.close()
    budget = int(3.5 * per_request)
    srv = native.Server(0, memory_budget=budget, max_active=64, step_rays=8 << 20)
    try:
        sid = srv.add_scene(field)
        ids = [srv.submit(sid, suns[k], 0, 4.65e-3, 6_000_000, seed=k, instance=k, poses=poses[k]) for k in range(10)]
        for rid in ids:
            c, st, _ = srv.wait(rid, timeout=120)
            assert st[0] == 6_000_000 and c.sum() == st[3]
        stats = srv.stats()
        assert stats["completed"] == 10
        assert 1 <= stats["peak_active"] <= 3
        assert stats["peak_arena_bytes"] <= budget
    finally:
        srv.close()


def test_server_rejects_bad_requests(gpu):
    from optixsoltracedemos_gb300 import native
    th = scenes.three_heliostats()
    srv = native.Server(0, memory_budget=1 << 20, max_active=4)
    try:
        sid = srv.add_scene(th.elements)
        with pytest.raises(native.CspError):
            srv.submit(sid + 3, th.sun_dir, 0, 4.65e-3, 1000)
        bad = th.elements.copy()
        bad["surface"][1] = scenes.SURFACE_PARABOLIC
        with pytest.raises(native.CspError):
            srv.submit(sid, th.sun_dir, 0, 4.65e-3, 1000, poses=bad)
        with pytest.raises(native.CspError):
            srv.submit(sid, th.sun_dir, 0, 4.65e-3, 0)
        with pytest.raises(native.CspError):
            srv.wait(12345)
        big = scenes.large_field(n_heliostats=10000, num_rays=1).elements
        sid2 = srv.add_scene(big)
        with pytest.raises(native.CspError):  # its own records (1.4 MB) exceed the 1 MiB budget
            srv.submit(sid2, th.sun_dir, 0, 4.65e-3, 1000, poses=big)
    finally:
        srv.close()


def test_server_sliced_requests_equal_batch(gpu):
    """Requests of 17M to 40M rays, traced in slices of 2^24 rays over several steps that overlap on
    the server's two step streams (one request's slices in consecutive steps, requests finishing in
    different steps), give the flux maps and counters of one batch run of the same instances."""
    from optixsoltracedemos_gb300 import native
    field = scenes.large_field(n_heliostats=600, num_rays=1).elements
    th = scenes.three_heliostats()
    jobs = []
    for k, (rays, el) in enumerate([(40_000_000, 60.0), (17_000_000, 30.0), (25_000_000, 45.0)]):
        sun = scenes.sun_vector(el, -30.0 + 25.0 * k)
        jobs.append((1, scenes.reaim(field, sun), sun, rays, 7 + k, k))
    jobs.append((0, None, th.sun_dir, 33_000_000, 11, 3))
    srv = native.Server(0, memory_budget=512 << 20, max_active=8)
    try:
        sids = [srv.add_scene(th.elements), srv.add_scene(field)]
        ids = [srv.submit(sids[s], sun, scenes.SUN_PILLBOX, 4.65e-3, rays, seed=seed, instance=inst, poses=poses)
               for s, poses, sun, rays, seed, inst in jobs]
        served = [srv.wait(rid, timeout=300)[:2] for rid in ids]
        assert srv.stats()["steps"] >= 3
    finally:
        srv.close()
    b = native.Batch(0)
    try:
        bs = [b.add_scene(th.elements), b.add_scene(field)]
        for s, poses, sun, rays, seed, inst in jobs:
            b.add_instance(bs[s], sun, scenes.SUN_PILLBOX, 4.65e-3, rays, seed=seed, instance=inst, poses=poses)
        b.run()
        for i, (c, st) in enumerate(served):
            np.testing.assert_array_equal(c, b.counts(i), err_msg=f"request {i}")
            np.testing.assert_array_equal(st, b.stats(i))
    finally:
        b.close()


def test_server_ray_indices_beyond_32_bits(gpu):
    """A request of 5e9 rays (ray indices past 2^32, sliced over many server steps) bins exactly
    what one batch launch of the same rays bins; an impatient wait times out and a later wait still
    gets the result."""
    from optixsoltracedemos_gb300 import native
    th = scenes.three_heliostats()
    rays = 5_000_000_000
    srv = native.Server(0, memory_budget=64 << 20, max_active=4, step_rays=1 << 30)
    try:
        sid = srv.add_scene(th.elements)
        rid = srv.submit(sid, th.sun_dir, th.sun_shape, th.sun_param, rays, seed=3, instance=1)
        with pytest.raises(native.CspError):
            srv.wait(rid, timeout=0.0)
        c_srv, st_srv, _ = srv.wait(rid, timeout=300)
        assert srv.stats()["steps"] >= 5
    finally:
        srv.close()
    b = native.Batch(0)
    try:
        sid = b.add_scene(th.elements)
        b.add_instance(sid, th.sun_dir, th.sun_shape, th.sun_param, rays, seed=3, instance=1)
        b.run()
        np.testing.assert_array_equal(b.counts(0), c_srv)
        np.testing.assert_array_equal(b.stats(0), st_srv)
        assert st_srv[0] == rays and st_srv[3] > 0.02 * rays
    finally:
        b.close()


def test_server_destroy_fails_held_requests(gpu):
    """A request still queued when the server is destroyed (admission held) never runs: a thread
    blocked waiting on it wakes with CSP_ERR_STATE before the server frees anything, and a second
    thread waiting on the same id gets an error instead of a result that was already handed out."""
    import threading
    from optixsoltracedemos_gb300 import native
    th = scenes.three_heliostats()
    srv = native.Server(0, memory_budget=64 << 20, max_active=4)
    sid = srv.add_scene(th.elements)
    srv.hold(True)
    rid = srv.submit(sid, th.sun_dir, th.sun_shape, th.sun_param, 1 << 20, seed=1)
    errors = []

    def waiter():
        try:
            srv.wait(rid)
        except native.CspError as e:
            errors.append(e.status)

    threads = [threading.Thread(target=waiter) for _ in range(2)]
    for t in threads:
        t.start()
    import time
    time.sleep(0.3)
    srv.close()
    for t in threads:
        t.join(timeout=60)
        assert not t.is_alive()
    assert sorted(errors) == [-6, -6]
