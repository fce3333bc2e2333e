"""GPU parity: the CUDA trace, called through the C ABI, against the oracle and the reference's own
golden records.  Integer/index data (stage codes, element ids) and the float32 hit positions must be
bit-identical (the kernels and the oracle perform the same IEEE float operations in the same order);
the FP64 oracle bounds the flux-map L2 error."""
import glob
import os

import numpy as np
import pytest

from optixsoltracedemos_gb300 import native, scenes
from optixsoltracedemos_gb300.flux import flux_map_from_hits, flux_l2

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def gpu_trace(sc, n, seed=0, instance=0, first=0, count=None, accel=native.ACCEL_AUTO):
    t = native.tracer_for(sc, seed=seed, instance=instance, num_rays=n, accel=accel)
    t.run()
    hits, ids = t.copy_hits(first, count)
    t.close()
    return hits, ids


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_reference_golden(gpu, path):
    g = np.load(path)
    sc = scenes.Scene("golden", g["elements"], g["sun_dir"], 0, float(g["sun_param"]), 0)
    first, n = int(g["first"]), len(g["hits"])
    hits, ids = gpu_trace(sc, first + n, seed=int(g["seed"]), instance=int(g["instance"]), first=first, count=n)
    np.testing.assert_array_equal(hits, g["hits"])
    np.testing.assert_array_equal(ids, g["ids"])


def _configs():
    return {
        "three_heliostats": scenes.three_heliostats(),
        "three_heliostats_ref": scenes.three_heliostats(reflectivity=1.0, slope_error=0.0),
        "single_parabolic": scenes.single_parabolic(),
        "single_parabolic_pillbox_spec": scenes.single_parabolic(sun_shape=0, sun_sigma=4.65e-3),
        "field_300": scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(40.0, 30.0)),
        "field_2000_parabolic": scenes.large_field(n_heliostats=2000, parabolic=True, sun=scenes.sun_vector(60.0, -45.0)),
        "corridor_multibounce": scenes.corridor(slope_error=1e-3),
        # the accurate arithmetic flag: cancellation-free cone sampler and cylinder roots
        "single_parabolic_accurate": scenes.single_parabolic(sun_shape=scenes.SUN_GAUSSIAN_ACCURATE),
        "three_heliostats_accurate": _with_shape(scenes.three_heliostats(), scenes.SUN_PILLBOX_ACCURATE),
        "field_300_accurate": _with_shape(scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(40.0, 30.0)),
                                          scenes.SUN_PILLBOX_ACCURATE),
    }


def _with_shape(sc, shape):
    sc.sun_shape = shape
    return sc


@pytest.mark.parametrize("name", list(_configs()))
def test_gpu_matches_oracle_bit_exact(gpu, oracle32, name):
    sc = _configs()[name]
    if name == "single_parabolic_pillbox_spec":
        sc.elements["specularity_error"][0] = 0.5e-3
        sc.elements["reflectivity"][0] = 0.93
    n = 60000
    # fields run through both search structures (grid by default, BVH forced)
    accels = (native.ACCEL_AUTO, native.ACCEL_BVH) if name.startswith("field") else (native.ACCEL_AUTO,)
    for seed, inst in ((0, 0), (987654321, 5)):
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, seed=seed, instance=inst)
        for accel in accels:
            hits, ids = gpu_trace(sc, n, seed=seed, instance=inst, accel=accel)
            np.testing.assert_array_equal(ids, oi)
            np.testing.assert_array_equal(hits, oh.astype(np.float32))


def _reach_edge_configs():
    """Element-list scenes at the edges of the sun-plane reach test (rays whose sun-plane point lies
    outside every element's reach rectangle skip their direction): wide pillbox cones up to the
    largest half angle the API accepts (0.5 rad), a wide Gaussian sun, a collimated zenith sun
    (axis-parallel rays: infinite slab reciprocals), and a sun 2 degrees above the horizon."""
    wide = scenes.single_parabolic(sun_shape=0, sun_sigma=0.3)
    very_wide = scenes.three_heliostats(sun_angle=0.5)
    gauss = scenes.single_parabolic(sun_sigma=30e-3)
    zenith = scenes.three_heliostats(sun_angle=0.0)
    zenith.sun_dir = np.array([0.0, 0.0, 1.0])
    low = scenes.three_heliostats()
    low.sun_dir = scenes.sun_vector(2.0, 10.0)
    return {"pillbox_0.3rad": wide, "pillbox_0.5rad": very_wide, "gaussian_30mrad": gauss,
            "collimated_zenith": zenith, "sun_2deg": low}


@pytest.mark.parametrize("name", list(_reach_edge_configs()))
def test_reach_pretest_edges_bit_exact(gpu, oracle32, name):
    sc = _reach_edge_configs()[name]
    n = 60000
    for seed, inst in ((3, 0), (55, 2)):
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, seed=seed, instance=inst)
        hits, ids = gpu_trace(sc, n, seed=seed, instance=inst)
        np.testing.assert_array_equal(ids, oi)
        np.testing.assert_array_equal(hits, oh.astype(np.float32))
        assert (oh[:, 1:, 0] != 0).any()


def _sungrid_edge_configs():
    """Field scenes at the edges of the sun-ray candidate grid (one cell of reach rectangles per sun
    ray, rectangles of more than 64 cells in a global list every ray scans): a sun 3 degrees above
    the horizon (rectangles stretched along the plane's steep axis), a wide Gaussian sun and a wide
    pillbox (rectangles widened by the cone, many of them global), a collimated zenith sun
    (axis-parallel rays), and a parabolic field at a low sun."""
    low = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(3.0, 40.0))
    gauss = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(30.0, -20.0))
    gauss.sun_shape, gauss.sun_param = scenes.SUN_GAUSSIAN, 40e-3
    wide = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(50.0, 100.0), sun_angle=0.2)
    zenith = scenes.large_field(n_heliostats=300, sun=np.array([0.0, 0.0, 1.0]), sun_angle=0.0)
    par_low = scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(8.0, -150.0), parabolic=True)
    return {"sun_3deg": low, "gaussian_40mrad": gauss, "pillbox_0.2rad": wide, "collimated_zenith": zenith,
            "parabolic_sun_8deg": par_low}


@pytest.mark.parametrize("name", list(_sungrid_edge_configs()))
def test_sungrid_edges_bit_exact(gpu, oracle32, name):
    sc = _sungrid_edge_configs()[name]
    n = 60000
    for seed, inst in ((7, 0), (31, 4)):
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, seed=seed, instance=inst)
        for accel in (native.ACCEL_AUTO, native.ACCEL_BVH):
            hits, ids = gpu_trace(sc, n, seed=seed, instance=inst, accel=accel)
            np.testing.assert_array_equal(ids, oi, err_msg=f"{name} accel {accel}")
            np.testing.assert_array_equal(hits, oh.astype(np.float32), err_msg=f"{name} accel {accel}")
        assert (oh[:, 1:, 0] != 0).any()


@pytest.mark.parametrize("first", [(1 << 32) - 5000, (1 << 40) + 12345], ids=["2^32-5000", "2^40+12345"])
def test_ray_indices_beyond_32_bits(gpu, oracle32, first):
    """Ray windows starting near and far beyond 2^32 (csp_trace_into with a first ray): the Halton
    loops past their tables, the 64-bit Philox counter and, for the field, the coherent order of
    a 400k-ray window offset by the first ray, against the oracle."""
    import torch
    cases = [(scenes.three_heliostats(), 60000), (scenes.single_parabolic(), 60000),
             (scenes.large_field(n_heliostats=300, sun=scenes.sun_vector(40.0, 30.0)), 400000)]
    for sc, n in cases:
        t = native.tracer_for(sc, seed=2, instance=1, num_rays=1024)
        try:
            hits = torch.zeros(n * 5 * 4, dtype=torch.float32, device="cuda")
            ids = torch.zeros(n * 5, dtype=torch.int32, device="cuda")
            t.trace_into(hits.data_ptr(), ids.data_ptr(), first, n)
            torch.cuda.synchronize()
        finally:
            t.close()
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=first, count=n, seed=2,
                                instance=1)
        np.testing.assert_array_equal(ids.cpu().numpy().view(np.uint32).reshape(n, 5), oi, err_msg=sc.name)
        np.testing.assert_array_equal(hits.cpu().numpy().reshape(n, 5, 4), oh.astype(np.float32), err_msg=sc.name)
        assert (oh[:, 1:, 0] != 0).any()


@pytest.mark.parametrize("accel", [native.ACCEL_BVH, native.ACCEL_GRID], ids=["bvh", "grid"])
def test_gpu_large_field_bit_exact(gpu, oracle32, accel):
    """2000 flat heliostats, cylinder receiver, through the BVH and through the field grid: a window
    of 100k rays starting mid-launch, against the oracle's brute-force closest hit."""
    sc = scenes.large_field(n_heliostats=2000, sun=scenes.sun_vector(35.0, 70.0))
    t = native.tracer_for(sc, seed=4, num_rays=400000, accel=accel)
    assert t.accel() == accel
    t.run()
    first, n = 150001, 100000
    hits, ids = t.copy_hits(first, n)
    t.close()
    oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=first, count=n, seed=4)
    np.testing.assert_array_equal(ids, oi)
    np.testing.assert_array_equal(hits, oh.astype(np.float32))
    assert (hits[:, :, 0] == 2).sum() > 1000


def test_coherent_order_windows_bit_exact(gpu, oracle32):
    """Field launches give each warp rays at a Halton-coherent stride (blocks of 1,990,656 rays, then
    of 331,776, then the identity order): windows in every region of a 2.4M-ray launch, and the
    block boundaries, against the oracle."""
    sc = scenes.large_field(n_heliostats=2000, sun=scenes.sun_vector(50.0, -30.0))
    N = 1990656 + 331776 + 5000
    t = native.tracer_for(sc, seed=9, num_rays=N)
    t.run()
    for first, n in ((0, 20000), (1990656 - 7000, 14000), (1990656 + 331776 - 7000, 12000), (N - 3000, 3000)):
        hits, ids = t.copy_hits(first, n)
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=first, count=n, seed=9)
        np.testing.assert_array_equal(ids, oi)
        np.testing.assert_array_equal(hits, oh.astype(np.float32))
    t.close()


@pytest.mark.parametrize("el,az,parabolic", [(45.0, 0.0, False), (11.0, 80.0, False), (78.0, -100.0, True),
                                              (25.0, 180.0, True)])
def test_grid_equals_bvh_full_field(gpu, el, az, parabolic):
    """10,000-heliostat field at several sun positions (low sun: long walks through the layer): the
    grid and the BVH give identical records and element ids for 1M rays; after re-aiming the
    heliostats (csp_update) too."""
    sc = scenes.large_field(sun=scenes.sun_vector(el, az), parabolic=parabolic)
    n = 1 << 20
    out = {}
    for accel in (native.ACCEL_GRID, native.ACCEL_BVH):
        t = native.tracer_for(sc, seed=7, num_rays=n, accel=accel)
        assert t.accel() == accel
        t.run()
        a = t.copy_hits()
        t.set_elements(scenes.reaim(sc.elements, scenes.sun_vector(el + 5.0, az + 10.0)))
        t.set_sun_vector(scenes.sun_vector(el + 5.0, az + 10.0))
        t.update()
        t.run()
        out[accel] = (a, t.copy_hits())
        t.close()
    for k in range(2):
        np.testing.assert_array_equal(out[native.ACCEL_GRID][k][1], out[native.ACCEL_BVH][k][1])
        np.testing.assert_array_equal(out[native.ACCEL_GRID][k][0], out[native.ACCEL_BVH][k][0])
    assert (out[native.ACCEL_GRID][0][0][:, :, 0] == 2).sum() > 1000


def test_accel_selection(gpu):
    """AUTO picks the grid for a planar field, the BVH for a non-planar scene of more than 8
    elements, the element list for small scenes; GRID on a non-planar scene is an error."""
    field = scenes.large_field(n_heliostats=300)
    t = native.tracer_for(field, num_rays=1)
    assert t.accel() == native.ACCEL_GRID
    t.close()
    t = native.tracer_for(scenes.three_heliostats(), num_rays=1)
    assert t.accel() == native.ACCEL_LIST
    t.close()
    # a stack of mirrors: 12 mirrors at heights 0..110 m, the layer is as tall as the field is wide
    e = scenes.make_elements(13)
    e["origin"][:12] = [[0.0, 0.0, 10.0 * k] for k in range(12)]
    e["aim_point"][:12] = [[0.0, 1.0, 10.0 * k + 1.0] for k in range(12)]
    e["width"][:12] = 5.0
    e["height"][:12] = 5.0
    e["origin"][12] = [0.0, 50.0, 50.0]
    e["aim_point"][12] = [0.0, 0.0, 50.0]
    e["width"][12] = 10.0
    e["height"][12] = 10.0
    stack = scenes.Scene("stack", e, np.array([0.0, 1.0, 0.2]), 0, 4.65e-3, 1)
    t = native.tracer_for(stack, num_rays=1)
    assert t.accel() == native.ACCEL_BVH
    t.close()
    with pytest.raises(native.CspError):
        native.tracer_for(stack, num_rays=1, accel=native.ACCEL_GRID)


def test_gpu_sun_plane_matches_oracle(gpu, oracle32):
    for sc in _configs().values():
        t = native.tracer_for(sc, num_rays=1)
        sp = t.sun_plane()
        t.close()
        _, sun = oracle32.scene_info(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param)
        np.testing.assert_array_equal(sp[:15], sun[:15].astype(np.float32))
        assert sp[15] == np.float32(sun[15])


def test_full_size_single_parabolic_sampled_and_properties(gpu, oracle32):
    """16M rays (the benchmark workload): bit-exact on sampled windows across the index range
    (including around 2^24 where the Halton base-2 path changes) and size-independent properties
    over all rays."""
    sc = scenes.single_parabolic()
    N = sc.num_rays
    t = native.tracer_for(sc, num_rays=N)
    t.run()
    for first in (0, 1234567, (1 << 24) - 4096, N - 4096):
        n = min(4096, N - first)
        hits, ids = t.copy_hits(first, n)
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=first, count=n)
        np.testing.assert_array_equal(ids, oi)
        np.testing.assert_array_equal(hits, oh.astype(np.float32))
    hits, ids = t.copy_hits(0, N)
    t.close()
    st = hits[:, :, 0]
    assert np.all(st[:, 0] == 0)                              # slot 0 is always the sun point
    assert np.all(np.isin(st, (0.0, 1.0, 2.0)))
    assert np.all((ids == native.NO_ELEMENT) == (st == 0))     # an id exactly where a record is
    recv = st == 2
    assert np.all(ids[recv] == 1) and np.all(ids[st == 1] == 0)
    # a receiver record ends the path: nothing after it
    after = np.cumsum(recv, axis=1) - recv
    assert not np.any((after > 0) & (st != 0))
    # sun points lie in the sun-plane parallelogram (Halton u, v in [0, 1))
    assert recv.sum() > 0.05 * N


# Coherent-order regions of a dense field launch of N rays: whole blocks of B1 = 32 * 2^8 3^5 rays,
# then blocks of B2 = 32 * 2^7 3^4 over the rest, then the identity order.
_B1, _B2 = 32 * 256 * 243, 32 * 128 * 81


@pytest.mark.parametrize("el,az,parabolic,shape", [(45.0, 0.0, False, 0), (15.0, 0.0, False, 0), (45.0, 0.0, True, 0),
                                                    (45.0, 0.0, False, 2)],
                         ids=["flat_45deg", "flat_15deg", "parabolic_45deg", "flat_45deg_accurate"])
def test_large_field_full_launch_windows_bit_exact(gpu, oracle32, el, az, parabolic, shape):
    """The 10,000-heliostat field (radial stagger, cylinder receiver at 200 m, pillbox 4.65 mrad,
    slope error 1.5 mrad) traced at its full size of 268,435,456 rays in one launch through the
    field grid, against the oracle's brute-force closest hit over all 10,001 elements on windows of
    50,000 rays: around 2^24 (where the Halton base-2 path changes), across the boundary between the
    B1 and B2 coherent-order regions, and at the end of the launch (identity-order tail)."""
    sc = scenes.large_field(sun=scenes.sun_vector(el, az), parabolic=parabolic)
    sc.sun_shape = shape
    N = sc.num_rays
    assert N == 1 << 28
    full1 = (N // _B1) * _B1
    t = native.tracer_for(sc, seed=17, instance=3, num_rays=N)
    try:
        assert t.accel() == native.ACCEL_GRID
        t.run()
        w = 50000
        for first in ((1 << 24) - w // 2, full1 - w // 2, N - w):
            hits, ids = t.copy_hits(first, w)
            oh, oi = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=first, count=w,
                                    seed=17, instance=3)
            np.testing.assert_array_equal(ids, oi, err_msg=f"window at {first}")
            np.testing.assert_array_equal(hits, oh.astype(np.float32), err_msg=f"window at {first}")
            assert (oh[:, 1:, 0] == 2).sum() > 1000
    finally:
        t.close()


def test_large_field_flux_l2_vs_fp64_oracle(gpu, oracle64):
    """Flux-map L2 of the full-size field trace (268,435,456 rays in one launch) against the FP64
    oracle with matched seeds, by the same method as the smaller workloads (100 x 100 bins on the
    cylinder), over a 524,288-ray window of the launch (the FP64 brute force over 10,001 elements
    bounds the window; ~16 receiver hits per bin).  With the accurate arithmetic flag the float
    trace is within 1 % (tolerance 0.01).  The reference's float formulas -- the cone sampler's
    z = cos(a) + (1 - cos(a)) r (~2e-4 rad of direction error, 8 cm at the receiver) and the
    cylinder's B^2 - 4AC (~1 mm on hit points from mirrors hundreds of metres away) -- move rays
    across bin edges and stay statistics-limited at this window (asserted below 10 %; the figure
    falls as 1/sqrt(hits per bin) over the whole launch)."""
    base = scenes.large_field()
    N = base.num_rays
    first, w = 1 << 26, 1 << 19
    oh, _ = oracle64.trace(base.elements, base.sun_dir, base.sun_shape, base.sun_param, first_ray=first, count=w,
                           with_ids=False)
    ref_map = flux_map_from_hits(oh, base.elements[-1], w)
    del oh
    l2 = {}
    for shape in (scenes.SUN_PILLBOX_ACCURATE, scenes.SUN_PILLBOX):
        sc = scenes.large_field()
        sc.sun_shape = shape
        t = native.tracer_for(sc, seed=0, num_rays=N, record_ids=False)
        try:
            t.run()
            hits, _ = t.copy_hits(first, w, with_ids=False)
        finally:
            t.close()
        l2[shape] = flux_l2(flux_map_from_hits(hits, sc.elements[-1], w), ref_map)
    print("large_field 512k-ray window flux L2 vs FP64: accurate arithmetic", l2[scenes.SUN_PILLBOX_ACCURATE],
          "reference arithmetic", l2[scenes.SUN_PILLBOX])
    assert l2[scenes.SUN_PILLBOX_ACCURATE] <= 0.01
    assert l2[scenes.SUN_PILLBOX] <= 0.10


def test_accurate_arithmetic_three_heliostats(gpu, oracle32, oracle64):
    """CSP_SUN_PILLBOX_ACCURATE on the three-heliostat workload at 1,048,576 rays: bit-identical to
    the oracle's restatement of the same arithmetic, and flux-map L2 against the FP64 oracle within
    1 % (tolerance 0.01).  The reference's float cone formula (CSP_SUN_PILLBOX, the default) stays
    above that bound at this ray count (6.9 %): its float z quantizes 1 - z in steps of 2^-24
    against 1 - cos(4.65 mrad) = 1.08e-5."""
    base = scenes.three_heliostats()
    n = base.num_rays
    assert n == 1 << 20
    oh64, _ = oracle64.trace(base.elements, base.sun_dir, base.sun_shape, base.sun_param, count=n, with_ids=False)
    ref_map = flux_map_from_hits(oh64, base.elements[-1], n)
    l2 = {}
    for shape in (scenes.SUN_PILLBOX_ACCURATE, scenes.SUN_PILLBOX):
        sc = scenes.three_heliostats()
        sc.sun_shape = shape
        hits, ids = gpu_trace(sc, n)
        first, w = 500000, 60000
        oh, oi = oracle32.trace(sc.elements, sc.sun_dir, shape, sc.sun_param, first_ray=first, count=w)
        np.testing.assert_array_equal(ids[first:first + w], oi)
        np.testing.assert_array_equal(hits[first:first + w], oh.astype(np.float32))
        l2[shape] = flux_l2(flux_map_from_hits(hits, sc.elements[-1], n), ref_map)
    print("three_heliostats 1M flux L2 vs FP64: accurate sampler", l2[scenes.SUN_PILLBOX_ACCURATE],
          "reference sampler", l2[scenes.SUN_PILLBOX])
    assert l2[scenes.SUN_PILLBOX_ACCURATE] <= 0.01
    assert 0.03 <= l2[scenes.SUN_PILLBOX] <= 0.12


def test_ray_windows_past_2_56_rejected(gpu):
    """The BVH and grid kernels queue rays with their bounce depth in the top 8 bits of the 64-bit
    ray index, so every entry point rejects a window reaching past 2^56 before any launch
    (CSP_ERR_INVALID_ARGUMENT): csp_trace_into on an initialized 300-heliostat field, csp_set_num_rays
    and csp_trace_noalloc.  Nothing is traced."""
    sc = scenes.large_field(n_heliostats=300)
    t = native.tracer_for(sc, num_rays=1024)
    try:
        for first, count in (((1 << 56) - 10, 1024), ((1 << 64) - 5, 16), (1 << 56, 1)):
            with pytest.raises(native.CspError) as e:
                t.trace_into(0x1000, None, first, count)
            assert e.value.status == -1 and "2^56" in str(e.value)
        with pytest.raises(native.CspError) as e:
            t.set_num_rays((1 << 56) + 1)
        assert e.value.status == -1
    finally:
        t.close()
    small = scenes.three_heliostats()
    with pytest.raises(native.CspError) as e:
        native.trace_noalloc(small.elements, small.sun_dir, small.sun_shape, small.sun_param, 0x1000,
                             first_ray=(1 << 56) - 3, num_rays=8)
    assert e.value.status == -1


def test_flux_map_l2_vs_fp64_oracle(gpu, oracle64):
    """Flux-map L2 of the GPU float trace against the FP64 oracle with matched seeds, at the
    benchmark workload's 16M rays (tolerance 1%).  The float trace follows the reference's float
    cone sampling, which moves ~1% of rays into a neighbouring bin relative to exact arithmetic, so
    the L2 falls as 1/sqrt(hits per bin); smaller ray counts are reported, not asserted at 1%."""
    sc = scenes.single_parabolic()
    n = sc.num_rays
    hits, _ = gpu_trace(sc, n)
    oh, _ = oracle64.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, with_ids=False)
    l2 = flux_l2(flux_map_from_hits(hits, sc.elements[-1], n), flux_map_from_hits(oh, sc.elements[-1], n))
    print("single_parabolic 16M flux L2 vs FP64 oracle:", l2)
    assert l2 <= 0.01
    sc = scenes.three_heliostats()
    n = 1 << 22
    hits, _ = gpu_trace(sc, n)
    oh, _ = oracle64.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=n, with_ids=False)
    l2 = flux_l2(flux_map_from_hits(hits, sc.elements[-1], n), flux_map_from_hits(oh, sc.elements[-1], n))
    print("three_heliostats 4M flux L2 vs FP64 oracle:", l2)
    assert l2 <= 0.05
