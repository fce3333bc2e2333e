"""Flux-map binning on the CPU: the oracle's float binning (the definition the device kernels follow)
against the double-precision restatement of the reference's post-processing script."""
import numpy as np
import pytest

from optixsoltracedemos_gb300 import flux, scenes


def test_oracle_atan2_accuracy(oracle32):
    rng = np.random.default_rng(0)
    y = rng.normal(size=100000).astype(np.float32)
    x = rng.normal(size=100000).astype(np.float32)
    a = oracle32.atan2(y, x)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.abs(a - ref).max() < 4e-7
    # axes and diagonals
    yy = np.array([0, 1, 0, -1, 1, -1, 1, -1], np.float32)
    xx = np.array([1, 0, -1, 0, 1, -1, -1, 1], np.float32)
    np.testing.assert_allclose(oracle32.atan2(yy, xx), np.arctan2(yy, xx), atol=4e-7)


def _target(native_lib, receiver, nx=100, ny=100):
    from optixsoltracedemos_gb300 import native
    return native.flux_target(receiver, nx, ny)


@pytest.mark.parametrize("name", ["three_heliostats", "single_parabolic"])
def test_flux_target_matches_host_frame(native_lib, name):
    sc = getattr(scenes, name)()
    rcv = sc.elements[-1]
    t = _target(native_lib, rcv)
    x, y, z = flux.element_axes(rcv)
    np.testing.assert_allclose(t[0:3], rcv["origin"], atol=1e-6)
    np.testing.assert_allclose(t[3:6], x, atol=1e-7)
    np.testing.assert_allclose(t[6:9], y, atol=1e-7)
    np.testing.assert_allclose(t[9:12], z, atol=1e-7)
    assert int(t[17]) == (1 if int(rcv["surface"]) == scenes.SURFACE_CYLINDER else 0)
    # bin area (m^2) as flux.py computes it
    w, h = float(rcv["width"]), float(rcv["height"])
    area = (2 * np.pi * 0.5 * w / 100) * (h / 100) if t[17] == 1 else (w / 100) * (h / 100)
    assert t[18] == pytest.approx(area, rel=1e-6)


@pytest.mark.parametrize("name,n", [("three_heliostats", 200000), ("single_parabolic", 100000)])
def test_float_binning_matches_double_restatement(native_lib, oracle32, name, n):
    """orc_flux_counts (float, the device definition) bins the same receiver records as
    flux.flux_map_from_hits (double): equal totals, and bins differ only for records within float
    rounding of a bin edge."""
    sc = getattr(scenes, name)(num_rays=n)
    hits, _ = oracle32.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, 0, n, seed=3)
    hits = hits.astype(np.float32)
    t = _target(native_lib, sc.elements[-1])
    counts, stats = oracle32.flux_counts(hits, t)
    f64 = flux.flux_map_from_hits(hits, sc.elements[-1], n)  # per-ray weight 1/n per bin area
    rcv = sc.elements[-1]
    area = float(t[18])
    c64 = np.rint(f64 * n * area).astype(np.int64)
    assert stats[2] == int((hits[..., 0] == 2.0).sum())
    assert stats[1] == int((hits[..., 0] == 1.0).sum())
    assert int(counts.sum()) == int(stats[3])
    assert abs(int(counts.sum()) - int(c64.sum())) <= max(2, int(1e-5 * stats[2]))
    moved = int(np.abs(counts.astype(np.int64) - c64).sum()) // 2
    assert moved <= max(2, int(1e-4 * stats[3])), (moved, int(stats[3]))
    assert stats[3] > 0
