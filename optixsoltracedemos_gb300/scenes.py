"""Synthetic scenes for the benchmark and parity workloads.

The reference ships no benchmark scenes (its large-field .stinput files are not in its repository),
so the five workloads are generated here, seeded, with the sizes, layouts and optical parameters of
the benchmark definitions:

  three_heliostats   3 flat 1.0 x 1.95 m mirrors at (-5,5,0), (0,5,0), (5,5,0) aimed at a flat 2 x 2 m
                     receiver centred (0,0,10) facing +y; sun (0,-1,1); pillbox 4.65 mrad;
                     reflectivity 0.9; slope error 1 mrad.  (Mirrors follow the reference demo
                     convention aim = origin + 100 * normal, demos/demo_three_heliostats.cpp:46.)
  single_parabolic   10 x 10 m paraboloid, focal length 100 m (c = 1/(2 f) = 0.005) at (0,100,0)
                     aimed at a cylindrical receiver r = 2 m, h = 4 m, axis +z, centred (0,0,100);
                     sun (0,0,1) (demos/demo_parabolic_surface.cpp:22); Gaussian sun 2.5 mrad;
                     slope error 1.5 mrad.
  large_field        10,000 flat 10 x 10 m heliostats on a radial stagger (radii 100-800 m,
                     azimuthal pitch 1.2 x mirror diagonal, alternate rings offset by half a pitch,
                     +-0.5 m jitter, seed 1) aimed at a cylindrical receiver r = 8 m, h = 20 m
                     centred 200 m up; sun elevation 45 deg, azimuth 0; pillbox 4.65 mrad;
                     slope error 1.5 mrad.
  batched_instances  the large field at 256 sun positions (elevation U(10,80) deg, azimuth
                     U(-120,120) deg, seed 2), heliostats re-aimed per instance, ray counts
                     log-uniform in [2^20, 2^25] (seed 3).
Heliostats are aimed on the bisector of the sun vector and the direction to the receiver centre.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ELEMENT_DTYPE = np.dtype(
    [
        ("origin", "<f8", 3),
        ("aim_point", "<f8", 3),
        ("zrot_deg", "<f8"),
        ("width", "<f8"),
        ("height", "<f8"),
        ("curv_x", "<f8"),
        ("curv_y", "<f8"),
        ("reflectivity", "<f8"),
        ("slope_error", "<f8"),
        ("specularity_error", "<f8"),
        ("surface", "<i4"),
        ("aperture", "<i4"),
    ],
    align=True,
)

SURFACE_FLAT = 0
SURFACE_PARABOLIC = 1
SURFACE_CYLINDER = 3
SUN_PILLBOX = 0
SUN_GAUSSIAN = 1
SUN_ACCURATE = 2  # flag: the trace in cancellation-free float formulas (cone sampler, cylinder roots)
SUN_PILLBOX_ACCURATE = SUN_PILLBOX | SUN_ACCURATE
SUN_GAUSSIAN_ACCURATE = SUN_GAUSSIAN | SUN_ACCURATE


@dataclass
class Scene:
    name: str
    elements: np.ndarray
    sun_dir: np.ndarray
    sun_shape: int
    sun_param: float
    num_rays: int
    meta: dict = field(default_factory=dict)


def make_elements(n: int) -> np.ndarray:
    e = np.zeros(n, ELEMENT_DTYPE)
    e["reflectivity"] = 1.0
    return e


def _unit(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def bisector_aim(origins: np.ndarray, sun_dir, target) -> np.ndarray:
    """aim point = origin + 100 * normalize(s_hat + normalize(target - origin))."""
    s = _unit(sun_dir)
    r = _unit(np.asarray(target, np.float64)[None, :] - origins)
    n = _unit(s[None, :] + r)
    return origins + 100.0 * n


def three_heliostats(reflectivity=0.9, slope_error=1e-3, sun_angle=4.65e-3, num_rays=1 << 20) -> Scene:
    sun = np.array([0.0, -1.0, 1.0])
    e = make_elements(4)
    origins = np.array([[-5.0, 5.0, 0.0], [0.0, 5.0, 0.0], [5.0, 5.0, 0.0]])
    e["origin"][:3] = origins
    e["aim_point"][:3] = bisector_aim(origins, sun, [0.0, 0.0, 10.0])
    e["width"][:3] = 1.0
    e["height"][:3] = 1.95
    e["surface"][:3] = SURFACE_FLAT
    e["reflectivity"][:3] = reflectivity
    e["slope_error"][:3] = slope_error
    e["origin"][3] = [0.0, 0.0, 10.0]
    e["aim_point"][3] = [0.0, 1.0, 10.0]
    e["width"][3] = 2.0
    e["height"][3] = 2.0
    e["surface"][3] = SURFACE_FLAT
    return Scene("three_heliostats", e, sun, SUN_PILLBOX, sun_angle, num_rays)


def single_parabolic(sun_sigma=2.5e-3, slope_error=1.5e-3, num_rays=1 << 24, sun_shape=SUN_GAUSSIAN) -> Scene:
    sun = np.array([0.0, 0.0, 1.0])
    e = make_elements(2)
    f = 100.0
    c = 1.0 / (2.0 * f)
    e["origin"][0] = [0.0, 100.0, 0.0]
    e["aim_point"][0] = bisector_aim(e["origin"][:1], sun, [0.0, 0.0, 100.0])[0]
    e["width"][0] = 10.0
    e["height"][0] = 10.0
    e["curv_x"][0] = c
    e["curv_y"][0] = c
    e["surface"][0] = SURFACE_PARABOLIC
    e["slope_error"][0] = slope_error
    e["origin"][1] = [0.0, 0.0, 100.0]
    e["aim_point"][1] = [0.0, -1.0, 100.0]
    e["width"][1] = 4.0   # 2 * radius
    e["height"][1] = 4.0  # full height, axis along +z
    e["surface"][1] = SURFACE_CYLINDER
    return Scene("single_parabolic", e, sun, sun_shape, sun_sigma, num_rays, {"focal_length": f})


def corridor(num_rays=1 << 20, sun=(0.8, 0.0, 1.0), sun_angle=4.65e-3, slope_error=0.0) -> Scene:
    """Two tall flat mirrors facing each other (x = -2 and x = +2, 20 m along z, 4 m along y) above
    a flat 4 x 4 m receiver facing up at z = -10.5: rays entering between the mirrors bounce back and
    forth several times, so paths reach the five-slot limit of the hit record."""
    e = make_elements(3)
    e["origin"][0] = [-2.0, 0.0, 0.0]
    e["aim_point"][0] = [1.0, 0.0, 0.0]
    e["origin"][1] = [2.0, 0.0, 0.0]
    e["aim_point"][1] = [-1.0, 0.0, 0.0]
    e["width"][:2] = 20.0
    e["height"][:2] = 4.0
    e["slope_error"][:2] = slope_error
    e["origin"][2] = [0.0, 0.0, -10.5]
    e["aim_point"][2] = [0.0, 0.0, 0.0]
    e["width"][2] = 4.0
    e["height"][2] = 4.0
    return Scene("corridor", e, np.asarray(sun, np.float64), SUN_PILLBOX, sun_angle, num_rays)


def radial_stagger(n=10000, r_min=100.0, r_max=800.0, mirror=10.0, seed=1) -> np.ndarray:
    """Heliostat base positions (z = 0) on a radial-stagger layout, truncated in ring order."""
    pitch = 1.2 * mirror * math.sqrt(2.0)
    # radial step chosen so that the rings between r_min and r_max hold at least n positions
    lo, hi = 1.0, 200.0
    for _ in range(60):
        step = 0.5 * (lo + hi)
        radii = np.arange(r_min, r_max + 1e-9, step)
        cap = sum(int(2 * math.pi * r // pitch) for r in radii)
        if cap >= n:
            lo = step
        else:
            hi = step
    step = lo
    pts = []
    rng = np.random.default_rng(seed)
    for i, r in enumerate(np.arange(r_min, r_max + 1e-9, step)):
        m = int(2 * math.pi * r // pitch)
        off = 0.5 if (i % 2) else 0.0
        ang = (np.arange(m) + off) * (2 * math.pi / m)
        ring = np.stack([r * np.sin(ang), r * np.cos(ang), np.zeros(m)], 1)
        pts.append(ring)
        if sum(len(p) for p in pts) >= n:
            break
    P = np.concatenate(pts, 0)[:n]
    P[:, :2] += rng.uniform(-0.5, 0.5, size=(n, 2))
    return P


def sun_vector(elevation_deg: float, azimuth_deg: float) -> np.ndarray:
    el, az = math.radians(elevation_deg), math.radians(azimuth_deg)
    return np.array([math.cos(el) * math.sin(az), math.cos(el) * math.cos(az), math.sin(el)])


def large_field(n_heliostats=10000, sun=None, slope_error=1.5e-3, sun_angle=4.65e-3, num_rays=1 << 28,
                seed=1, parabolic=False, focal_length=100.0) -> Scene:
    if sun is None:
        sun = sun_vector(45.0, 0.0)
    recv = np.array([0.0, 0.0, 200.0])
    P = radial_stagger(n_heliostats, seed=seed)
    e = make_elements(n_heliostats + 1)
    h = e[:n_heliostats]
    h["origin"] = P
    h["aim_point"] = bisector_aim(P, sun, recv)
    h["width"] = 10.0
    h["height"] = 10.0
    h["slope_error"] = slope_error
    if parabolic:
        h["surface"] = SURFACE_PARABOLIC
        h["curv_x"] = 1.0 / (2.0 * focal_length)
        h["curv_y"] = 1.0 / (2.0 * focal_length)
    else:
        h["surface"] = SURFACE_FLAT
    e["origin"][-1] = recv
    e["aim_point"][-1] = recv + np.array([0.0, -1.0, 0.0])
    e["width"][-1] = 16.0
    e["height"][-1] = 20.0
    e["surface"][-1] = SURFACE_CYLINDER
    return Scene("large_field", e, np.asarray(sun, np.float64), SUN_PILLBOX, sun_angle, num_rays,
                 {"n_heliostats": n_heliostats})


def reaim(elements: np.ndarray, sun) -> np.ndarray:
    """Copy of a field with every heliostat re-aimed for a new sun vector (receiver = last)."""
    e = elements.copy()
    recv = e["origin"][-1]
    e["aim_point"][:-1] = bisector_aim(e["origin"][:-1], sun, recv)
    return e


def batched_instances(n_instances=256, n_heliostats=10000, seed_sun=2, seed_rays=3, min_log2=20, max_log2=25):
    """Per-instance (sun vector, ray count) for the batched workload."""
    rs = np.random.default_rng(seed_sun)
    el = rs.uniform(10.0, 80.0, n_instances)
    az = rs.uniform(-120.0, 120.0, n_instances)
    rr = np.random.default_rng(seed_rays)
    counts = np.exp(rr.uniform(min_log2 * math.log(2), max_log2 * math.log(2), n_instances)).astype(np.int64)
    suns = np.stack([sun_vector(a, b) for a, b in zip(el, az)], 0)
    return suns, counts
