"""Receiver flux maps from hit records (host side).

Restates the reference's post-processing metric (scripts/post_processing/flux_map_calculator.py:
135-179 and plot_flux_map_gpu.py:174-210): stage-2 (receiver) records are projected to receiver
coordinates, binned on an nx x ny grid and scaled by DNI * sun-plane area / rays / bin area.
  flat receiver      local (x, y) over [-w/2, w/2] x [-h/2, h/2] in the receiver's own axes
  cylinder receiver  angle around the axis in [0, 2 pi) (measured from the local x axis) and the
                     axial coordinate over [-H/2, H/2]; cap hits (|axial| at H/2) are excluded
Out-of-range bins are clipped as in the reference script.
"""
from __future__ import annotations

import math

import numpy as np

from .scenes import SURFACE_CYLINDER


def element_axes(e) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Local x, y, z axes of an element (rows of the global-to-local matrix, lib/math_util.h:41-59)."""
    o = np.asarray(e["origin"], np.float64)
    n = np.asarray(e["aim_point"], np.float64) - o
    ln = np.linalg.norm(n)
    n = n / ln if ln > 0 else np.zeros(3)
    a, b, g = math.atan2(n[0], n[2]), math.asin(n[1]), float(e["zrot_deg"]) * math.pi / 180.0
    ca, sa, cb, sb, cg, sg = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(g), math.sin(g)
    x = np.array([ca * cg + sa * sb * sg, -cb * sg, -sa * cg + ca * sb * sg])
    y = np.array([ca * sg - sa * sb * cg, cb * cg, -sa * sg - ca * sb * cg])
    z = np.array([sa * cb, sb, ca * cb])
    return x, y, z


def receiver_coords(points: np.ndarray, receiver) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(u, v, keep) of receiver hit points: flat (x, y); cylinder (angle, axial), keep = side hits."""
    x, y, z = element_axes(receiver)
    t = points - np.asarray(receiver["origin"], np.float64)[None, :]
    if int(receiver["surface"]) == SURFACE_CYLINDER:
        r = 0.5 * float(receiver["width"])
        lx, ly, lz = t @ x, t @ y, t @ z
        ang = np.mod(np.arctan2(lz, lx), 2.0 * np.pi)
        half = 0.5 * float(receiver["height"])
        # cap hits sit at |axial| = half (to float rounding of the trace); side hits strictly inside
        keep = np.abs(ly) < half - 1e-4 * max(half, r)
        return ang, ly, keep
    return t @ x, t @ y, np.ones(len(points), bool)


def flux_map_from_hits(hits: np.ndarray, receiver, num_rays: int, nx: int = 100, ny: int = 100,
                       dni: float = 1000.0, sun_area: float | None = None) -> np.ndarray:
    """hits: [N, 5, 4] records {stage, x, y, z}.  Returns the [nx, ny] flux map (W/m^2 when sun_area
    is given, otherwise per-ray weight 1/num_rays)."""
    h = np.asarray(hits).reshape(-1, 4)
    pts = h[h[:, 0] == 2.0][:, 1:4].astype(np.float64)
    u, v, keep = receiver_coords(pts, receiver)
    u, v = u[keep], v[keep]
    w, H = float(receiver["width"]), float(receiver["height"])
    if int(receiver["surface"]) == SURFACE_CYLINDER:
        bx = np.floor(u * nx / (2.0 * np.pi)).astype(np.int64)
        by = np.floor((v + H / 2) * ny / H).astype(np.int64)
        bin_area = (2.0 * np.pi * 0.5 * w / nx) * (H / ny)
    else:
        bx = np.floor((u + w / 2) * nx / w).astype(np.int64)
        by = np.floor((v + H / 2) * ny / H).astype(np.int64)
        bin_area = (w / nx) * (H / ny)
    bx = np.clip(bx, 0, nx - 1)
    by = np.clip(by, 0, ny - 1)
    per_ray = (dni * sun_area / num_rays) if sun_area is not None else 1.0 / num_rays
    f = np.zeros((nx, ny), np.float64)
    np.add.at(f, (bx, by), per_ray / bin_area)
    return f


def flux_l2(f: np.ndarray, f_ref: np.ndarray) -> float:
    """Relative L2 error ||F - F_ref|| / ||F_ref||."""
    den = float(np.linalg.norm(f_ref))
    return float(np.linalg.norm(f - f_ref)) / den if den > 0 else float(np.linalg.norm(f))


def sun_plane_area(sun_plane: np.ndarray) -> float:
    """Area of the sun-plane parallelogram from csp_get_sun_plane's output (v0, v1, v3)."""
    v0, v1, v3 = sun_plane[3:6].astype(np.float64), sun_plane[6:9].astype(np.float64), sun_plane[12:15].astype(np.float64)
    return float(np.linalg.norm(np.cross(v1 - v0, v3 - v0)))
