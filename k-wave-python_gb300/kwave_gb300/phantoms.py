"""Seeded synthetic initial-pressure phantoms and sensor layouts of the
reconstruction workloads (the reference ships no data for them)."""
from __future__ import annotations

import numpy as np


def vessel_phantom(n, rng, pml=20):
    """n x n p0 of 15 line segments (width 1-4 px, anti-aliased edges) and 5
    discs (radius 2-6 px), amplitudes U(0.5, 2), overlapping features taking
    the maximum, inside the central half of the region within the PML.

    A feature's value clip(w + 0.5 - distance, 0, 1) is zero more than
    w + 0.5 px from it, so each feature is evaluated only on its bounding box
    grown by w + 1 px: the same values as over the whole grid, at a fraction
    of the cost."""
    p0 = np.zeros((n, n))
    lo, hi = pml + 0.25 * (n - 2 * pml), n - pml - 0.25 * (n - 2 * pml)

    def box(xa, xb, ya, yb, pad):
        i0, i1 = max(0, int(np.floor(min(xa, xb) - pad))), min(n, int(np.ceil(max(xa, xb) + pad)) + 1)
        j0, j1 = max(0, int(np.floor(min(ya, yb) - pad))), min(n, int(np.ceil(max(ya, yb) + pad)) + 1)
        gx, gy = np.meshgrid(np.arange(i0, i1), np.arange(j0, j1), indexing="ij")
        return (slice(i0, i1), slice(j0, j1)), gx, gy

    for _ in range(15):
        x0, y0, x1, y1 = rng.uniform(lo, hi, 4)
        w = rng.uniform(1, 4) / 2
        sl, gx, gy = box(x0, x1, y0, y1, w + 1)
        vx, vy = x1 - x0, y1 - y0
        t = np.clip(((gx - x0) * vx + (gy - y0) * vy) / max(vx * vx + vy * vy, 1e-9), 0, 1)
        dist = np.hypot(gx - (x0 + t * vx), gy - (y0 + t * vy))
        p0[sl] = np.maximum(p0[sl], rng.uniform(0.5, 2) * np.clip(w + 0.5 - dist, 0, 1))
    for _ in range(5):
        cx, cy, r = rng.uniform(lo, hi), rng.uniform(lo, hi), rng.uniform(2, 6)
        sl, gx, gy = box(cx, cx, cy, cy, r + 1)
        p0[sl] = np.maximum(p0[sl], rng.uniform(0.5, 2) * np.clip(r + 0.5 - np.hypot(gx - cx, gy - cy), 0, 1))
    return p0


def circle_points(n_points, radius):
    """(2, n_points) Cartesian points on a circle about the grid centre, the
    layout of kwave.utils.mapgen.make_cart_circle with the first point at
    angle 0."""
    th = 2 * np.pi * np.arange(n_points) / n_points
    return np.stack([radius * np.cos(th), radius * np.sin(th)])
