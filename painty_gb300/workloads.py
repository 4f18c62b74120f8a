"""Seeded synthetic workloads for the paint path (no files, no network).

The reference paints from a scanned footprint PNG, measured pigments and user strokes; these
generators stand in for them with fixed seeds:

* footprint_image   64x64 imprint footprint: radial falloff x value noise, values in [0, 1]
* pigments          base pigments, K ~ U[0.01, 5], S ~ U[0.05, 3] per channel
* stroke_paints     per-stroke paint: Dirichlet(0.3) weights mixed as PaintMixer::mixSinglePaint
* strokes           Catmull-Rom control polygons (8 points uniform on the canvas), radii
* composite_stack   L stacked paint layers for the composite stress case
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def footprint_image(seed: int = 7, size: int = 64, cells: int = 8) -> np.ndarray:
    """Radial falloff (1 - (d/R)^2, clipped) times smoothstep-interpolated value noise."""
    rng = np.random.default_rng(seed)
    lattice = rng.random((cells + 1, cells + 1))
    coord = (np.arange(size) + 0.5) / size * cells
    i0 = np.minimum(coord.astype(np.int64), cells - 1)
    t = coord - i0
    t = t * t * (3.0 - 2.0 * t)
    a = lattice[i0][:, i0]
    b = lattice[i0][:, i0 + 1]
    c = lattice[i0 + 1][:, i0]
    d = lattice[i0 + 1][:, i0 + 1]
    tx = t[None, :]
    ty = t[:, None]
    noise = (a * (1 - tx) + b * tx) * (1 - ty) + (c * (1 - tx) + d * tx) * ty
    r = size / 2.0
    yy, xx = np.mgrid[0:size, 0:size]
    dist = np.hypot(xx + 0.5 - r, yy + 0.5 - r) / r
    falloff = np.clip(1.0 - dist * dist, 0.0, 1.0)
    return np.ascontiguousarray(falloff * noise)


def stroke_texture(seed: int = 13, rows: int = 32, cols: int = 128, cells: int = 8) -> np.ndarray:
    """Thickness texture of a brush-stroke sample (stands in for painty's scanned stroke
    samples): a bristle profile across the width (rows) times smoothed value noise along the
    length, values in [0, 1], tapering to 0 at the stroke's ends and sides."""
    rng = np.random.default_rng(seed)
    across = (np.arange(rows) + 0.5) / rows
    bristles = 0.6 + 0.4 * rng.random(rows)
    side = np.clip(1.0 - (2.0 * across - 1.0) ** 4, 0.0, 1.0) * bristles
    lattice = rng.random(cells + 1)
    x = (np.arange(cols) + 0.5) / cols * cells
    i0 = np.minimum(x.astype(np.int64), cells - 1)
    t = x - i0
    t = t * t * (3.0 - 2.0 * t)
    along = lattice[i0] * (1 - t) + lattice[i0 + 1] * t
    along *= np.clip(np.minimum(x, cells - x) / 0.75, 0.0, 1.0)
    return np.ascontiguousarray(side[:, None] * along[None, :])


def pigments(seed: int = 11, n: int = 14):
    rng = np.random.default_rng(seed)
    K = rng.uniform(0.01, 5.0, (n, 3))
    S = rng.uniform(0.05, 3.0, (n, 3))
    return K, S


def mix_single_paint_np(weights: np.ndarray, K: np.ndarray, S: np.ndarray):
    """PaintMixer::mixSinglePaint (PaintMixer.cxx:327-355) with its accumulation order."""
    wsum = 0.0
    for w in weights:
        wsum += float(w)
    norm = 1.0 if abs(wsum - 1.0) < 10e-6 else 1.0 / wsum
    k = np.zeros(3)
    s = np.zeros(3)
    for l in range(len(weights)):
        for i in range(3):
            k[i] += norm * float(weights[l]) * K[l, i]
            s[i] += norm * float(weights[l]) * S[l, i]
    return k, s


def mix_paints_np(weights: np.ndarray, K: np.ndarray, S: np.ndarray):
    """mix_single_paint_np for many weight rows at once (weights (n, pigments)), with the same
    accumulation order per row: equal to it bit for bit."""
    W = np.asarray(weights, dtype=np.float64)
    wsum = np.cumsum(W, axis=1)[:, -1]
    norm = np.where(np.abs(wsum - 1.0) < 10e-6, 1.0, 1.0 / wsum)
    nw = norm[:, None] * W
    k = np.cumsum(nw[:, :, None] * K[None, :, :], axis=1)[:, -1, :]
    s = np.cumsum(nw[:, :, None] * S[None, :, :], axis=1)[:, -1, :]
    return k, s


@dataclass
class Stroke:
    path: np.ndarray  # (n, 2) control points, x then y
    radius: float
    K: np.ndarray
    S: np.ndarray
    spacing: float


def strokes(width: int, height: int, n: int, seed: int = 3, rmin: float = 8.0,
            rmax: float = 32.0, points: int = 8, log_radius: bool = False,
            spacing_factor: float = 0.25, pigment_seed: int = 11) -> list[Stroke]:
    """Strokes through `points` control points uniform on the canvas; radius U[rmin, rmax]
    (log-uniform with log_radius); paint = Dirichlet(0.3) mix of the base pigments; stamp
    spacing spacing_factor * radius."""
    rng = np.random.default_rng(seed)
    PK, PS = pigments(pigment_seed)
    out = []
    for _ in range(n):
        path = np.stack([rng.uniform(0, width, points), rng.uniform(0, height, points)], axis=1)
        if log_radius:
            r = float(np.exp(rng.uniform(np.log(rmin), np.log(rmax))))
        else:
            r = float(rng.uniform(rmin, rmax))
        w = rng.dirichlet(np.full(len(PK), 0.3))
        k, s = mix_single_paint_np(w, PK, PS)
        out.append(Stroke(np.ascontiguousarray(path), r, k, s, spacing_factor * r))
    return out


def substrate(rows: int, cols: int, seed: int = 5, lo: float = 0.80, hi: float = 0.95):
    """R0 ~ U[lo, hi] per channel per pixel, interleaved (rows, cols, 3)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, (rows, cols, 3))


def composite_stack(rows: int, cols: int, layers: int = 8, seed: int = 1,
                    dtype=np.float32):
    """Planar layer stack for the composite stress case.

    Returns K, S of shape (L, 3, rows, cols), V of shape (L, rows, cols) and R0 of shape
    (3, rows, cols): K ~ U[0.01, 5], S ~ U[0.05, 3], h ~ U[0, 0.5] with 20% of pixels at
    h = 0 and 5% with h ~ U[1e-7, 1e-4] (the small-argument branch), R0 ~ U[0.8, 0.95].
    """
    rng = np.random.default_rng(seed)
    K = rng.uniform(0.01, 5.0, (layers, 3, rows, cols)).astype(dtype)
    S = rng.uniform(0.05, 3.0, (layers, 3, rows, cols)).astype(dtype)
    V = rng.uniform(0.0, 0.5, (layers, rows, cols))
    sel = rng.random((layers, rows, cols))
    V[sel < 0.20] = 0.0
    small = (sel >= 0.20) & (sel < 0.25)
    V[small] = rng.uniform(1e-7, 1e-4, int(small.sum()))
    V = V.astype(dtype)
    R0 = rng.uniform(0.8, 0.95, (3, rows, cols)).astype(dtype)
    return K, S, V, R0


def paint_config0(canvas, brush, strokes_list, on_stroke=None):
    """Config-0 style painting: per stroke setRadius, dip, paintStroke at the stroke spacing."""
    total = 0
    for i, s in enumerate(strokes_list):
        brush.setRadius(s.radius)
        brush.dip((s.K, s.S))
        total += brush.paintStroke(s.path, canvas, spacing=s.spacing)
        if on_stroke is not None:
            on_stroke(i)
    return total


def batch_canvases(n: int, seed: int = 2, smin: float = 256, smax: float = 2048,
                   strokes_min: int = 50, strokes_max: int = 2000, rmin: float = 4.0,
                   rmax: float = 64.0, max_strokes=None, pigment_seed: int = 11):
    """The batching workload: n canvases with side log-uniform in [smin, smax] and aspect
    U[0.5, 2]; strokes per canvas log-uniform in [strokes_min, strokes_max] (optionally capped
    at max_strokes); radius log-uniform in [rmin, rmax]; 8 uniform control points; spacing
    0.25 r; Dirichlet(0.3) paints; substrate R0 ~ U[0.80, 0.95]. Canvas c is drawn from its
    own generator (seeded with (seed, c)), so canvases are independent of one another.
    Returns [(rows, cols, R0 (rows, cols, 3) float32)] and strokes as
    (canvas, path, radius, spacing, K, S)."""
    PK, PS = pigments(pigment_seed)
    canvases, strokes_out = [], []
    for c in range(n):
        rng = np.random.default_rng([seed, c])
        side = float(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        asp = rng.uniform(0.5, 2.0)
        cols, rows = int(side * np.sqrt(asp)), int(side / np.sqrt(asp))
        ns = int(np.exp(rng.uniform(np.log(strokes_min), np.log(strokes_max))))
        if max_strokes is not None:
            ns = min(ns, max_strokes)
        r0 = (0.80 + 0.15 * rng.random((rows, cols, 3), dtype=np.float32)).astype(np.float32)
        canvases.append((rows, cols, r0))
        u = rng.random((ns, 8, 2))
        paths = u * np.array([cols, rows], dtype=np.float64)
        radii = np.exp(rng.uniform(np.log(rmin), np.log(rmax), ns))
        K, S = mix_paints_np(rng.dirichlet(np.full(len(PK), 0.3), ns), PK, PS)
        for j in range(ns):
            r = float(radii[j])
            strokes_out.append((c, np.ascontiguousarray(paths[j]), r, 0.25 * r, K[j], S[j]))
    return canvases, strokes_out
