"""How much of one canvas's painting could run concurrently: the dependency bound.

painty paints a canvas's stamps strictly in order (FootprintBrush::paintStroke over each
stroke, painty/renderer/FootprintBrush.hxx:206-268). Two stamps can run at the same time
without changing any result only when neither touches what the other reads or writes: a stamp
reads and writes the canvas and the brush's snapshot inside its grown box (its F x F box grown
by the radius and clipped to the canvas, FootprintBrush.hxx:278-319), and each stroke starts
from a clean pickup map (dip, :150-166). This module computes, for one canvas, the longest
chain of stamps that must stay ordered when the canvas is cut into G x G tiles and a stamp
waits only for the earlier stamps of other strokes whose grown boxes shared a tile with it:
the as-soon-as-possible schedule of that dependency graph with unlimited workers.

  serial work W      = sum of the stamps' costs (what one worker does today)
  critical path C    = the finish time of the ASAP schedule
  W / C              = the most any stroke-level scheduler could gain on this canvas

A stamp's cost is the batch kernel's cost model (SM cycles: a fixed part plus a part per
support-disc pixel). Stamp centres follow paintStroke's Catmull-Rom stepping (Spline.hxx:27-73)
in numpy (the schedule needs only the boxes).
"""
from __future__ import annotations

import math

import numpy as np

STAMP_FIXED = 7000.0      # SM cycles per stamp (the batch kernel's cost model)
STAMP_PER_PIXEL = 12.0    # SM cycles per support-disc pixel


def _footprint_side(radius: float) -> int:
    width = int(2.0 * math.ceil(radius) + 1.0)
    size_map = int(math.ceil(math.sqrt(2.0) * width))
    return width + 2 * ((size_map - width) // 2)


def stamp_centres(path: np.ndarray, spacing: float) -> np.ndarray:
    """Stamp centres of paintStroke along `path` at chord spacing `spacing`: (n, 2)."""
    p = np.asarray(path, dtype=np.float64)
    n = len(p)
    out = []
    for i in range(n - 1):
        pp, p0, p1, pn = p[max(i - 1, 0)], p[i], p[i + 1], p[min(i + 2, n - 1)]
        dist = float(np.hypot(*(p1 - p0)))
        steps = int(dist / spacing)
        if steps <= 0:
            continue
        t = np.arange(1, steps + 1) * spacing / dist
        t2, t3 = t * t, t * t * t
        b1 = -0.5 * t + t2 - 0.5 * t3
        b2 = 1.0 - 2.5 * t2 + 1.5 * t3
        b3 = 0.5 * t + 2.0 * t2 - 1.5 * t3
        b4 = -0.5 * t2 + 0.5 * t3
        out.append(np.outer(b1, pp) + np.outer(b2, p0) + np.outer(b3, p1) + np.outer(b4, pn))
    return np.concatenate(out) if out else np.zeros((0, 2))


def canvas_dependency_bound(rows: int, cols: int, strokes, tile: int = 32):
    """strokes: [(path, radius, spacing)] of one canvas, in painting order.
    Returns (stamps, serial work W, critical path C) with W and C in SM cycles."""
    tx, ty = (cols + tile - 1) // tile, (rows + tile - 1) // tile
    release = np.zeros(tx * ty)  # finish time of the latest stamp that touched each tile
    work = 0.0
    crit = 0.0
    nstamps = 0
    for path, radius, spacing in strokes:
        c = stamp_centres(path, spacing)
        n = len(c)
        if n == 0:
            continue
        F = _footprint_side(radius)
        wr = (F - 1) // 2
        disc = math.pi * (math.ceil(radius) + 0.5 + 0.7072) ** 2
        cost = STAMP_FIXED + STAMP_PER_PIXEL * disc
        # grown boxes (FootprintBrush.hxx:293-305), clipped, as tile rectangles
        x0 = np.maximum(np.trunc(c[:, 0] - wr - radius), 0)
        y0 = np.maximum(np.trunc(c[:, 1] - wr - radius), 0)
        x1 = np.minimum(np.trunc(c[:, 0] + wr + radius), cols - 1)
        y1 = np.minimum(np.trunc(c[:, 1] + wr + radius), rows - 1)
        live = (x0 <= x1) & (y0 <= y1)
        tx0, ty0 = (x0 // tile).astype(np.int64), (y0 // tile).astype(np.int64)
        tx1, ty1 = (x1 // tile).astype(np.int64), (y1 // tile).astype(np.int64)
        # every (stamp, tile) pair
        w = np.where(live, tx1 - tx0 + 1, 0)
        h = np.where(live, ty1 - ty0 + 1, 0)
        cnt = w * h
        j = np.repeat(np.arange(n), cnt)
        k = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        ti = tx0[j] + k % w[j]
        tj = ty0[j] + k // w[j]
        tid = tj * tx + ti

        def inside(s, a, b):  # tile (a, b) inside stamp s's tile rectangle
            ok = (s >= 0) & (s < n)
            s2 = np.clip(s, 0, n - 1)
            return ok & live[s2] & (a >= tx0[s2]) & (a <= tx1[s2]) & (b >= ty0[s2]) & (b <= ty1[s2])

        enter = ~inside(j - 1, ti, tj)
        leave = ~inside(j + 1, ti, tj)
        # a stamp starts after its predecessor and after the earlier strokes' last stamps on
        # the tiles it enters; the stroke's own earlier visits finished before its predecessor
        ready = np.full(n, -np.inf)
        np.maximum.at(ready, j[enter], release[tid[enter]])
        idx = np.arange(n)
        end = cost * (idx + 1) + np.maximum.accumulate(np.maximum(ready, 0.0) - cost * idx)
        np.maximum.at(release, tid[leave], end[j[leave]])
        work += cost * n
        crit = max(crit, float(end[-1]))
        nstamps += n
    return nstamps, work, crit
