"""The dependency bound of a canvas's strokes (painty_gb300.schedule) against a brute-force
as-soon-as-possible schedule over every pair of stamps that share a tile."""
import math

import numpy as np

from painty_gb300 import schedule, workloads


def _brute(rows, cols, strokes, tile):
    stamps = []  # (stroke, cost, tile set)
    for si, (path, r, sp) in enumerate(strokes):
        F = schedule._footprint_side(r)
        wr = (F - 1) // 2
        cost = schedule.STAMP_FIXED + schedule.STAMP_PER_PIXEL * math.pi * (math.ceil(r) + 0.5 + 0.7072) ** 2
        for cx, cy in schedule.stamp_centres(path, sp):
            x0, y0 = max(math.trunc(cx - wr - r), 0), max(math.trunc(cy - wr - r), 0)
            x1, y1 = min(math.trunc(cx + wr + r), cols - 1), min(math.trunc(cy + wr + r), rows - 1)
            tiles = {(a, b) for a in range(x0 // tile, x1 // tile + 1)
                     for b in range(y0 // tile, y1 // tile + 1)} if x0 <= x1 and y0 <= y1 else set()
            stamps.append((si, cost, tiles))
    end = []
    for i, (si, cost, tiles) in enumerate(stamps):
        start = 0.0
        for j in range(i):
            sj, _, tj = stamps[j]
            if sj == si or tiles & tj:
                start = max(start, end[j])
        end.append(start + cost)
    return len(stamps), sum(c for _, c, _ in stamps), max(end)


def test_dependency_bound_matches_brute_force():
    rows, cols = 70, 90
    ss = workloads.strokes(cols, rows, 6, seed=5, rmin=3, rmax=9)
    strokes = [(s.path, s.radius, s.spacing * 4) for s in ss]
    for tile in (8, 16, 32):
        n, W, C = schedule.canvas_dependency_bound(rows, cols, strokes, tile=tile)
        bn, bW, bC = _brute(rows, cols, strokes, tile)
        assert n == bn and np.isclose(W, bW) and np.isclose(C, bC), (tile, C, bC)
        assert C <= W


def test_stamp_centres_match_the_oracle(oracle):
    ss = workloads.strokes(200, 150, 3, seed=8)
    for s in ss:
        got = schedule.stamp_centres(s.path, s.spacing)
        want = oracle.stroke_stamps(s.path, s.spacing)[:, :2]
        assert got.shape == want.shape and np.allclose(got, want, atol=1e-9)
