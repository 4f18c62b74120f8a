"""Host-side placement of independent work across GPUs (one process per GPU).

A canvas's stamps are globally ordered, so a canvas never spans GPUs; canvases (and the
composite's pixel rows) are independent, so they are partitioned with no data exchange.
Every rank computes the same assignment from the same inputs.
"""
from __future__ import annotations

import heapq

import numpy as np


def canvas_shard(work, rank: int, world: int) -> list[int]:
    """Canvases of `rank` under a longest-processing-time assignment of `work` (one estimate
    per canvas) to `world` ranks: heaviest first onto the least-loaded rank, ties by rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    work = np.asarray(work, dtype=np.float64)
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    heap = [(0.0, r) for r in range(world)]
    mine = []
    for i in order:
        load, r = heapq.heappop(heap)
        if r == rank:
            mine.append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    return sorted(mine)


def row_shard(rows: int, rank: int, world: int) -> tuple[int, int]:
    """Rows [lo, hi) of `rank` when an image's rows are split into `world` near-equal bands."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    return rows * rank // world, rows * (rank + 1) // world


def stroke_work(path, radius: float, spacing: float) -> float:
    """Work estimate of one stroke: its stamps times the stamp's support-disc pixels."""
    p = np.asarray(path, dtype=np.float64)
    n = float(np.sum(np.floor(np.linalg.norm(np.diff(p, axis=0), axis=1) / spacing)))
    return n * np.pi * (np.sqrt(2.0) * (radius + 1.0)) ** 2
