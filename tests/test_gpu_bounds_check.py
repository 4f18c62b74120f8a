"""The bounds-checked build on tiny canvases (GPU).

PAINTY_BOUNDS_CHECK=1 makes the package load libpainty_gb300_checked.so, whose stamp kernels
test every computed index against its buffer before the access and report an out-of-range
access as an error instead of faulting. On 13 x 9 canvases with radii 1, 2 and 4 -- stamps
half outside the canvas, on the edges where truncation duplicates a column or row, with and
without the snapshot, single calls and batches -- it must report nothing and paint exactly what
the oracle paints (F64 bit for bit, FP32 within the stamp tests' tolerance), twice alike.
"""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

PROBE = r"""
import json, sys
import numpy as np
sys.path.insert(0, ROOT)
import painty_gb300 as pg
from oracle.oracle import Oracle
from painty_gb300 import workloads

assert pg.bounds_checked()
o = Oracle()
fp = workloads.footprint_image(seed=7)
rows, cols = 9, 13
out = {"single": {}, "batch": {}, "f32_rel": 0.0}


def session(seed):
    rng = np.random.default_rng(seed)
    strokes = []
    for k in range(4):
        K, S = rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)
        st = np.stack([rng.uniform(-6, cols + 6, 30), rng.uniform(-6, rows + 6, 30),
                       rng.uniform(-7, 7, 30)], axis=1)
        st[:3, :2] = [[0.5, 0.25], [12.7, 8.9], [-0.3, 4.0]]
        strokes.append((K, S, st))
    return rng.uniform(0.8, 0.95, (rows, cols, 3)), strokes


def paint(storage, r, snap, seed):
    r0, strokes = session(seed)
    c = pg.Canvas(rows, cols, storage)
    c.upload("R0", r0)
    b = pg.FootprintBrush(r, fp)
    b.setPickupRate(0.05)
    b.setDepositionRate(0.1)
    b.setUseSnapshotBuffer(snap)
    oc = o.canvas(rows, cols)
    oc.set("R0", r0)
    ob = o.brush(r, fp)
    ob.set_rates(0.05, 0.1)
    ob.set_snapshot(snap)
    for K, S, st in strokes:
        b.dip((K, S))
        ob.dip(K, S)
        b.stamps(st, c)
        ob.stamps(oc, st)
    return c, oc


for r in (1.0, 2.0, 4.0):
    for snap in (True, False):
        c, oc = paint("f64", r, snap, int(r * 10) + snap)
        c2, _ = paint("f64", r, snap, int(r * 10) + snap)
        out["single"][f"{r}/{snap}"] = all(
            np.array_equal(c.download(p), oc.get(p)) and np.array_equal(c.download(p), c2.download(p))
            for p in ("K", "S", "V"))
        c, oc = paint("f32", r, snap, int(r * 10) + snap)
        for p in ("K", "S", "V"):
            g, w = c.download(p), oc.get(p)
            out["f32_rel"] = max(out["f32_rel"],
                                 float((np.abs(g - w) / np.maximum(np.abs(w), 1.0)).max()))

# batches of tiny canvases, strokes along paths that leave the canvas
rng = np.random.default_rng(3)
specs = [(rows, cols), (cols, rows), (rows, rows)]
strokes = []
for ci, (rr, cc) in enumerate(specs):
    for _ in range(3):
        path = np.stack([rng.uniform(-4, cc + 4, 5), rng.uniform(-4, rr + 4, 5)], axis=1)
        r = float(rng.choice([1.0, 2.0, 4.0]))
        strokes.append((ci, path, r, 0.25 * r, rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)))
for storage in ("f64", "f16"):
    cs, bs = [], []
    for rr, cc in specs:
        cs.append(pg.Canvas(rr, cc, storage))
        b = pg.FootprintBrush(2.0, fp)
        b.setPickupRate(0.05)
        b.setDepositionRate(0.1)
        bs.append(b)
    pg.paint_batch(cs, bs, strokes)
    same = True
    if storage == "f64":
        for ci, (rr, cc) in enumerate(specs):
            oc = o.canvas(rr, cc)
            ob = o.brush(2.0, fp)
            ob.set_rates(0.05, 0.1)
            for cj, path, r, sp, K, S in strokes:
                if cj == ci:
                    ob.set_radius(r)
                    ob.dip(K, S)
                    ob.paint_stroke(oc, path, sp)
            same = same and all(np.array_equal(cs[ci].download(p), oc.get(p)) for p in ("K", "S", "V"))
    out["batch"][storage] = same
print(json.dumps(out))
"""


def test_bounds_checked_build_on_tiny_canvases():
    from test_gpu_stamps import F32_REL_TOL
    env = dict(__import__("os").environ, PAINTY_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {str(ROOT)!r}\n" + PROBE],
                       capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(res["single"].values()), res
    assert all(res["batch"].values()), res
    assert res["f32_rel"] <= F32_REL_TOL, res
