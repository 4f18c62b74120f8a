"""Batched painting (painty_paint_batch) vs sequential painty calls and the oracle (GPU)."""
import numpy as np
import pytest

from painty_gb300 import workloads

pytestmark = pytest.mark.gpu


def _canvases(rng, n, smin=40, smax=160):
    out = []
    for _ in range(n):
        side = float(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        asp = rng.uniform(0.5, 2.0)
        out.append((max(8, int(side / np.sqrt(asp))), max(8, int(side * np.sqrt(asp)))))
    return out


def _session(rng, sizes, strokes_per=(2, 6), rmin=1.5, rmax=20.0):
    strokes = []
    for ci, (rows, cols) in enumerate(sizes):
        for _ in range(int(rng.integers(*strokes_per))):
            path = np.stack([rng.uniform(-5, cols + 5, 6), rng.uniform(-5, rows + 5, 6)], axis=1)
            r = float(np.exp(rng.uniform(np.log(rmin), np.log(rmax))))
            strokes.append((ci, path, r, 0.25 * r if rng.random() < 0.7 else 1.0,
                            rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)))
    # interleave the canvases at random, each canvas's strokes keeping their order
    queues = {}
    for s in strokes:
        queues.setdefault(s[0], []).append(s)
    seq = []
    while queues:
        ci = list(queues)[int(rng.integers(len(queues)))]
        seq.append(queues[ci].pop(0))
        if not queues[ci]:
            del queues[ci]
    return seq


def _setup(pg, sizes, storage, rng_seed=7, snap=True):
    rng = np.random.default_rng(rng_seed)
    fp = workloads.footprint_image(seed=7)
    cs, bs, r0s = [], [], []
    for rows, cols in sizes:
        c = pg.Canvas(rows, cols, storage)
        r0 = rng.uniform(0.8, 0.95, (rows, cols, 3))
        c.upload("R0", r0)
        b = pg.FootprintBrush(3.0, fp)
        b.setPickupRate(0.05)
        b.setDepositionRate(0.1)
        b.setUseSnapshotBuffer(snap)
        cs.append(c)
        bs.append(b)
        r0s.append(r0)
    return cs, bs, r0s


# radii up to 20; and 40-75, whose cell maps do not fit in shared memory beside the
# support-disc list (global cell maps)
@pytest.mark.parametrize("snap,rmin,rmax", [(True, 1.5, 20.0), (False, 1.5, 20.0),
                                            (True, 40.0, 75.0)])
def test_batch_f64_equals_sequential_and_oracle(pg, oracle, snap, rmin, rmax):
    rng = np.random.default_rng(11 + snap)
    if rmax > 30:
        sizes = _canvases(rng, 3, smin=120, smax=220)
        strokes = _session(rng, sizes, strokes_per=(2, 4), rmin=rmin, rmax=rmax)
    else:
        sizes = _canvases(rng, 7)
        strokes = _session(rng, sizes)
    cs, bs, r0s = _setup(pg, sizes, "f64", snap=snap)
    n = pg.paint_batch(cs, bs, strokes)
    # sequential painty calls through the single-canvas entry points
    cs2, bs2, _ = _setup(pg, sizes, "f64", snap=snap)
    n2 = 0
    for ci, path, r, spacing, K, S in strokes:
        bs2[ci].setRadius(r)
        bs2[ci].dip((K, S))
        n2 += bs2[ci].paintStroke(path, cs2[ci], spacing=spacing)
    assert n == n2
    fp = workloads.footprint_image(seed=7)
    for ci, (rows, cols) in enumerate(sizes):
        oc = oracle.canvas(rows, cols)
        oc.set("R0", r0s[ci])
        ob = oracle.brush(3.0, fp)
        ob.set_rates(0.05, 0.1)
        ob.set_snapshot(snap)
        for cj, path, r, spacing, K, S in strokes:
            if cj != ci:
                continue
            ob.set_radius(r)
            ob.dip(K, S)
            ob.paint_stroke(oc, path, spacing)
        for p in ("K", "S", "V"):
            a = cs[ci].download(p)
            assert np.array_equal(a, cs2[ci].download(p)), (ci, p)
            assert np.array_equal(a, oc.get(p)), (ci, p, "oracle")
        # the brush keeps the last stroke's pickup map, as the sequential calls leave it
        assert np.array_equal(bs[ci].getPickupMap("V"), bs2[ci].getPickupMap("V"))
        assert bs[ci].info() == bs2[ci].info()


@pytest.mark.parametrize("cluster", ["1", "2"])
def test_batch_forced_cluster_large_radii_f64(pg, oracle, monkeypatch, cluster):
    """One CTA per canvas (and a 2-CTA cluster) with radii 40-75, whose cell maps live in
    global memory beside the pickup map and owner table in shared or global memory: F64
    bit-exact against the oracle."""
    monkeypatch.setenv("PAINTY_BATCH_CLUSTER", cluster)
    rng = np.random.default_rng(21)
    sizes = _canvases(rng, 4, smin=120, smax=220)
    strokes = _session(rng, sizes, strokes_per=(2, 4), rmin=40.0, rmax=75.0)
    cs, bs, r0s = _setup(pg, sizes, "f64")
    pg.paint_batch(cs, bs, strokes)
    assert pg.batch_last_shape()[0] == int(cluster)
    fp = workloads.footprint_image(seed=7)
    for ci, (rows, cols) in enumerate(sizes):
        oc = oracle.canvas(rows, cols)
        oc.set("R0", r0s[ci])
        ob = oracle.brush(3.0, fp)
        ob.set_rates(0.05, 0.1)
        for cj, path, r, spacing, K, S in strokes:
            if cj == ci:
                ob.set_radius(r)
                ob.dip(K, S)
                ob.paint_stroke(oc, path, spacing)
        for p in ("K", "S", "V"):
            assert np.array_equal(cs[ci].download(p), oc.get(p)), (ci, p)


# 512-thread CTAs (two per SM): radii up to 20 with and without the snapshot, and 35-50
# (footprint sides up to 143, global cell maps), alone and as 2-CTA clusters
@pytest.mark.parametrize("snap,rmin,rmax,cluster", [(True, 1.5, 20.0, "1"), (False, 1.5, 20.0, "1"),
                                                    (True, 35.0, 50.0, "1"), (True, 1.5, 20.0, "2")])
def test_batch_512_threads_f64(pg, oracle, monkeypatch, snap, rmin, rmax, cluster):
    monkeypatch.setenv("PAINTY_BATCH_THREADS", "512")
    monkeypatch.setenv("PAINTY_BATCH_CLUSTER", cluster)
    rng = np.random.default_rng(31 + snap)
    sizes = _canvases(rng, 5, smin=90, smax=200)
    strokes = _session(rng, sizes, strokes_per=(2, 5), rmin=rmin, rmax=rmax)
    cs, bs, r0s = _setup(pg, sizes, "f64", snap=snap)
    pg.paint_batch(cs, bs, strokes)
    assert pg.batch_last_shape()[0] == int(cluster) and pg.batch_last_shape()[2] == 512
    fp = workloads.footprint_image(seed=7)
    for ci, (rows, cols) in enumerate(sizes):
        oc = oracle.canvas(rows, cols)
        oc.set("R0", r0s[ci])
        ob = oracle.brush(3.0, fp)
        ob.set_rates(0.05, 0.1)
        ob.set_snapshot(snap)
        for cj, path, r, spacing, K, S in strokes:
            if cj == ci:
                ob.set_radius(r)
                ob.dip(K, S)
                ob.paint_stroke(oc, path, spacing)
        for p in ("K", "S", "V"):
            assert np.array_equal(cs[ci].download(p), oc.get(p)), (ci, p)


@pytest.mark.parametrize("split", ["8:1", "4:2", "2:1"])
def test_batch_split_launch_f64(pg, oracle, monkeypatch, split):
    """The heaviest canvases on a launch of their own (clusters of 8, 4 or 2), the rest next to
    it on a side stream: F64 bit-exact against the oracle, and reported."""
    monkeypatch.setenv("PAINTY_BATCH_SPLIT", split)
    rng = np.random.default_rng(51)
    sizes = _canvases(rng, 6, smin=80, smax=180)
    strokes = _session(rng, sizes, strokes_per=(2, 5), rmin=2.0, rmax=18.0)
    cs, bs, r0s = _setup(pg, sizes, "f64")
    pg.paint_batch(cs, bs, strokes)
    ch, h = (int(x) for x in split.split(":"))
    assert pg.batch_last_split() == (ch, h)
    fp = workloads.footprint_image(seed=7)
    for ci, (rows, cols) in enumerate(sizes):
        oc = oracle.canvas(rows, cols)
        oc.set("R0", r0s[ci])
        ob = oracle.brush(3.0, fp)
        ob.set_rates(0.05, 0.1)
        for cj, path, r, spacing, K, S in strokes:
            if cj == ci:
                ob.set_radius(r)
                ob.dip(K, S)
                ob.paint_stroke(oc, path, spacing)
        for p in ("K", "S", "V"):
            assert np.array_equal(cs[ci].download(p), oc.get(p)), (ci, p)


def test_batch_512_threads_large_boxes_equal_1024(pg, monkeypatch):
    """Boxes up to side 255 fit 512-thread CTAs (radius 70: side 199, its edge duplicates in
    waves): the same results as 1024-thread CTAs, bit for bit."""
    rng = np.random.default_rng(41)
    sizes = _canvases(rng, 2, smin=150, smax=200)
    strokes = _session(rng, sizes, strokes_per=(1, 2), rmin=70.0, rmax=70.0)
    out = {}
    for nt in ("512", "1024"):
        monkeypatch.setenv("PAINTY_BATCH_THREADS", nt)
        cs, bs, _ = _setup(pg, sizes, "f32")
        pg.paint_batch(cs, bs, strokes)
        assert pg.batch_last_shape()[2] == int(nt)
        out[nt] = [[c.download(p) for p in ("K", "S", "V")] for c in cs]
    for a, b in zip(out["512"], out["1024"]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_batch_f32_close_to_sequential(pg):
    rng = np.random.default_rng(5)
    sizes = _canvases(rng, 12, 64, 300)
    strokes = _session(rng, sizes, (3, 9), 2.0, 40.0)
    cs, bs, _ = _setup(pg, sizes, "f32")
    pg.paint_batch(cs, bs, strokes)
    cs2, bs2, _ = _setup(pg, sizes, "f32")
    for ci, path, r, spacing, K, S in strokes:
        bs2[ci].setRadius(r)
        bs2[ci].dip((K, S))
        bs2[ci].paintStroke(path, cs2[ci], spacing=spacing)
    for ci in range(len(sizes)):
        for p in ("K", "S", "V"):
            a, b = cs[ci].download(p), cs2[ci].download(p)
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1.0)
            assert rel.max() <= 1e-4, (ci, p, rel.max())


def test_batch_then_single_calls_continue(pg, oracle):
    """After a batch, the canvas and brush continue exactly as after sequential calls."""
    rng = np.random.default_rng(9)
    sizes = [(50, 70)]
    strokes = _session(rng, sizes, (3, 4))
    cs, bs, r0s = _setup(pg, sizes, "f64")
    pg.paint_batch(cs, bs, strokes)
    extra = np.array([[10.5, 12.5, 0.3], [20.25, 18.0, 1.0]])
    bs[0].stamps(extra, cs[0])
    fp = workloads.footprint_image(seed=7)
    oc = oracle.canvas(50, 70)
    oc.set("R0", r0s[0])
    ob = oracle.brush(3.0, fp)
    ob.set_rates(0.05, 0.1)
    for _, path, r, spacing, K, S in strokes:
        ob.set_radius(r)
        ob.dip(K, S)
        ob.paint_stroke(oc, path, spacing)
    ob.stamps(oc, extra)
    for p in ("K", "S", "V"):
        assert np.array_equal(cs[0].download(p), oc.get(p)), p


def test_batch_rejects_bad_input(pg):
    fp = workloads.footprint_image(seed=7)
    c = pg.Canvas(20, 20)
    b = pg.FootprintBrush(3.0, fp)
    with pytest.raises(ValueError):
        pg.paint_batch([c], [b], [(1, np.zeros((2, 2)), 3.0, 1.0, np.ones(3), np.ones(3))])
    with pytest.raises(ValueError):
        pg.paint_batch([c, c], [b, b], [])
    with pytest.raises(ValueError):
        pg.paint_batch([c], [b], [(0, np.zeros((2, 2)), 3.0, 0.0, np.ones(3), np.ones(3))])
