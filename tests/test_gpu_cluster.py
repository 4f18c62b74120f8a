"""Thread-block clusters sharing each stamp: results must not depend on the cluster size.

PAINTY_STAMP_CLUSTER / PAINTY_BATCH_CLUSTER force the cluster size of the single-canvas and the
batched launches (the defaults come from the stamp size and the batch cost model)."""
import numpy as np
import pytest

from painty_gb300 import workloads
from test_gpu_batch import _canvases, _session, _setup
from test_gpu_stamps import _gpu_replay

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cl", [2, 4, 8, 16])
@pytest.mark.parametrize("name", ["snap_small", "nosnap_small", "snap_default_rates"])
def test_single_canvas_cluster_bitexact_vs_reference(pg, golden, monkeypatch, cl, name):
    monkeypatch.setenv("PAINTY_STAMP_CLUSTER", str(cl))
    fx = golden["stamps"]
    c, b = _gpu_replay(pg, fx, name)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), fx[f"{name}/out_{p}"]), p
        assert np.array_equal(b.getPickupMap(p), fx[f"{name}/pickup_{p}"]), "pickup " + p


# radii 10-40, and 50-64 (cell maps in global memory beside the support-disc list); every CTA
# of a cluster classifies its share of the disc into every CTA's map
@pytest.mark.parametrize("storage,rmin,rmax", [("f32", 10, 40), ("f16", 10, 40), ("f32", 50, 64)])
def test_single_canvas_cluster_sizes_agree(pg, monkeypatch, storage, rmin, rmax):
    fp = workloads.footprint_image(seed=7)
    strokes = workloads.strokes(300, 220, 6, seed=19, rmin=rmin, rmax=rmax)
    out = {}
    for cl in (1, 2, 4, 8, 16):
        monkeypatch.setenv("PAINTY_STAMP_CLUSTER", str(cl))
        c = pg.Canvas(220, 300, storage)
        c.upload("R0", np.full((220, 300, 3), 0.85))
        b = pg.FootprintBrush(strokes[0].radius, fp)
        b.setPickupRate(0.05)
        b.setDepositionRate(0.1)
        workloads.paint_config0(c, b, strokes)
        out[cl] = [c.download(p) for p in ("K", "S", "V")]
    for cl in (2, 4, 8, 16):
        for a, b in zip(out[1], out[cl]):
            assert np.array_equal(a, b), cl


@pytest.mark.parametrize("cl", [2, 4])
def test_batch_cluster_f64_equals_oracle(pg, oracle, monkeypatch, cl):
    monkeypatch.setenv("PAINTY_BATCH_CLUSTER", str(cl))
    rng = np.random.default_rng(23 + cl)
    sizes = _canvases(rng, 5)
    strokes = _session(rng, sizes)
    cs, bs, r0s = _setup(pg, sizes, "f64")
    pg.paint_batch(cs, bs, strokes)
    fp = workloads.footprint_image(seed=7)
    for ci, (rows, cols) in enumerate(sizes):
        oc = oracle.canvas(rows, cols)
        oc.set("R0", r0s[ci])
        ob = oracle.brush(3.0, fp)
        ob.set_rates(0.05, 0.1)
        for cj, path, r, spacing, K, S in strokes:
            if cj != ci:
                continue
            ob.set_radius(r)
            ob.dip(K, S)
            ob.paint_stroke(oc, path, spacing)
        for p in ("K", "S", "V"):
            assert np.array_equal(cs[ci].download(p), oc.get(p)), (ci, p)
        assert np.array_equal(bs[ci].getPickupMap("V"), ob.pickup("V"))


def test_batch_cluster_sizes_agree_f16(pg, monkeypatch):
    rng = np.random.default_rng(31)
    sizes = _canvases(rng, 9, 64, 300)
    strokes = _session(rng, sizes, (3, 8), 2.0, 40.0)
    out = {}
    for cl in (1, 2, 4):
        monkeypatch.setenv("PAINTY_BATCH_CLUSTER", str(cl))
        cs, bs, _ = _setup(pg, sizes, "f16")
        pg.paint_batch(cs, bs, strokes)
        out[cl] = [[c.download(p) for p in ("K", "S", "V")] for c in cs]
    for cl in (2, 4):
        for ci in range(len(sizes)):
            for a, b in zip(out[1][ci], out[cl][ci]):
                assert np.array_equal(a, b), (cl, ci)
