"""Texture brush (TextureBrush + Smudge) on the GPU vs painty's own results and the oracle.

F64 storage repeats painty's double arithmetic in its order (device code without fused
multiply-adds): canvas planes must equal the reference-generated fixtures and the oracle bit
for bit, and so must the smudge pickup map.
"""
import numpy as np
import pytest

from painty_gb300 import workloads
from test_texture_brush_oracle import _run, _session, replay_texture_fixture

pytestmark = pytest.mark.gpu

F32_REL_TOL = 1e-3   # per-value relative error of K, S, V after a stroke session (FP32)
F32_DELTA_E = 0.05   # CIEDE2000 of the composed canvas, FP32 storage vs the double oracle
F16_DELTA_E = 0.5    # the same, FP16 storage
BF16_DELTA_E = 0.5   # the same, BF16 storage: missed (below)
# BF16 keeps 8 significant bits of K and S, and the smudge re-blends a pixel at every step that
# covers it (about 2r steps per stroke); with stochastic rounding this session measures
# 1.5-2.2 max (mean 0.13) depending on the rounding bits: an expected failure
BF16_XFAIL = pytest.mark.xfail(strict=True, reason="BF16 storage misses dE < 0.5 under the "
                                                   "smudge (measured 1.5-2.2 max)")


def _gpu_run(pg, storage, rows, cols, tex, session, smudge=True, scale=1.0, r0=0.9):
    c = pg.Canvas(rows, cols, storage)
    c.upload("R0", np.full((rows, cols, 3), r0) if np.isscalar(r0) else r0)
    b = pg.TextureBrush(tex)
    b.enableSmudge(smudge)
    b.setThicknessScale(scale)
    counts = []
    for path, r, K, S in session:
        b.setRadius(r)
        b.dip((K, S))
        counts.append(b.paintStroke(path, c))
    return c, b, counts


@pytest.mark.parametrize("name", ["smudge", "nosmudge"])
def test_f64_bitexact_vs_reference_fixture(pg, golden, name):
    fx = golden["texture"]
    c, _ = replay_texture_fixture(pg, fx, name, storage="f64")
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), fx[f"{name}/out_{p}"]), p


# cluster "": the default launch (a 16-CTA cluster in FP64); "1": one CTA, with both smudge maps
# in shared memory for radii up to 20 and in global memory for 36-44; "2": a 2-CTA cluster
@pytest.mark.parametrize("smudge,rmin,rmax,cluster", [
    (True, 2.0, 20.0, ""), (False, 2.0, 20.0, ""), (True, 36.0, 44.0, ""),
    (True, 2.0, 20.0, "1"), (True, 36.0, 44.0, "1"), (True, 2.0, 20.0, "2")])
def test_f64_bitexact_vs_oracle_random(pg, oracle, monkeypatch, smudge, rmin, rmax, cluster):
    if cluster:
        monkeypatch.setenv("PAINTY_SMUDGE_CLUSTER", cluster)
    rng = np.random.default_rng(101 + smudge)
    rows, cols = 72, 96
    tex = workloads.stroke_texture(seed=13)
    sess = _session(rng, rows, cols, 8 if rmax < 30 else 3, rmin=rmin, rmax=rmax)
    c, b, counts = _gpu_run(pg, "f64", rows, cols, tex, sess, smudge)
    oc = oracle.canvas(rows, cols)
    oc.set("R0", np.full((rows, cols, 3), 0.9))
    ob = oracle.texture_brush(tex)
    ob.enable_smudge(smudge)
    ocounts = []
    for path, r, K, S in sess:
        ob.set_radius(r)
        ob.dip(K, S)
        ocounts.append(ob.paint_stroke(oc, path))
    assert counts == ocounts
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), oc.get(p)), p
    if smudge:
        for p in ("K", "S", "V"):
            assert np.array_equal(b.getSmudgeMap(p), ob.smudge_map(p)), "smudge " + p


def test_f64_straight_stroke(pg, oracle):
    """painty's TextureBrushTest geometry (TextureBrushTest.cxx:27-31), scaled down."""
    rows, cols = 96, 128
    tex = workloads.stroke_texture(seed=5)
    path = np.array([[6.25, 31.25], [50.0, 31.25], [81.25, 31.25]])
    sess = [(path, 5.0, np.array([0.2, 0.3, 0.4]), np.array([0.1, 0.23, 0.14]))]
    c, _, _ = _gpu_run(pg, "f64", rows, cols, tex, sess, True, 2.0)
    oc = _run(oracle, rows, cols, tex, sess, True, 2.0)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), oc.get(p)), p
    v = c.download("V")
    assert v[31, 40] > 0.0 and v[5, 40] == 0.0


def test_degenerate_and_off_canvas_strokes(pg, oracle):
    rows, cols = 40, 40
    tex = workloads.stroke_texture(seed=3)
    sess = [(np.array([[10.0, 10.0]]), 5.0, np.ones(3), np.ones(3)),                 # one point
            (np.array([[10.0, 10.0], [10.0, 10.0]]), 5.0, np.ones(3), np.ones(3)),   # zero length
            (np.array([[-50.0, -50.0], [-20.0, -30.0]]), 4.0, np.ones(3), np.ones(3))]  # off canvas
    c, _, counts = _gpu_run(pg, "f64", rows, cols, tex, sess)
    oc = _run(oracle, rows, cols, tex, sess)
    assert counts[0] == 0 and counts[2] == 0
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), oc.get(p)), p


def test_radius_change_resets_smudge(pg, oracle):
    """setRadius by 0.5 or more makes a new, empty smudge (TextureBrush.hxx:33-41)."""
    rows, cols = 50, 70
    tex = workloads.stroke_texture(seed=9)
    rng = np.random.default_rng(4)
    sess = _session(rng, rows, cols, 2, 6.0, 10.0)
    c, b, _ = _gpu_run(pg, "f64", rows, cols, tex, sess)
    assert b.getSmudgeMap("V").any()
    b.setRadius(30.0)
    m = b.getSmudgeMap("V")
    assert m.shape == (60, 60) and not m.any()


@pytest.mark.parametrize("storage", ["f32", "f16", pytest.param("bf16", marks=BF16_XFAIL)])
def test_reduced_precision_vs_oracle(pg, oracle, storage):
    rng = np.random.default_rng(55)
    rows, cols = 80, 100
    tex = workloads.stroke_texture(seed=13)
    sess = _session(rng, rows, cols, 8)
    c, _, _ = _gpu_run(pg, storage, rows, cols, tex, sess)
    oc = _run(oracle, rows, cols, tex, sess)
    got = pg.Renderer().compose(c).download()
    want = oc.compose()
    de_max, de_mean = oracle.delta_e(got, want)
    lim = {"f32": F32_DELTA_E, "f16": F16_DELTA_E, "bf16": BF16_DELTA_E}[storage]
    assert de_max < lim, (de_max, de_mean)
    if storage == "f32":
        for p in ("K", "S", "V"):
            g, w = c.download(p), oc.get(p)
            rel = np.abs(g - w) / np.maximum(np.abs(w), 1.0)
            assert rel.max() <= F32_REL_TOL, (p, rel.max())


def test_brush_binds_to_one_math_mode(pg):
    tex = workloads.stroke_texture(seed=3)
    b = pg.TextureBrush(tex)
    b.setRadius(5.0)
    path = np.array([[5.0, 5.0], [20.0, 12.0]])
    b.paintStroke(path, pg.Canvas(30, 30, "f64"))
    with pytest.raises(pg.PaintyValueError):
        b.paintStroke(path, pg.Canvas(30, 30, "f32"))
