"""The texture brush restated in the oracle (TextureBrush.hxx + Smudge.hxx) against painty's own
headers compiled by the reference harness: canvas state bit for bit after stroke sessions."""
import numpy as np
import pytest

from painty_gb300 import workloads


def _session(rng, rows, cols, n, rmin=4.0, rmax=18.0):
    out = []
    for _ in range(n):
        k = int(rng.integers(2, 6))
        path = np.stack([rng.uniform(-10, cols + 10, k), rng.uniform(-10, rows + 10, k)], axis=1)
        out.append((path, float(rng.uniform(rmin, rmax)), rng.uniform(0.01, 5, 3),
                    rng.uniform(0.05, 3, 3)))
    return out


def _run(o, rows, cols, tex, session, smudge=True, scale=1.0):
    c = o.canvas(rows, cols)
    c.set("R0", np.full((rows, cols, 3), 0.9))
    b = o.texture_brush(tex)
    b.enable_smudge(smudge)
    b.set_thickness_scale(scale)
    for path, r, K, S in session:
        b.set_radius(r)
        b.dip(K, S)
        b.paint_stroke(c, path)
    return c


@pytest.mark.parametrize("smudge", [True, False])
def test_texture_brush_oracle_matches_reference(oracle, reference, smudge):
    rng = np.random.default_rng(7 + smudge)
    rows, cols = 60, 80
    tex = workloads.stroke_texture(seed=13)
    sess = _session(rng, rows, cols, 6)
    a = _run(oracle, rows, cols, tex, sess, smudge)
    b = _run(reference, rows, cols, tex, sess, smudge)
    for p in ("K", "S", "V"):
        assert np.array_equal(a.get(p), b.get(p)), p
    assert a.get("V").max() > 0.0


def test_texture_brush_straight_stroke(oracle, reference):
    """painty's own TextureBrushTest geometry (TextureBrushTest.cxx:27-31), scaled down."""
    rows, cols = 96, 128
    tex = workloads.stroke_texture(seed=5)
    path = np.array([[6.25, 31.25], [50.0, 31.25], [81.25, 31.25]])
    sess = [(path, 5.0, np.array([0.2, 0.3, 0.4]), np.array([0.1, 0.23, 0.14]))]
    a = _run(oracle, rows, cols, tex, sess, True, 2.0)
    b = _run(reference, rows, cols, tex, sess, True, 2.0)
    for p in ("K", "S", "V"):
        assert np.array_equal(a.get(p), b.get(p)), p
    v = a.get("V")
    assert v[31, 40] > 0.0 and v[5, 40] == 0.0  # on the stroke, and far off it


def test_texture_brush_degenerate_paths(oracle, reference):
    rows, cols = 40, 40
    tex = workloads.stroke_texture(seed=3)
    sess = [(np.array([[10.0, 10.0]]), 5.0, np.ones(3), np.ones(3)),          # one point: no-op
            (np.array([[10.0, 10.0], [10.0, 10.0]]), 5.0, np.ones(3), np.ones(3))]  # zero length
    a = _run(oracle, rows, cols, tex, sess)
    b = _run(reference, rows, cols, tex, sess)
    for p in ("K", "S", "V"):
        assert np.array_equal(a.get(p), b.get(p)), p


def test_texture_brush_off_canvas_is_a_no_op(oracle):
    """painty builds a thickness map of negative size for a stroke whose bounds miss the canvas
    (TextureBrush.hxx:77-84, 135-136) and fails; here such a stroke changes nothing."""
    rows, cols = 40, 40
    tex = workloads.stroke_texture(seed=3)
    c = _run(oracle, rows, cols, tex,
             [(np.array([[-50.0, -50.0], [-20.0, -30.0]]), 4.0, np.ones(3), np.ones(3))])
    assert not c.get("V").any()


def replay_texture_fixture(o, fx, name, storage=None):
    """Replays a texture-brush session of the golden fixture on the oracle (storage None) or on
    the library's Canvas / TextureBrush (storage given; `o` is the package)."""
    rows, cols, smudge, scale, tseed = fx[f"{name}/meta"]
    rows, cols = int(rows), int(cols)
    tex = workloads.stroke_texture(seed=int(tseed))
    if storage is None:
        c = o.canvas(rows, cols)
        c.set("R0", fx[f"{name}/r0"])
        b = o.texture_brush(tex)
        b.enable_smudge(bool(smudge))
        b.set_thickness_scale(scale)
    else:
        c = o.Canvas(rows, cols, storage)
        c.upload("R0", fx[f"{name}/r0"])
        b = o.TextureBrush(tex)
        b.enableSmudge(bool(smudge))
        b.setThicknessScale(scale)
    i = 0
    while f"{name}/stroke{i}/path" in fx:
        K, S = fx[f"{name}/stroke{i}/paint"]
        if storage is None:
            b.set_radius(fx[f"{name}/stroke{i}/radius"][0])
            b.dip(K, S)
            b.paint_stroke(c, fx[f"{name}/stroke{i}/path"])
        else:
            b.setRadius(fx[f"{name}/stroke{i}/radius"][0])
            b.dip((K, S))
            b.paintStroke(fx[f"{name}/stroke{i}/path"], c)
        i += 1
    return c, b


@pytest.mark.parametrize("name", ["smudge", "nosmudge"])
def test_texture_brush_oracle_matches_golden(oracle, golden, name):
    """The oracle against the committed reference outputs (runs without the reference)."""
    fx = golden["texture"]
    c, _ = replay_texture_fixture(oracle, fx, name)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.get(p), fx[f"{name}/out_{p}"]), p
