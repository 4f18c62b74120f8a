"""The restated oracle against painty's own headers compiled here (bit for bit)."""
import numpy as np
import pytest

from painty_gb300 import workloads


def test_math_bitexact(oracle, reference):
    rng = np.random.default_rng(5)
    for _ in range(500):
        x = float(rng.choice([rng.uniform(-30, 30), rng.uniform(-1e-3, 1e-3)]))
        assert oracle.coth(x) == reference.coth(x)
        K, S, R0 = rng.uniform(0, 5, 3), rng.uniform(0, 3, 3), rng.uniform(0, 1, 3)
        d = float(rng.uniform(0, 2))
        a = oracle.compute_reflectance(K, S, R0, d)
        b = reference.compute_reflectance(K, S, R0, d)
        assert np.array_equal(a, b, equal_nan=True)
        p = rng.uniform(-50, 50, 5)
        assert oracle.catmull_rom_1d(*p) == reference.catmull_rom_1d(*p)
        pts = rng.uniform(0, 100, (6, 2))
        u = float(rng.uniform(0, 1))
        assert np.array_equal(oracle.spline_catmull_rom(pts, u), reference.spline_catmull_rom(pts, u))
        img = rng.random((5, 7))
        x, y = rng.uniform(-2, 8, 2)
        assert oracle.interpolate(img, x, y) == reference.interpolate(img, x, y)


def test_color_bitexact(oracle, reference):
    rng = np.random.default_rng(6)
    for _ in range(300):
        a, b = rng.random(3), rng.random(3)
        la, lb = oracle.rgb2lab(a), oracle.rgb2lab(b)
        np.testing.assert_allclose(la, reference.rgb2lab(a), rtol=1e-15, atol=1e-13)
        assert abs(oracle.ciede2000(la, lb) - reference.ciede2000(la, lb)) < 1e-12


@pytest.mark.parametrize("snap", [True, False])
def test_stamps_bitexact(oracle, reference, snap):
    fp = workloads.footprint_image(seed=9)
    rng = np.random.default_rng(12 + snap)
    rows, cols = 45, 63
    oc, rc = oracle.canvas(rows, cols), reference.canvas(rows, cols)
    r0 = rng.uniform(0.8, 0.95, (rows, cols, 3))
    oc.set("R0", r0)
    rc.set("R0", r0)
    ob, rb = oracle.brush(5.0, fp), reference.brush(5.0, fp)
    for b in (ob, rb):
        b.set_rates(0.05, 0.1)
        b.set_snapshot(snap)
    for s in range(8):
        rad = float(rng.uniform(0.5, 14))
        K, S = rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)
        st = np.stack([rng.uniform(-8, cols + 8, 25), rng.uniform(-8, rows + 8, 25),
                       rng.uniform(-7, 7, 25)], axis=1)
        for b, c in ((ob, oc), (rb, rc)):
            b.set_radius(rad)
            b.dip(K, S)
            b.stamps(c, st)
        assert ob.info()[1:] == rb.info()
        assert np.array_equal(ob.footprint(), rb.footprint())
    for p in ("K", "S", "V"):
        assert np.array_equal(oc.get(p), rc.get(p)), p
        assert np.array_equal(ob.pickup(p), rb.pickup(p)), p
    assert np.array_equal(oc.compose(), rc.compose())
    oc.dry()
    rc.dry()
    for p in ("R0", "h", "K", "V"):
        assert np.array_equal(oc.get(p), rc.get(p)), p


def test_stroke_bitexact(oracle, reference):
    fp = workloads.footprint_image(seed=9)
    for seed in range(3):
        rng = np.random.default_rng(seed)
        oc, rc = oracle.canvas(50, 70), reference.canvas(50, 70)
        ob, rb = oracle.brush(3.5, fp), reference.brush(3.5, fp)
        K, S = rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)
        path = rng.uniform(-5, 75, (5, 2))
        for b in (ob, rb):
            b.dip(K, S)
        n1 = ob.paint_stroke(oc, path, 1.0)
        n2 = rb.paint_stroke(rc, path)
        assert n1 == n2
        for p in ("K", "S", "V"):
            assert np.array_equal(oc.get(p), rc.get(p))


def test_stamps_edge_parameters_bitexact(oracle, reference):
    """Rates at 0 and 1, radii from below painty's 0.5 setup threshold to a box larger than
    the canvas, snapshot on and off, stamps on, across and outside a 9 x 13 canvas."""
    fp = workloads.footprint_image(seed=9)
    rng = np.random.default_rng(1)
    K, S = rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)
    st = np.stack([rng.uniform(-3, 16, 30), rng.uniform(-3, 12, 30), rng.uniform(-7, 7, 30)],
                  axis=1)
    r0 = rng.uniform(0.5, 1, (9, 13, 3))
    for rad in (0.0, 0.3, 1.0, 2.0, 4.0, 40.0):
        for rates in ((0.0, 0.0), (1.0, 1.0), (0.0, 1.0), (1.0, 0.0)):
            for snap in (True, False):
                oc, rc = oracle.canvas(9, 13), reference.canvas(9, 13)
                ob, rb = oracle.brush(rad, fp), reference.brush(rad, fp)
                for b, c in ((ob, oc), (rb, rc)):
                    c.set("R0", r0)
                    b.set_rates(*rates)
                    b.set_snapshot(snap)
                    b.dip(K, S)
                    b.stamps(c, st)
                case = (rad, rates, snap)
                assert ob.info()[1:] == rb.info(), case
                for p in ("K", "S", "V"):
                    assert np.array_equal(oc.get(p), rc.get(p), equal_nan=True), (case, p)
                    if rb.info()[1] > 0:
                        assert np.array_equal(ob.pickup(p), rb.pickup(p), equal_nan=True), (case, p)


def _tiny_brush_scenario(lib, tiny_stamp: bool):
    fp = workloads.footprint_image(seed=9)
    rng = np.random.default_rng(4)
    c = lib.canvas(15, 21)
    c.set("R0", rng.uniform(0.6, 0.9, (15, 21, 3)))
    a, b = lib.brush(0.3, fp), lib.brush(3.0, fp)
    a.set_snapshot(True)
    b.set_snapshot(False)
    a.dip(np.full(3, 2.0), np.full(3, 0.5))
    b.dip(np.array([4.0, 0.2, 1.0]), np.array([0.3, 2.0, 0.7]))
    a.stamps(c, np.array([[10.0, 7.0, 0.0]]))  # the snapshot: a copy of the canvas
    b.stamps(c, np.array([[10.0, 7.0, 0.2], [11.0, 7.5, 0.4]]))  # the canvas changes under it
    before = [c.get(p) for p in ("K", "S", "V")]
    if tiny_stamp:
        a.stamps(c, np.array([[10.3, 7.2, 0.0]]))
    after = [c.get(p) for p in ("K", "S", "V")]
    a.set_radius(3.0)
    a.stamps(c, np.array([[10.0, 7.0, 0.1]]))  # picks up from the snapshot's interior
    return before, after, [c.get(p) for p in ("K", "S", "V")]


def test_brush_below_setup_radius(oracle, reference):
    """A brush created with radius < 0.5 never sets up its maps (FootprintBrush.hxx:46-63 ignores
    changes below 0.5, and the radius starts at 0, :437), so its footprint is 0 x 0. Its stamps
    leave the canvas unchanged, yet with the snapshot on each one still refreshes the snapshot
    at the stamp's centre pixel (updateSnapshot, :278-319, with half-sizes (0 - 1) / 2 = 0).
    The oracle does the same, and the refresh changes what a later, larger stamp picks up."""
    for tiny in (True, False):
        o, r = _tiny_brush_scenario(oracle, tiny), _tiny_brush_scenario(reference, tiny)
        for xo, xr in zip(o, r):
            for u, v in zip(xo, xr):
                assert np.array_equal(u, v)
        for u, v in zip(r[0], r[1]):  # the tiny stamp leaves the canvas as it was
            assert np.array_equal(u, v)
    with_tiny, without = _tiny_brush_scenario(reference, True), _tiny_brush_scenario(reference, False)
    assert not all(np.array_equal(u, v) for u, v in zip(with_tiny[2], without[2]))


def test_mix_single_paint_bitexact(oracle, reference, pg):
    """PaintMixer::mixSinglePaint (painty's own PaintMixer.cxx, its Ceres fitting routines
    compiled against a stand-in and not run) against the oracle and the library's host code:
    weights that sum to one, that do not (normalised when more than painty's Eps away), and
    sparse ones, bit for bit."""
    K, S = workloads.pigments()
    rng = np.random.default_rng(8)
    cases = [rng.dirichlet(np.full(len(K), a)) for a in (0.1, 0.3, 1.0, 5.0) for _ in range(5)]
    cases += [c * s for c in cases[:6] for s in (0.5, 1.0 + 1e-12, 2.0, 1e-3)]
    one_hot = np.zeros(len(K))
    one_hot[3] = 1.0
    cases += [one_hot, np.zeros(len(K))]
    for w in cases:
        kr, sr = reference.mix_single_paint(w, K, S)
        ko, so = oracle.mix_single_paint(w, K, S)
        kl, sl = pg.mix_single_paint(w, K, S)
        for a, b in ((kr, ko), (sr, so), (kr, kl), (sr, sl)):
            assert np.array_equal(a, b, equal_nan=True), w
