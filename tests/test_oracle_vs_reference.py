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
