"""The oracle against the reference's own known-answer tests and reference-generated fixtures."""
import numpy as np
import pytest

from painty_gb300 import workloads


def test_reflectance_kat(oracle, golden):
    k = golden["kat"]["reflectance"]
    r = oracle.compute_reflectance(k["K"], k["S"], k["R0"], k["d"])
    np.testing.assert_allclose(r, k["expected"], atol=k["tolerance"])
    # d = 0 returns R0 (KubelkaMunkTest.cxx:26)
    r0 = oracle.compute_reflectance(k["K"], k["S"], k["R0"], 0.0)
    assert abs(r0[0] - k["R0"][0]) < k["tolerance"]
    # S = 0 is floored to 1e-11 (KubelkaMunkTest.cxx:28-30)
    rs = oracle.compute_reflectance(k["K"], [0.0, 0.0, 0.0], k["R0"], k["d"])
    assert abs(rs[0] - k["s_zero_channel0"]) < k["tolerance"]


def test_coth_kat(oracle, golden):
    k = golden["kat"]["coth"]
    assert oracle.coth(0.0) == float("inf")  # MathTest.cxx:84
    for x, want in k["cases"]:
        assert abs(oracle.coth(x) - want) < k["tolerance"]


def test_spline_kat(oracle, golden):
    k = golden["kat"]["catmull_rom"]
    assert abs(oracle.catmull_rom_1d(*k["args"]) - k["expected"]) < k["tolerance"]
    s = golden["kat"]["spline_eval"]
    got = oracle.spline_catmull_rom(np.array(s["points"]), s["u"])
    np.testing.assert_allclose(got, s["expected"], atol=s["tolerance"])


def test_bilinear_kat(oracle, golden):
    k = golden["kat"]["bilinear"]
    img = np.array(k["image_channel0"])
    assert abs(oracle.interpolate(img, *k["position"]) - k["expected"]) < k["tolerance"]


def test_border_reflect(oracle):
    img = np.arange(12, dtype=np.float64).reshape(3, 4)
    # BORDER_REFLECT: index -1 -> 0, n -> n-1; at integer positions Interpolate returns the pixel
    assert oracle.interpolate(img, -1.0, 0.0) == img[0, 0]
    assert oracle.interpolate(img, 4.0, 2.0) == img[2, 3]
    assert oracle.interpolate(img, 1.0, 1.0) == img[1, 1]
    assert abs(oracle.interpolate(img, 3.5, 0.0) - img[0, 3]) < 1e-12


def _replay(oracle, fx, name):
    rows, cols, snap, pr, dr = fx[f"{name}/meta"]
    rows, cols = int(rows), int(cols)
    c = oracle.canvas(rows, cols)
    c.set("R0", fx[f"{name}/r0"])
    b = oracle.brush(3.0, fx["footprint_full"])
    b.set_rates(pr, dr)
    b.set_snapshot(bool(snap))
    i = 0
    while f"{name}/stroke{i}/radius" in fx:
        b.set_radius(fx[f"{name}/stroke{i}/radius"][0])
        K, S = fx[f"{name}/stroke{i}/paint"]
        b.dip(K, S)
        b.stamps(c, fx[f"{name}/stroke{i}/stamps"])
        i += 1
    return c, b


@pytest.mark.parametrize("name", ["snap_small", "nosnap_small", "snap_default_rates"])
def test_oracle_matches_reference_fixture(oracle, golden, name):
    """Bit-exact against planes produced by painty's own FootprintBrush code."""
    fx = golden["stamps"]
    c, b = _replay(oracle, fx, name)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.get(p), fx[f"{name}/out_{p}"]), p
        assert np.array_equal(b.pickup(p), fx[f"{name}/pickup_{p}"]), "pickup " + p
    assert np.array_equal(c.compose(), fx[f"{name}/out_compose"])
    c.dry()
    assert np.array_equal(c.get("R0"), fx[f"{name}/dry_R0"])
    assert np.array_equal(c.get("h"), fx[f"{name}/dry_h"])


def test_oracle_stroke_matches_reference_fixture(oracle, golden):
    fx = golden["stamps"]
    c = oracle.canvas(40, 60)
    c.set("R0", np.full((40, 60, 3), 0.9))
    b = oracle.brush(4.0, fx["footprint_full"])
    b.set_rates(0.05, 0.1)
    b.dip(np.array([0.3, 1.2, 2.0]), np.array([0.5, 0.4, 0.9]))
    n = b.paint_stroke(c, fx["stroke/path"], 1.0)
    assert n == int(fx["stroke/count"][0])
    for p in ("K", "S", "V"):
        assert np.array_equal(c.get(p), fx[f"stroke/out_{p}"])


def test_hand_single_stamp(oracle):
    """theta = 0, one stamp on an empty canvas: V = footprint, (K, S) = paint where fp > 0
    (blend(fp, paint, 0, .) returns paint: FootprintBrush.hxx:331-340, 422-429)."""
    fp_img = workloads.footprint_image(seed=7)
    c = oracle.canvas(30, 30)
    b = oracle.brush(4.0, fp_img)
    K, S = np.array([0.5, 1.0, 2.0]), np.array([0.3, 0.2, 0.1])
    b.dip(K, S)
    b.imprint(c, 15.0, 15.0, 0.0)
    _, F, _ = b.info()
    fp = b.footprint()
    wr = (F - 1) // 2
    V = c.get("V")
    np.testing.assert_array_equal(V[15 - wr:15 + wr + 1, 15 - wr:15 + wr + 1], fp)
    Kc = c.get("K")
    mask = fp > 0.001
    np.testing.assert_allclose(Kc[15 - wr:15 + wr + 1, 15 - wr:15 + wr + 1][mask],
                               np.broadcast_to(K, (mask.sum(), 3)), rtol=1e-15)


def test_fp64_oracle_agrees_with_reference_formula(oracle):
    rng = np.random.default_rng(0)
    for _ in range(2000):
        K = rng.uniform(0.01, 5, 3)
        S = rng.uniform(0.05, 3, 3)
        R0 = rng.uniform(0.0, 1.0, 3)
        d = float(rng.choice([rng.uniform(1e-7, 1e-4), rng.uniform(0, 0.5), rng.uniform(0, 50)]))
        a = oracle.compute_reflectance(K, S, R0, d)
        R, T = oracle.km_fp64(K, S, R0, d)
        np.testing.assert_allclose(R, a, rtol=1e-9, atol=1e-12)
        assert np.all((T >= 0) & (T <= 1.0 + 1e-12))


def test_fp64_oracle_finite_at_zero_absorption(oracle):
    K = np.zeros(3)
    S = np.array([0.5, 1.0, 2.0])
    R0 = np.array([0.2, 0.5, 0.9])
    ref = oracle.compute_reflectance(K, S, R0, 0.3)
    assert np.all(np.isnan(ref))  # the reference: b = 0, 0 * coth(0) = NaN
    R, T = oracle.km_fp64(K, S, R0, 0.3)
    # non-absorbing layer: R = (S d (1 - R0) + R0) / (S d (1 - R0) + 1)
    sd = S * 0.3
    np.testing.assert_allclose(R, (sd * (1 - R0) + R0) / (sd * (1 - R0) + 1), rtol=1e-14)
    np.testing.assert_allclose(T, 1.0 / (1.0 + sd), rtol=1e-14)


def test_fp64_series_branch_continuous(oracle):
    K = np.array([0.4, 0.4, 0.4])
    S = np.array([1.0, 1.0, 1.0])
    R0 = np.array([0.7, 0.7, 0.7])
    b = np.sqrt(0.4 * 2.4)
    d0 = 1e-3 / b
    lo, _ = oracle.km_fp64(K, S, R0, d0 * (1 - 1e-9))
    hi, _ = oracle.km_fp64(K, S, R0, d0 * (1 + 1e-9))
    np.testing.assert_allclose(lo, hi, rtol=1e-10)


def test_mix_single_paint(oracle):
    K, S = workloads.pigments()
    rng = np.random.default_rng(1)
    w = rng.dirichlet(np.full(14, 0.3))
    k1, s1 = oracle.mix_single_paint(w, K, S)
    k2, s2 = workloads.mix_single_paint_np(w, K, S)
    assert np.array_equal(k1, k2) and np.array_equal(s1, s2)
    # weights not summing to one are normalised (PaintMixer.cxx:337-340)
    k3, _ = oracle.mix_single_paint(w * 2.0, K, S)
    np.testing.assert_allclose(k3, k1, rtol=1e-14)


def test_ciede2000_sanity(oracle):
    lab = oracle.rgb2lab(np.array([0.5, 0.5, 0.5]))
    assert oracle.ciede2000(lab, lab) == 0.0
    # published CIEDE2000 test pair (Sharma, Wu, Dalal 2005, pair 1): 2.0425
    d = oracle.ciede2000(np.array([50.0, 2.6772, -79.7751]), np.array([50.0, 0.0, -82.7485]))
    assert abs(d - 2.0425) < 1e-4


def test_planar_f32_composite_in_double_equals_interleaved(oracle):
    """The planar float32 composite kept in double (the reference the precision figures are
    measured against) equals the interleaved double composite of the same values."""
    from painty_gb300 import workloads
    K, S, V, R0 = workloads.composite_stack(23, 31, layers=5, seed=3)
    got = oracle.compose_layers_f32_planar_f64(K, S, V, R0, threads=3)
    il = lambda a: np.ascontiguousarray(np.moveaxis(a, 0, -1).reshape(-1, 3), dtype=np.float64)
    want = oracle.compose_layers(np.stack([il(K[l]) for l in range(5)]),
                                 np.stack([il(S[l]) for l in range(5)]),
                                 V.reshape(5, -1).astype(np.float64), il(R0))
    assert np.array_equal(got.reshape(-1, 3), want)
