"""Imprint-brush stamping kernel vs painty's own results and the oracle (GPU).

F64 storage repeats the reference's double arithmetic in its order: results must be bit for
bit those of painty's FootprintBrush (reference-generated fixtures) and of the oracle.
"""
import numpy as np
import pytest

from painty_gb300 import workloads

pytestmark = pytest.mark.gpu

# FP32 storage vs the double oracle after a stroke sequence: per-value error of K, S, V
# relative to max(|value|, 1), and CIEDE2000 of the composed canvas
F32_REL_TOL = 1e-4
F32_DELTA_E = 0.05
# 16-bit storage (FP32 arithmetic) vs the double oracle: CIEDE2000 of the composed canvas
F16_DELTA_E = 0.5
BF16_DELTA_E = 0.5


def _gpu_replay(pg, fx, name, storage="f64"):
    rows, cols, snap, pr, dr = fx[f"{name}/meta"]
    rows, cols = int(rows), int(cols)
    c = pg.Canvas(rows, cols, storage)
    c.upload("R0", fx[f"{name}/r0"])
    b = pg.FootprintBrush(3.0, fx["footprint_full"])
    b.setPickupRate(pr)
    b.setDepositionRate(dr)
    b.setUseSnapshotBuffer(bool(snap))
    i = 0
    while f"{name}/stroke{i}/radius" in fx:
        b.setRadius(fx[f"{name}/stroke{i}/radius"][0])
        K, S = fx[f"{name}/stroke{i}/paint"]
        b.dip((K, S))
        b.stamps(fx[f"{name}/stroke{i}/stamps"], c)
        i += 1
    return c, b


@pytest.mark.parametrize("name", ["snap_small", "nosnap_small", "snap_default_rates"])
def test_f64_bitexact_vs_reference_fixture(pg, golden, name):
    fx = golden["stamps"]
    c, b = _gpu_replay(pg, fx, name)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), fx[f"{name}/out_{p}"]), p
        assert np.array_equal(b.getPickupMap(p), fx[f"{name}/pickup_{p}"]), "pickup " + p
    c.dryCanvas()
    assert np.array_equal(c.get_h(), fx[f"{name}/dry_h"])


def test_f64_stroke_bitexact_vs_reference_fixture(pg, golden):
    fx = golden["stamps"]
    c = pg.Canvas(40, 60, "f64")
    c.upload("R0", np.full((40, 60, 3), 0.9))
    b = pg.FootprintBrush(4.0, fx["footprint_full"])
    b.setPickupRate(0.05)
    b.setDepositionRate(0.1)
    b.dip((np.array([0.3, 1.2, 2.0]), np.array([0.5, 0.4, 0.9])))
    n = b.paintStroke(fx["stroke/path"], c, spacing=1.0)
    assert n == int(fx["stroke/count"][0])
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), fx[f"stroke/out_{p}"]), p


def _random_session(rng, rows, cols, nstrokes, rmin, rmax, nstamps):
    out = []
    for _ in range(nstrokes):
        rad = float(rng.uniform(rmin, rmax))
        K, S = rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)
        st = np.stack([rng.uniform(-10, cols + 10, nstamps), rng.uniform(-10, rows + 10, nstamps),
                       rng.uniform(-7, 7, nstamps)], axis=1)
        out.append((rad, K, S, st))
    return out


def _run_both(pg, oracle, storage, rows, cols, session, snap=True, rates=(0.05, 0.1), fp_seed=7):
    fp = workloads.footprint_image(seed=fp_seed)
    c = pg.Canvas(rows, cols, storage)
    oc = oracle.canvas(rows, cols)
    r0 = np.random.default_rng(99).uniform(0.8, 0.95, (rows, cols, 3))
    c.upload("R0", r0)
    oc.set("R0", r0)
    b = pg.FootprintBrush(session[0][0], fp)
    ob = oracle.brush(session[0][0], fp)
    b.setPickupRate(rates[0])
    b.setDepositionRate(rates[1])
    ob.set_rates(*rates)
    b.setUseSnapshotBuffer(snap)
    ob.set_snapshot(snap)
    for rad, K, S, st in session:
        b.setRadius(rad)
        ob.set_radius(rad)
        b.dip((K, S))
        ob.dip(K, S)
        b.stamps(st, c)
        ob.stamps(oc, st)
    return c, b, oc, ob


@pytest.mark.parametrize("snap", [True, False])
def test_f64_bitexact_vs_oracle_random(pg, oracle, snap):
    rng = np.random.default_rng(31 + snap)
    session = _random_session(rng, 70, 90, 6, 0.6, 24.0, 30)
    c, b, oc, ob = _run_both(pg, oracle, "f64", 70, 90, session, snap=snap)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), oc.get(p)), p
        assert np.array_equal(b.getPickupMap(p), ob.pickup(p)), p


def test_f64_bitexact_large_radius_global_owner_table(pg, oracle):
    """Radius 85: the owner table (242^2 ints) exceeds shared memory and lives in global."""
    rng = np.random.default_rng(5)
    session = [(85.0, rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3),
                np.array([[100.0, 90.0, 0.3], [120.5, 100.25, 2.1], [10.5, 5.5, -1.0]]))]
    c, b, oc, ob = _run_both(pg, oracle, "f64", 200, 240, session)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), oc.get(p)), p


def test_f64_edge_duplicates(pg, oracle):
    """Centres with fractional parts at the top-left edge: trunc() maps two columns and two
    rows onto canvas column / row 0."""
    rng = np.random.default_rng(8)
    st = np.array([[0.5, 0.25, 0.0], [0.75, 0.5, 0.7], [1.5, 0.9, -2.0], [0.1, 30.5, 1.1],
                   [40.3, 0.6, 3.0], [-0.5, -0.5, 0.4]])
    session = [(6.0, rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3), st)] * 3
    c, b, oc, ob = _run_both(pg, oracle, "f64", 50, 60, session)
    for p in ("K", "S", "V"):
        assert np.array_equal(c.download(p), oc.get(p)), p


def test_hand_single_stamp_empty_canvas(pg):
    fp = workloads.footprint_image(seed=7)
    c = pg.Canvas(30, 30, "f64")
    b = pg.FootprintBrush(4.0, fp)
    K, S = np.array([0.5, 1.0, 2.0]), np.array([0.3, 0.2, 0.1])
    b.dip((K, S))
    b.imprint((15.0, 15.0), 0.0, c)
    F = b.info()[1]
    wr = (F - 1) // 2
    V = c.download("V")
    np.testing.assert_array_equal(V[15 - wr:15 + wr + 1, 15 - wr:15 + wr + 1], b.getFootprint())
    assert V.sum() == b.getFootprint().sum()


# BF16 keeps 8 significant bits; a pixel re-blended by every stamp over it drifts. With the
# stochastic rounding of 16-bit stores this case measures about 1.5 max, 0.3 mean: above the
# 0.5 target, recorded as an expected failure.
BF16_XFAIL = pytest.mark.xfail(strict=True, reason="BF16 storage misses dE < 0.5 on painting "
                                                   "(measured about 1.5 max)")


@pytest.mark.parametrize("storage", ["f32", "f16", pytest.param("bf16", marks=BF16_XFAIL)])
def test_reduced_precision_vs_oracle(pg, oracle, storage):
    rng = np.random.default_rng(41)
    session = _random_session(rng, 80, 100, 8, 3.0, 20.0, 40)
    c, b, oc, ob = _run_both(pg, oracle, storage, 80, 100, session)
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


def test_stroke_api_matches_oracle_f64(pg, oracle):
    fp = workloads.footprint_image(seed=7)
    for i, s in enumerate(workloads.strokes(120, 90, 4, seed=17, rmin=3, rmax=10)):
        c = pg.Canvas(90, 120, "f64")
        oc = oracle.canvas(90, 120)
        b = pg.FootprintBrush(s.radius, fp)
        ob = oracle.brush(s.radius, fp)
        b.dip((s.K, s.S))
        ob.dip(s.K, s.S)
        n1 = b.paintStroke(s.path, c, spacing=s.spacing)
        n2 = ob.paint_stroke(oc, s.path, s.spacing)
        assert n1 == n2
        for p in ("K", "S", "V"):
            assert np.array_equal(c.download(p), oc.get(p)), (i, p)


def test_deterministic(pg):
    rng = np.random.default_rng(3)
    session = _random_session(rng, 64, 64, 4, 4.0, 16.0, 25)
    outs = []
    for _ in range(2):
        fp = workloads.footprint_image(seed=7)
        c = pg.Canvas(64, 64, "f32")
        b = pg.FootprintBrush(5.0, fp)
        for rad, K, S, st in session:
            b.setRadius(rad)
            b.dip((K, S))
            b.stamps(st, c)
        outs.append([c.download(p, dtype=np.float32) for p in ("K", "S", "V")])
    for a, b2 in zip(*outs):
        assert np.array_equal(a, b2)


def test_imprint_equals_stamps(pg):
    fp = workloads.footprint_image(seed=7)
    st = np.array([[20.3, 21.7, 0.4], [25.0, 22.0, 0.9], [28.1, 24.9, 1.3]])
    res = []
    for mode in range(2):
        c = pg.Canvas(48, 48, "f64")
        b = pg.FootprintBrush(6.0, fp)
        b.dip((np.array([1.0, 2.0, 3.0]), np.array([0.5, 0.5, 0.5])))
        if mode == 0:
            b.stamps(st, c)
        else:
            for x, y, t in st:
                b.imprint((x, y), t, c)
        res.append(c.download("V"))
    assert np.array_equal(res[0], res[1])


def test_invalid_stamp_rejected(pg):
    fp = workloads.footprint_image(seed=7)
    c = pg.Canvas(16, 16)
    b = pg.FootprintBrush(3.0, fp)
    with pytest.raises(ValueError):
        b.imprint((float("nan"), 1.0), 0.0, c)
    with pytest.raises(ValueError):
        b.paintStroke(np.array([[0.0, 0.0], [5.0, 5.0]]), c, spacing=0.0)


def test_host_setup_matches_oracle(pg, oracle):
    """Footprint resample and stroke expansion (host code) give the oracle's exact bits."""
    fp = workloads.footprint_image(seed=7)
    for r in (0.7, 3.2, 8.0, 19.6, 31.1, 64.0):
        b = pg.FootprintBrush(r, fp)
        ob = oracle.brush(r, fp)
        assert b.info() == ob.info()
        assert np.array_equal(b.getFootprint(), ob.footprint()), r


def test_f32_config0_full_vs_oracle(pg, oracle):
    """The plain workload in full -- 1024 x 768 FP32 canvas, 200 Catmull-Rom strokes, r U[8,32],
    spacing 0.25 r, rates 0.1 / 0.05, snapshot on -- against the double oracle: K, S, V within
    F32_REL_TOL and the composite within F32_DELTA_E."""
    rows, cols = 768, 1024
    strokes = workloads.strokes(cols, rows, 200, seed=3)
    fp = workloads.footprint_image(seed=7)
    r0 = workloads.substrate(rows, cols, seed=5)
    c = pg.Canvas(rows, cols, "f32")
    c.setBackground(r0)
    b = pg.FootprintBrush(strokes[0].radius, fp)
    b.setPickupRate(0.05)
    b.setDepositionRate(0.1)
    n = workloads.paint_config0(c, b, strokes)
    oc = oracle.canvas(rows, cols)
    oc.set("R0", r0)
    ob = oracle.brush(strokes[0].radius, fp)
    ob.set_rates(0.05, 0.1)
    no = 0
    for s in strokes:
        ob.set_radius(s.radius)
        ob.dip(s.K, s.S)
        no += ob.paint_stroke(oc, s.path, s.spacing)
    assert n == no and n > 100000
    errs = {}
    for p in ("K", "S", "V"):
        g, w = c.download(p), oc.get(p)
        errs[p] = float((np.abs(g - w) / np.maximum(np.abs(w), 1.0)).max())
    de_max, de_mean = oracle.delta_e(pg.Renderer().compose(c).download(), oc.compose())
    assert max(errs.values()) <= F32_REL_TOL and de_max <= F32_DELTA_E, (errs, de_max, de_mean)
