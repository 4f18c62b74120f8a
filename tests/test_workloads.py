import numpy as np

from painty_gb300 import workloads


def test_footprint_range_and_determinism():
    a = workloads.footprint_image(seed=7)
    b = workloads.footprint_image(seed=7)
    assert a.shape == (64, 64) and np.array_equal(a, b)
    assert a.min() >= 0.0 and a.max() <= 1.0 and a.max() > 0.5
    assert a[0, 0] == 0.0  # radial falloff reaches zero at the corners


def test_strokes_shapes():
    ss = workloads.strokes(1024, 768, 10, seed=3)
    assert len(ss) == 10
    for s in ss:
        assert s.path.shape == (8, 2)
        assert 8 <= s.radius <= 32
        assert abs(s.spacing - 0.25 * s.radius) < 1e-12
        assert np.all(s.K > 0) and np.all(s.S > 0)


def test_composite_stack_distribution():
    K, S, V, R0 = workloads.composite_stack(64, 64, layers=8, seed=1)
    assert K.shape == (8, 3, 64, 64) and V.shape == (8, 64, 64)
    frac_zero = float((V == 0).mean())
    frac_small = float(((V > 0) & (V < 1e-4)).mean())
    assert 0.17 < frac_zero < 0.23 and 0.03 < frac_small < 0.07
    assert K.min() >= 0.01 and S.min() >= 0.05 and R0.min() >= 0.8


def test_vectorised_mix_equals_mix_single_paint():
    """mix_paints_np (rows of weights at once) equals mix_single_paint_np row by row, bit for
    bit, including rows whose weights need normalising."""
    PK, PS = workloads.pigments(11)
    rng = np.random.default_rng(4)
    W = rng.dirichlet(np.full(14, 0.3), 50)
    W[::7] *= 1.7  # off-normal rows
    k, s = workloads.mix_paints_np(W, PK, PS)
    for i in range(len(W)):
        k1, s1 = workloads.mix_single_paint_np(W[i], PK, PS)
        assert np.array_equal(k[i], k1) and np.array_equal(s[i], s1)


def test_batch_canvases_reproducible_and_independent():
    a = workloads.batch_canvases(4, seed=2, smin=64, smax=128, strokes_min=3, strokes_max=6)
    b = workloads.batch_canvases(6, seed=2, smin=64, smax=128, strokes_min=3, strokes_max=6)
    for (ra, ca, r0a), (rb, cb, r0b) in zip(a[0], b[0][:4]):
        assert (ra, ca) == (rb, cb) and np.array_equal(r0a, r0b)
    sa = [x for x in a[1]]
    sb = [x for x in b[1] if x[0] < 4]
    assert len(sa) == len(sb)
    for x, y in zip(sa, sb):
        assert x[0] == y[0] and np.array_equal(x[1], y[1]) and x[2] == y[2]
    assert all(0.80 <= r0.min() and r0.max() <= 0.95 for _, _, r0 in a[0])
