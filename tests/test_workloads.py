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
