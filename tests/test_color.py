"""painty_gb300.color (the bench's CIEDE2000) against the oracle's restatement of painty's
ColorConverter (Color.hxx), which the reference build pins."""
import numpy as np

from painty_gb300 import color


def test_lab_matches_oracle(oracle):
    rng = np.random.default_rng(4)
    rgb = rng.uniform(0.0, 1.0, (200, 3))
    rgb[:10] = rng.uniform(0.0, 1e-3, (10, 3))  # the linear segment of f
    got = color.linear_rgb_to_lab(rgb)
    want = np.stack([oracle.rgb2lab(c) for c in rgb])
    assert np.abs(got - want).max() < 1e-10


def test_ciede2000_matches_oracle(oracle):
    rng = np.random.default_rng(5)
    a = color.linear_rgb_to_lab(rng.uniform(0.0, 1.0, (300, 3)))
    b = color.linear_rgb_to_lab(rng.uniform(0.0, 1.0, (300, 3)))
    b[:20] = a[:20] + rng.normal(0, 0.3, (20, 3))  # small differences
    b[20:25] = [[50.0, 0.0, 0.0]] * 5               # zero chroma (hue conventions)
    got = color.ciede2000(a, b)
    want = np.array([oracle.ciede2000(x, y) for x, y in zip(a, b)])
    assert np.abs(got - want).max() < 1e-9


def test_ciede2000_published_pair():
    # first pair of Sharma, Wu and Dalal's CIEDE2000 test data: 2.0425
    d = color.ciede2000(np.array([50.0, 2.6772, -79.7751]), np.array([50.0, 0.0, -82.7485]))
    assert abs(float(d) - 2.0425) < 1e-4
