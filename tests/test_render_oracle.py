"""Renderer::render (the lit canvas) restated in the oracle, pinned bit for bit to painty's own
Renderer.hxx: the committed reference outputs, and the reference itself where it is built."""
import numpy as np
import pytest

CASES = ["random_a", "random_b", "painted"]


def _canvas(o, fx, name):
    rows, cols = fx[f"{name}/V"].shape
    c = o.canvas(rows, cols)
    for p in ("R0", "K", "S", "V"):
        c.set(p, fx[f"{name}/{p}"])
    return c


@pytest.mark.parametrize("name", CASES)
def test_render_oracle_matches_golden(oracle, golden, name):
    fx = golden["render"]
    out = _canvas(oracle, fx, name).render()
    assert np.array_equal(out, fx[f"{name}/out"])
    assert 0.0 <= out.min() and out.max() <= 1.0


def test_render_oracle_matches_reference(oracle, reference):
    rng = np.random.default_rng(12)
    rows, cols = 31, 45
    planes = {"R0": rng.uniform(0.8, 0.95, (rows, cols, 3)),
              "K": rng.uniform(0.01, 5, (rows, cols, 3)),
              "S": rng.uniform(0.05, 3, (rows, cols, 3)),
              "V": rng.uniform(0, 2, (rows, cols)) * (rng.random((rows, cols)) < 0.5)}
    outs = []
    for o in (oracle, reference):
        c = o.canvas(rows, cols)
        for p, a in planes.items():
            c.set(p, a)
        outs.append(c.render())
    assert np.array_equal(outs[0], outs[1])
