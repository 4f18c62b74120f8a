"""Renderer::render fused on the GPU vs painty's own outputs (committed fixtures) and the
oracle. F64 canvases compute in double with painty's operation order; CUDA's pow / exp / tan /
acos / cosh / sinh and the host libm differ in their last bits, so F64 compares within
F64_REL_TOL. F32 and 16-bit canvases compute in float."""
import numpy as np
import pytest

from test_render_oracle import CASES

pytestmark = pytest.mark.gpu

F64_REL_TOL = 1e-11   # lit value, F64 canvas vs painty (libm ulps through the shading)
F32_ABS_TOL = 5e-5    # lit value in [0, 1], F32 canvas vs the double oracle
F16_ABS_TOL = 5e-3    # FP16 K / S / V storage
BF16_ABS_TOL = 3e-2   # BF16 K / S storage


def _gpu_canvas(pg, fx, name, storage):
    rows, cols = fx[f"{name}/V"].shape
    c = pg.Canvas(rows, cols, storage)
    for p in ("R0", "K", "S", "V"):
        c.upload(p, fx[f"{name}/{p}"])
    return c


@pytest.mark.parametrize("name", CASES)
def test_render_f64_vs_reference_fixture(pg, golden, name):
    fx = golden["render"]
    c = _gpu_canvas(pg, fx, name, "f64")
    got = pg.Renderer().render(c).download()
    np.testing.assert_allclose(got, fx[f"{name}/out"], rtol=F64_REL_TOL, atol=1e-14)


@pytest.mark.parametrize("storage,tol", [("f32", F32_ABS_TOL), ("f16", F16_ABS_TOL),
                                         ("bf16", BF16_ABS_TOL)])
def test_render_reduced_precision_vs_oracle(pg, oracle, storage, tol):
    rng = np.random.default_rng(21)
    rows, cols = 67, 83
    planes = {"R0": rng.uniform(0.8, 0.95, (rows, cols, 3)),
              "K": rng.uniform(0.01, 5, (rows, cols, 3)),
              "S": rng.uniform(0.05, 3, (rows, cols, 3)),
              "V": rng.uniform(0, 1, (rows, cols)) * (rng.random((rows, cols)) < 0.6)}
    c = pg.Canvas(rows, cols, storage)
    oc = oracle.canvas(rows, cols)
    for p, a in planes.items():
        c.upload(p, a)
    # the oracle sees what the canvas stores
    for p in ("K", "S", "V"):
        oc.set(p, c.download(p))
    oc.set("R0", c.download("R0"))
    got = pg.Renderer().render(c).download()
    want = oc.render()
    err = np.abs(got - want).max()
    assert err <= tol, err


def test_render_after_painting(pg, oracle):
    """A painted canvas: brush ridges in the volume give the normals structure."""
    from painty_gb300 import workloads
    fp = workloads.footprint_image(seed=7)
    c = pg.Canvas(50, 70, "f64")
    oc = oracle.canvas(50, 70)
    b = pg.FootprintBrush(5.0, fp)
    ob = oracle.brush(5.0, fp)
    K, S = np.array([0.3, 1.2, 2.0]), np.array([0.5, 0.4, 0.9])
    b.dip((K, S))
    ob.dip(K, S)
    path = np.array([[5.0, 5.0], [30.0, 12.5], [62.0, 40.0], [20.0, 43.0]])
    b.paintStroke(path, c)
    ob.paint_stroke(oc, path)
    np.testing.assert_allclose(pg.Renderer().render(c).download(), oc.render(),
                               rtol=F64_REL_TOL, atol=1e-14)
