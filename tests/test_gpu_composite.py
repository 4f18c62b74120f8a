"""KM composite kernel vs the oracle (GPU)."""
import numpy as np
import pytest

from painty_gb300 import workloads
from tests.gpu_helpers import gpu_compose, oracle_compose

pytestmark = pytest.mark.gpu

# FP32 storage and arithmetic vs painty's double ComputeReflectance on the same inputs
F32_ABS_TOL = 1e-5
# FP16/BF16 storage (K, S, V rounded on store) vs the FP64 oracle, as CIEDE2000
HALF_DELTA_E = 0.5


@pytest.mark.parametrize("shape,L", [((61, 203), 8), ((64, 64), 1), ((17, 5), 3)])
def test_f32_matches_reference(pg, oracle, shape, L):
    K, S, V, R0 = workloads.composite_stack(*shape, layers=L, seed=L)
    got = gpu_compose(pg, K, S, V, R0, "f32")
    want = oracle_compose(oracle, K, S, V, R0, mode=0)
    err = np.abs(got - want).max()
    assert err <= F32_ABS_TOL, err


def test_f32_small_thickness_branch(pg, oracle):
    """Thickness in [1e-7, 1e-4] (the series branch) and exactly 0 (R0 passthrough)."""
    rows, cols, L = 32, 96, 4
    K, S, V, R0 = workloads.composite_stack(rows, cols, layers=L, seed=9)
    rng = np.random.default_rng(1)
    V = np.where(rng.random(V.shape) < 0.5, rng.uniform(1e-7, 1e-4, V.shape), 0.0).astype(np.float32)
    got = gpu_compose(pg, K, S, V, R0, "f32")
    want = oracle_compose(oracle, K, S, V, R0, mode=0)
    assert np.abs(got - want).max() <= F32_ABS_TOL
    # pixels with all layers at h = 0 are exactly R0
    zero = (V == 0).all(axis=0)
    assert np.array_equal(got[:, zero], R0[:, zero].astype(np.float64))


def test_f64_matches_reference(pg, oracle):
    K, S, V, R0 = workloads.composite_stack(40, 70, layers=5, seed=3, dtype=np.float64)
    got = gpu_compose(pg, K, S, V, R0, "f64")
    want = oracle_compose(oracle, K, S, V, R0, mode=0)
    assert np.abs(got - want).max() <= 1e-13


@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_half_storage_delta_e(pg, oracle, storage):
    K, S, V, R0 = workloads.composite_stack(48, 160, layers=8, seed=4, dtype=np.float64)
    got = gpu_compose(pg, K, S, V, R0, storage)
    want = oracle_compose(oracle, K, S, V, R0, mode=1)
    de_max, de_mean = oracle.delta_e(np.moveaxis(got, 0, -1), np.moveaxis(want, 0, -1))
    assert de_max < HALF_DELTA_E, (de_max, de_mean)


# FP16/BF16 storage with FP32 arithmetic vs the double oracle on the values the layers
# actually hold (downloaded back): only the arithmetic differs. The sizes give the bulk-copy
# kernel one partial tile, many tiles per block (1100 x 1100: 1182 tiles of 1024 pixels), and
# two launches of 16 + 2 layers; afterwards no copy pipeline may have stalled.
HALF_F32_MATH_ABS_TOL = 2e-5


@pytest.mark.parametrize("storage", ["f16", "bf16"])
@pytest.mark.parametrize("rows,cols,L", [(48, 160, 8), (1100, 1100, 8), (300, 517, 18)])
def test_half_storage_fp32_math(pg, oracle, storage, rows, cols, L):
    K, S, V, R0 = workloads.composite_stack(rows, cols, layers=L, seed=rows + L, dtype=np.float64)
    V[:, :, :16] = 0.0  # pixels no layer covers: exactly R0
    layers = []
    Ks, Ss, Vs = np.empty_like(K), np.empty_like(S), np.empty_like(V)
    for l in range(L):
        ly = pg.PaintLayer(rows, cols, storage)
        ly.upload("K", K[l], planar=True)
        ly.upload("S", S[l], planar=True)
        ly.upload("V", V[l], planar=True)
        Ks[l], Ss[l], Vs[l] = (ly.download("K", planar=True), ly.download("S", planar=True),
                               ly.download("V"))
        layers.append(ly)
    r0 = pg.Image(rows, cols, "f32")
    r0.upload(R0, planar=True)
    out = pg.Image(rows, cols, "f32")
    pg.compose_layers(layers, r0, out)
    got = out.download(dtype=np.float64, planar=True)
    R0s = R0.astype(np.float32).astype(np.float64)
    want = oracle_compose(oracle, Ks, Ss, Vs, R0s, mode=0)
    err = np.abs(got - want).max()
    assert err <= HALF_F32_MATH_ABS_TOL, err
    assert np.array_equal(got[:, :, :16], R0s[:, :, :16])
    assert pg.take_device_faults() == 0


def test_fused_equals_unfused_bitwise(pg):
    K, S, V, R0 = workloads.composite_stack(33, 130, layers=8, seed=5)
    a = gpu_compose(pg, K, S, V, R0, "f32", fused=True)
    b = gpu_compose(pg, K, S, V, R0, "f32", fused=False)
    assert np.array_equal(a, b)


def test_more_layers_than_one_launch(pg, oracle):
    K, S, V, R0 = workloads.composite_stack(16, 72, layers=19, seed=6)
    got = gpu_compose(pg, K, S, V, R0, "f32")
    want = oracle_compose(oracle, K, S, V, R0, mode=0)
    assert np.abs(got - want).max() <= 2 * F32_ABS_TOL


def test_inplace_and_zero_layers(pg):
    K, S, V, R0 = workloads.composite_stack(16, 40, layers=3, seed=7)
    a = gpu_compose(pg, K, S, V, R0, "f32")
    b = gpu_compose(pg, K, S, V, R0, "f32", inplace=True)
    assert np.array_equal(a, b)
    z = gpu_compose(pg, K[:0], S[:0], V[:0], R0, "f32")
    assert np.array_equal(z, R0.astype(np.float64))


def test_fp32_vs_fp64_oracle_delta_e(pg, oracle):
    K, S, V, R0 = workloads.composite_stack(64, 128, layers=8, seed=8)
    got = gpu_compose(pg, K, S, V, R0, "f32")
    want = oracle_compose(oracle, K, S, V, R0, mode=1)
    de_max, _ = oracle.delta_e(np.moveaxis(got, 0, -1), np.moveaxis(want, 0, -1))
    assert de_max < 0.01


def test_canvas_compose_and_dry(pg, oracle):
    rows, cols = 23, 57
    rng = np.random.default_rng(2)
    K = rng.uniform(0.01, 5, (rows, cols, 3))
    S = rng.uniform(0.05, 3, (rows, cols, 3))
    V = np.where(rng.random((rows, cols)) < 0.3, 0.0, rng.uniform(0, 2, (rows, cols)))
    R0 = rng.uniform(0.8, 0.95, (rows, cols, 3))
    for storage, tol in (("f64", 1e-13), ("f32", 2e-5)):
        c = pg.Canvas(rows, cols, storage)
        oc = oracle.canvas(rows, cols)
        for p, a in (("K", K), ("S", S), ("V", V), ("R0", R0)):
            c.upload(p, a)
            oc.set(p, a)
        out = pg.Renderer().compose(c).download()
        assert np.abs(out - oc.compose()).max() <= tol
        c.dryCanvas()
        oc.dry()
        assert np.abs(c.getR0() - oc.get("R0")).max() <= tol
        assert np.abs(c.get_h() - oc.get("h")).max() <= 1e-6
        assert not c.download("V").any() and not c.download("K").any()


def test_upload_download_roundtrip(pg):
    rows, cols = 19, 77
    rng = np.random.default_rng(3)
    a = rng.random((rows, cols, 3))
    for storage in ("f32", "f64"):
        ly = pg.PaintLayer(rows, cols, storage)
        ly.upload("K", a)
        back = ly.download("K")
        tol = 0 if storage == "f64" else 1e-7
        assert np.abs(back - a).max() <= tol
        ly.upload("S", a.astype(np.float32))
        np.testing.assert_array_equal(ly.download("S", dtype=np.float32), a.astype(np.float32))
        planar = np.ascontiguousarray(np.moveaxis(a, -1, 0))
        ly.upload("K", planar, planar=True)
        assert np.abs(ly.download("K") - a).max() <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["f32", "f64", "f16"])
def test_layer_set_cells(pg, storage):
    """PaintLayer::set(i, j, k, s, v) on planar layers and a canvas's packed wet layer; the
    last of repeated cells wins."""
    rng = np.random.default_rng(8)
    for layer in (pg.PaintLayer(20, 30, storage), pg.Canvas(20, 30, storage).getPaintLayer()):
        rc = np.array([[0, 0], [5, 7], [19, 29], [5, 7], [10, 3]])
        K, S, V = rng.uniform(0, 5, (5, 3)), rng.uniform(0, 3, (5, 3)), rng.uniform(0, 1, 5)
        layer.setCells(rc, K, S, V)
        layer.setCell(10, 3, K[0], S[0], 0.25)
        gk, gs, gv = layer.download("K"), layer.download("S"), layer.download("V")
        want = {(0, 0): 0, (5, 7): 3, (19, 29): 2}
        tol = {"f64": 0.0, "f32": 1e-7, "f16": 2e-3}[storage]  # the storage's rounding
        for (r, c), m in want.items():
            np.testing.assert_allclose(gk[r, c], K[m], rtol=tol)
            np.testing.assert_allclose(gs[r, c], S[m], rtol=tol)
            np.testing.assert_allclose(gv[r, c], V[m], rtol=tol)
        np.testing.assert_allclose(gk[10, 3], K[0], rtol=tol)
        assert gv[10, 3] == 0.25  # exact in every storage
        assert gv.sum() == pytest.approx(sum(V[m] for m in want.values()) + 0.25, rel=1e-3)
    with pytest.raises(pg.PaintyValueError):
        pg.PaintLayer(4, 4, storage).setCell(4, 0, [1, 1, 1], [1, 1, 1], 1.0)


@pytest.mark.parametrize("rows,cols,L", [(37, 101, 3), (300, 130, 8), (9, 64, 17), (20, 20, 0)])
def test_host_composite_equals_device_composite(pg, rows, cols, L):
    """painty_compose_layers_host (host stacks in, host image out, transfers pipelined in row
    bands) equals painty_compose_layers on device layers bit for bit; 17 layers take two
    passes of the fused kernel, 0 layers return R0."""
    K, S, V, R0 = workloads.composite_stack(rows, cols, layers=max(L, 1), seed=rows + L)
    K, S, V = K[:L], S[:L], V[:L]
    got = pg.compose_layers_host(K, S, V, R0)
    want = gpu_compose(pg, K, S, V, R0) if L else R0.astype(np.float64)
    assert np.array_equal(got.astype(np.float64), want)


@pytest.mark.parametrize("rows,cols,L", [(64, 100, 8), (33, 37, 3), (16, 16, 18)])
def test_host_composite_pinned_in_place(pg, rows, cols, L):
    """With pinned host buffers the composite reads the stacks and writes the image in place
    (33 x 37 pixels, not a multiple of 4, take the banded copies instead): both equal the
    device composite bit for bit."""
    torch = pytest.importorskip("torch")
    K, S, V, R0 = workloads.composite_stack(rows, cols, layers=L, seed=rows * cols + L)

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
        t[...] = a
        return t

    out = pinned(np.zeros((3, rows, cols), np.float32))
    got = pg.compose_layers_host(pinned(K), pinned(S), pinned(V), pinned(R0), out=out)
    assert got is out
    want = gpu_compose(pg, K, S, V, R0)
    assert np.array_equal(out.astype(np.float64), want)
