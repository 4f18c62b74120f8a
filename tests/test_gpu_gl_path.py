"""painty's GL canvas path (CanvasGpu / TextureBrushGpu shaders) as CUDA vs the oracle's float
restatement. The strip raster and imprint use exact integer coverage and float arithmetic
without fused multiply-adds on both sides: F32 canvases must match bit for bit. The compose
and dry-step shaders call cosh / sinh, whose last bits differ between CUDA and the host libm:
those compare within GL_REL_TOL."""
import numpy as np
import pytest

from test_gl_path_oracle import _dictionary

pytestmark = pytest.mark.gpu

GL_REL_TOL = 2e-5  # compose / dry step: relative difference of R (cosh, sinh ulps)
F16_ABS_TOL = 4e-3  # 16-bit storage: K, S relative and V absolute difference after strokes


def _random_gl_canvas(pg, rows, cols, storage="f32", seed=0, paint=True):
    rng = np.random.default_rng(seed)
    K = rng.uniform(0.01, 5.0, (rows, cols, 3)).astype(np.float32)
    S = rng.uniform(0.05, 3.0, (rows, cols, 3)).astype(np.float32)
    V = (rng.uniform(0.0, 1.0, (rows, cols)) * (rng.random((rows, cols)) < 0.7)).astype(np.float32)
    VL = rng.uniform(0.0, 1.0, (rows, cols)).astype(np.float32)
    R0 = rng.uniform(0.8, 0.95, (rows, cols, 3)).astype(np.float32)
    if not paint:
        K[:] = 0
        S[:] = 0
        V[:] = 0
        VL[:] = 0
    c = pg.Canvas(rows, cols, storage)
    c.upload("K", K)
    c.upload("S", S)
    c.upload("V", V)
    c.upload("VL", VL)
    c.upload("R0", R0)
    # what the canvas stores (16-bit storage rounds on upload)
    K = c.download("K", dtype=np.float32)
    S = c.download("S", dtype=np.float32)
    V = c.download("V", dtype=np.float32)
    VL = c.download("VL", dtype=np.float32)
    K4 = np.ascontiguousarray(np.concatenate([K, V[..., None]], axis=-1))
    S4 = np.ascontiguousarray(np.concatenate([S, VL[..., None]], axis=-1))
    R4 = np.ascontiguousarray(np.concatenate([R0, np.ones((rows, cols, 1), np.float32)], axis=-1))
    return c, K4, S4, R4


def _gl_state(c):
    K = c.download("K", dtype=np.float32)
    S = c.download("S", dtype=np.float32)
    V = c.download("V", dtype=np.float32)
    VL = c.download("VL", dtype=np.float32)
    return (np.concatenate([K, V[..., None]], axis=-1), np.concatenate([S, VL[..., None]], axis=-1))


def test_compose_glsl_vs_oracle(pg, oracle):
    c, K4, S4, R4 = _random_gl_canvas(pg, 70, 90)
    got = c.getComposedGlsl().download(dtype=np.float64)
    want = oracle.glsl_compose(K4, S4, R4)[..., :3].astype(np.float64)
    np.testing.assert_allclose(got, want, rtol=GL_REL_TOL, atol=1e-6)
    # R0 untouched (the shader composes onto a copy)
    np.testing.assert_array_equal(c.download("R0", dtype=np.float32), R4[..., :3])


def test_dry_step_vs_oracle(pg, oracle):
    c, K4, S4, R4 = _random_gl_canvas(pg, 60, 50, seed=1)
    for portion in (0.1, 0.25, 1.0):
        c.dryStep(portion)
        K4, R4 = oracle.glsl_dry_step(K4, S4, R4, portion)
        np.testing.assert_array_equal(c.download("V", dtype=np.float32), K4[..., 3])
        np.testing.assert_allclose(c.download("R0"), R4[..., :3], rtol=GL_REL_TOL, atol=1e-6)
        R4[..., :3] = c.download("R0", dtype=np.float32)  # continue from the same state
    assert not c.download("V").any()


def _dictionaries(pg, oracle, seed):
    """The same texture dictionary in the oracle and the library (two size and two length
    classes of three textures each)."""
    od, _ = _dictionary(oracle, seed=seed)
    gd = pg.TextureBrushDictionary(seed)
    rng = np.random.default_rng(seed)
    for rc, nr in ((4, 10), (16, 34)):
        for lc, nc in ((50, 60), (200, 220)):
            for k in range(3):
                gd.add(rc, lc, rng.random((nr, nc)))
    return od, gd


def _stroke_session(rng, rows, cols, n):
    out = []
    for _ in range(n):
        k = int(rng.integers(2, 7))
        path = np.stack([rng.uniform(-15, cols + 15, k), rng.uniform(-15, rows + 15, k)], axis=1)
        out.append((path, float(rng.uniform(2.0, 20.0)), rng.uniform(0.01, 5, 3),
                    rng.uniform(0.05, 3, 3), float(rng.uniform(0.5, 2.0))))
    return out


@pytest.mark.parametrize("paint", [False, True])
def test_texture_brush_gpu_bitexact_vs_oracle(pg, oracle, paint):
    rows, cols = 96, 128
    c, K4, S4, _ = _random_gl_canvas(pg, rows, cols, seed=5, paint=paint)
    od, gd = _dictionaries(pg, oracle, 3)
    ob = oracle.gpu_texture_brush()
    gb = pg.TextureBrushGpu(gd)
    for path, r, K, S, scale in _stroke_session(np.random.default_rng(11 + paint), rows, cols, 10):
        for b in (ob, gb):
            (b.set_radius if b is ob else b.setRadius)(r)
        ob.dip(K, S)
        gb.dip((K, S))
        ob.set_thickness_scale(scale)
        gb.setThicknessScale(scale)
        assert ob.paint_stroke(od, K4, S4, path) == 0
        gb.paintStroke(path, c)
        assert gb.lastTexture() == ob.last_texture()
    gk, gs = _gl_state(c)
    np.testing.assert_array_equal(gk, K4)
    np.testing.assert_array_equal(gs, S4)
    assert (K4[..., 3] > 0).mean() > 0.2


@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_texture_brush_gpu_16bit(pg, oracle, storage):
    rows, cols = 64, 80
    c, K4, S4, _ = _random_gl_canvas(pg, rows, cols, storage=storage, seed=2, paint=False)
    od, gd = _dictionaries(pg, oracle, 7)
    ob = oracle.gpu_texture_brush()
    gb = pg.TextureBrushGpu(gd)
    for path, r, K, S, scale in _stroke_session(np.random.default_rng(8), rows, cols, 5):
        ob.set_radius(r)
        gb.setRadius(r)
        ob.dip(K, S)
        gb.dip((K, S))
        assert ob.paint_stroke(od, K4, S4, path) == 0
        gb.paintStroke(path, c)
    gk, gs = _gl_state(c)
    tol = 8e-3 if storage == "bf16" else F16_ABS_TOL
    np.testing.assert_allclose(gk[..., :3], K4[..., :3], rtol=tol, atol=1e-3)
    np.testing.assert_allclose(gs[..., :3], S4[..., :3], rtol=tol, atol=1e-3)
    np.testing.assert_allclose(gk[..., 3], K4[..., 3], rtol=1e-3, atol=1e-3)


def test_gl_path_errors(pg):
    gd = pg.TextureBrushDictionary(0)
    gb = pg.TextureBrushGpu(gd)
    with pytest.raises(pg.PaintyError):
        gb.enableSmudge(True)
    gb.enableSmudge(False)
    with pytest.raises(pg.PaintyError):  # empty dictionary
        gb.paintStroke(np.array([[1.0, 1.0], [5.0, 5.0]]), pg.Canvas(16, 16, "f32"))
    gd.add(4, 10, np.random.default_rng(0).random((8, 10)))
    with pytest.raises(pg.PaintyError):  # the GL path is float
        gb.paintStroke(np.array([[1.0, 1.0], [5.0, 5.0]]), pg.Canvas(16, 16, "f64"))
    with pytest.raises(pg.PaintyError):
        pg.Canvas(16, 16, "f64").dryStep(0.1)
    gb.paintStroke(np.array([[1.0, 1.0]]), pg.Canvas(16, 16, "f32"))  # one point: nothing


def test_sbr_render_thread_matches_direct_calls(pg):
    """SbrRenderThread's worker paints what direct TextureBrushGpu calls paint (drying off)."""
    rows, cols = 80, 100
    rng = np.random.default_rng(6)
    textures = [((4, 50), rng.random((10, 60))), ((4, 200), rng.random((10, 220))),
                ((16, 50), rng.random((34, 60))), ((16, 200), rng.random((34, 220)))]
    strokes = _stroke_session(np.random.default_rng(2), rows, cols, 8)
    bg = np.full((rows, cols, 3), 0.85)
    d1, d2 = pg.TextureBrushDictionary(4), pg.TextureBrushDictionary(4)
    for (rc, lc), t in textures:
        d1.add(rc, lc, t)
        d2.add(rc, lc, t)
    sbr = pg.SbrRenderThread(rows, cols, d1, background=bg, dry_interval=0.0)
    futs = [sbr.render(p, r, (K, S)) for p, r, K, S, _ in strokes]
    img = sbr.getLinearRgbImage().result()
    assert all(f.done() for f in futs)
    sbr.dryCanvas().result()
    dried = sbr.getLinearRgbImage().result()
    sbr.close()
    c = pg.Canvas(rows, cols, "f32")
    c.setBackground(bg)
    b = pg.TextureBrushGpu(d2)
    for p, r, K, S, _ in strokes:
        b.dip((K, S))
        b.setRadius(r)
        b.paintStroke(p, c)
    np.testing.assert_array_equal(img, c.getComposedGlsl().download())
    c.dryStep(1.0)
    np.testing.assert_array_equal(dried, c.getComposedGlsl().download())
    with pytest.raises(pg.PaintyError):
        pg.SbrRenderThread(8, 8, d1, dry_interval=0.0).enableSmudge(True)
