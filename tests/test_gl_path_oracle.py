"""The oracle's restatement of painty's GL canvas path (gl_path.cpp): hand-derived cases of the
compute shaders, the texture dictionary's lookup and the strip raster + imprint; and the
compute passes bit for bit against painty's own shader sources compiled as C++
(oracle/glsl_ref.cpp), where the reference checkout is present."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def glsl_ref():
    from oracle.oracle import GlslReference
    if not GlslReference.available():
        pytest.skip("reference checkout not present (oracle/_ref cannot be built here)")
    return GlslReference()


def _gl_canvas(rng, rows, cols):
    """Random K4 / S4 / R4 with the edge cases the shaders branch on: V zero, below and just
    above the 1e-5 threshold, tiny S (|b S d| < 1e-5), large b S d (coth's > 20 branch)."""
    K4 = np.empty((rows, cols, 4), np.float32)
    S4 = np.empty((rows, cols, 4), np.float32)
    R4 = np.empty((rows, cols, 4), np.float32)
    K4[..., :3] = rng.uniform(0.0, 5.0, (rows, cols, 3))
    S4[..., :3] = rng.uniform(0.05, 3.0, (rows, cols, 3))
    K4[..., 3] = rng.choice([0.0, 5e-6, 1.1e-5, 0.01, 0.3, 1.0, 4.0, 40.0], (rows, cols)) * \
        rng.uniform(0.5, 1.5, (rows, cols))
    S4[..., 3] = rng.uniform(0.0, 2.0, (rows, cols))
    R4[..., :3] = rng.uniform(0.0, 1.0, (rows, cols, 3))
    R4[..., 3] = 1.0
    tiny = rng.random((rows, cols)) < 0.05
    S4[tiny, 0] = 1e-7
    zeroK = rng.random((rows, cols)) < 0.05
    K4[zeroK, 1] = 0.0
    return K4, S4, R4


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def test_compose_matches_painty_shader(oracle, glsl_ref):
    """ComposeLayerOnSubstrate.compute.glsl: the restatement equals painty's shader source
    compiled as C++, bit for bit, on a canvas whose size is not a multiple of the 16 x 16
    work group."""
    rng = np.random.default_rng(21)
    K4, S4, R4 = _gl_canvas(rng, 37, 53)
    assert _same(oracle.glsl_compose(K4, S4, R4), glsl_ref.compose(K4, S4, R4))


@pytest.mark.parametrize("portion", [0.0, 5e-6, 0.05, 0.5, 5.0])
def test_dry_step_matches_painty_shader(oracle, glsl_ref, portion):
    """DryingStep.compute.glsl: K4 (V) and R4 after one step, bit for bit."""
    rng = np.random.default_rng(22)
    K4, S4, R4 = _gl_canvas(rng, 29, 41)
    ko, ro = oracle.glsl_dry_step(K4, S4, R4, portion)
    kr, rr = glsl_ref.dry_step(K4, S4, R4, portion)
    assert _same(ko, kr) and _same(ro, rr)


@pytest.mark.parametrize("x0,y0,aoi_w,aoi_h", [(0, 0, 53, 37), (3, 2, 17, 9), (-5, -3, 20, 33),
                                                (40, 30, 30, 30), (-20, 10, 5, 1),
                                                (60, 0, 4, 4)])
def test_imprint_and_clear_match_painty_shaders(oracle, glsl_ref, x0, y0, aoi_w, aoi_h):
    """PaintTextureFootprintOnCanvas.compute.glsl and ClearTextureFootprint.compute.glsl over
    an area of interest (offset, whole 16 x 16 tiles, the flipped texture rows, the canvas
    bounds), on canvases with empty pixels and an empty texture in places, bit for bit."""
    rng = np.random.default_rng(abs(23 + x0 + 7 * y0))
    rows, cols = 37, 53
    K4, S4, _ = _gl_canvas(rng, rows, cols)
    K4[rng.random((rows, cols)) < 0.3, 3] = 0.0
    warped = rng.uniform(0.0, 1.0, (rows, cols)).astype(np.float32)
    warped[rng.random((rows, cols)) < 0.3] = 0.0
    Kb, Sb = rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)
    for scale in (0.0, 0.7, 2.5):
        ko, so = oracle.glsl_imprint(warped, K4, S4, x0, y0, aoi_w, aoi_h, Kb, Sb, scale)
        kr, sr = glsl_ref.imprint(warped, K4, S4, x0, y0, aoi_w, aoi_h, Kb, Sb, scale)
        assert _same(ko, kr) and _same(so, sr), scale
    assert _same(oracle.glsl_clear(warped, x0, y0, aoi_w, aoi_h),
                 glsl_ref.clear(warped, x0, y0, aoi_w, aoi_h))


def _glsl_reflectance_np(K, S, r0, d):
    """ComposeLayerOnSubstrate.compute.glsl:28-47 in float64 numpy (shader semantics)."""
    a = 1.0 + K / S
    b = np.sqrt(np.maximum(a * a - 1.0, 0.0))
    bSh = b * S * d
    if np.any(np.abs(bSh) < 1e-5):
        return r0
    bc = np.where(bSh > 20.0, 1.0, np.cosh(bSh) / np.sinh(bSh))
    return (1.0 - r0 * (a - bc)) / (a - r0 + bc)


def _px(K, S, V, R0, VL=0.0):
    K4 = np.array([[[*K, V]]], np.float32)
    S4 = np.array([[[*S, VL]]], np.float32)
    R4 = np.array([[[*R0, 1.0]]], np.float32)
    return K4, S4, R4


def test_glsl_compose_pixel(oracle):
    K, S, R0 = np.array([0.5, 1.2, 2.0]), np.array([0.7, 0.3, 1.1]), np.array([0.9, 0.85, 0.8])
    for V in (0.05, 0.4, 3.0):
        out = oracle.glsl_compose(*_px(K, S, V, R0))[0, 0]
        want = _glsl_reflectance_np(K.astype(np.float32).astype(np.float64),
                                    S.astype(np.float32).astype(np.float64),
                                    R0.astype(np.float32).astype(np.float64),
                                    np.float64(np.float32(V)))
        np.testing.assert_allclose(out[:3], want, rtol=2e-6, atol=2e-7)
        assert out[3] == 1.0


def test_glsl_compose_thresholds(oracle):
    R0 = np.array([0.9, 0.8, 0.7])
    # |d| <= 1e-5 keeps R0
    out = oracle.glsl_compose(*_px([1, 1, 1], [1, 1, 1], 1e-6, R0))[0, 0]
    np.testing.assert_array_equal(out[:3], R0.astype(np.float32))
    # K = 0 in one channel: b = 0 there, so |bSh| < 1e-5 and the shader keeps R0 (the CPU
    # path gives NaN)
    out = oracle.glsl_compose(*_px([0, 1, 1], [1, 1, 1], 0.5, R0))[0, 0]
    np.testing.assert_array_equal(out[:3], R0.astype(np.float32))


def test_glsl_dry_step(oracle):
    K, S, R0 = np.array([0.5, 1.2, 2.0]), np.array([0.7, 0.3, 1.1]), np.array([0.9, 0.85, 0.8])
    K4, S4, R4 = _px(K, S, 0.25, R0)
    k1, r1 = oracle.glsl_dry_step(K4, S4, R4, 0.1)
    assert k1[0, 0, 3] == np.float32(np.float32(0.25) - np.float32(0.1))
    np.testing.assert_array_equal(k1[0, 0, :3], K4[0, 0, :3])
    want = oracle.glsl_compose(*_px(K, S, np.float32(0.25) - k1[0, 0, 3], R0))[0, 0]
    np.testing.assert_array_equal(r1[0, 0], want)
    # less paint than the portion: all of it dries
    k2, r2 = oracle.glsl_dry_step(k1, S4, r1, 1.0)
    assert k2[0, 0, 3] == 0.0


def _dictionary(oracle, seed=3):
    rng = np.random.default_rng(seed)
    d = oracle.texture_dictionary(seed)
    idx = {}
    for rc, rows in ((4, 10), (16, 34)):
        for lc, cols in ((50, 60), (200, 220)):
            for k in range(3):
                idx[(rc, lc, k)] = d.add(rc, lc, rng.random((rows, cols)))
    return d, idx


def test_dictionary_lookup_classes(oracle):
    d, idx = _dictionary(oracle)
    short = np.array([[0.0, 0.0], [50.0, 0.0]])
    long_ = np.array([[0.0, 0.0], [100.0, 0.0], [200.0, 10.0]])
    # brush size 10 -> size class of 10-row textures; short path -> 60-col class
    for _ in range(5):
        assert d.lookup(short, 10.0) in {idx[(4, 50, k)] for k in range(3)}
        assert d.lookup(long_, 33.0) in {idx[(16, 200, k)] for k in range(3)}
    # the seeded pick repeats
    a = [oracle.texture_dictionary(9) for _ in range(2)]
    rng = np.random.default_rng(0)
    for x in a:
        for k in range(4):
            x.add(8, 40, rng.random((12, 40)) + k)
    assert [a[0].lookup(short, 12.0) for _ in range(8)] == [a[1].lookup(short, 12.0) for _ in range(8)]


def test_gpu_texture_brush_straight_stroke(oracle):
    """Texture rows ramp 0..1 down the image: the strip's right side (t = 0, GL's bottom row =
    the image's last row) carries the high end; V and the lighting volume follow the texture."""
    d = oracle.texture_dictionary(1)
    rows_t, cols_t = 16, 64
    ramp = np.repeat(np.linspace(0.0, 1.0, rows_t)[:, None], cols_t, axis=1)
    d.add(5, 60, ramp)
    b = oracle.gpu_texture_brush()
    b.set_radius(8.0)
    b.dip(np.array([1.0, 2.0, 3.0]), np.array([0.5, 0.6, 0.7]))
    H, W = 64, 96
    K4 = np.zeros((H, W, 4), np.float32)
    S4 = np.zeros((H, W, 4), np.float32)
    path = np.array([[10.0, 32.0], [50.0, 32.0], [86.0, 32.0]])
    assert b.paint_stroke(d, K4, S4, path) == 0
    V = K4[..., 3]
    # heading +x: d = (-t.y, t.x) = (0, 1), so the right side (c + r d) is at y = 40
    assert V[39, 48] > V[25, 48] > 0.0
    assert V[39, 48] > 0.8 and V[25, 48] < 0.2
    assert V[5, 48] == 0.0 and V[60, 48] == 0.0
    painted = V > 0
    np.testing.assert_allclose(K4[painted][:, :3],
                               np.broadcast_to(np.float32([1.0, 2.0, 3.0]), (painted.sum(), 3)),
                               rtol=1e-6)
    np.testing.assert_array_equal(S4[..., 3], V)  # empty canvas: lighting volume = Vtex = V
    assert not oracle_warped_any(b, H, W)


def oracle_warped_any(b, H, W):
    import ctypes as C
    ptr = b._warped(b.h)
    a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float)), (H * W,))
    return bool(a.any())


def test_gpu_texture_brush_rounds_the_dispatch_up(oracle):
    """The imprint covers the stroke bounds' 16 x 16 tiles: there, existing paint with no new
    paint gets its lighting volume set to its volume."""
    d = oracle.texture_dictionary(1)
    d.add(5, 60, np.random.default_rng(2).random((16, 64)))
    b = oracle.gpu_texture_brush()
    b.set_radius(3.0)
    H, W = 64, 64
    K4 = np.zeros((H, W, 4), np.float32)
    S4 = np.zeros((H, W, 4), np.float32)
    K4[..., 3] = 0.5  # existing paint everywhere, lighting volume 0
    K4[..., :3] = 1.0
    path = np.array([[10.0, 10.0], [14.0, 10.0]])
    b.paint_stroke(d, K4, S4, path)
    # bounds x 7..17 (width 11 -> one tile: x 7..22), y 7..13 (one tile: y 7..22)
    assert S4[20, 21, 3] == 0.5 and S4[20, 23, 3] == 0.0 and S4[23, 20, 3] == 0.0
    assert S4[6, 10, 3] == 0.0


@pytest.fixture(scope="module")
def tdict_ref():
    from oracle.oracle import TDictReference
    if not TDictReference.available():
        pytest.skip("reference checkout not present (oracle/_ref cannot be built here)")
    return TDictReference()


def _length_class(avg_lengths, n_size, length, truncate):
    """lookup's length scan (TextureBrushDictionary.cxx:45-53): the initial best "distance" is
    the first class's mean length and the initial index 1; `truncate` takes the distance as
    abs(int(x)), the abs(int) overload."""
    ml, i1 = avg_lengths[0], 1
    for i in range(n_size):
        x = avg_lengths[i] - length
        d = float(abs(int(x))) if truncate else abs(x)
        if d < ml:
            ml, i1 = d, i
    return i1


def test_texture_dictionary_matches_painty(oracle, tdict_ref, tmp_path):
    """painty's own TextureBrushDictionary.cxx (file-name classes, class averages, the two
    min-max normalisations, the flip into GL rows, lookup's class choice) against the oracle:
    the same class for every lookup and the same GL texture for every entry painty picks.

    Two kinds of input are left out, where painty's code has no single meaning. With fewer
    length classes than size classes the length scan runs past them (TextureBrushDictionary.cxx:
    45-53). And the scan takes an unqualified abs() of a double (:48): libstdc++ without the
    C++ <math.h> resolves it to abs(int), which truncates the distance (as this build does),
    other standard libraries to the double overload (as the oracle does); lookups whose class
    depends on that choice are checked against the truncating reading only. painty's random
    pick among a class's candidates (std::random_device) is not reproducible, so picks are
    compared by class."""
    rng = np.random.default_rng(31)
    entries = []
    for rc, rows in ((3, 6), (9, 18), (27, 54)):
        for lc, cols in ((20, 30), (90, 100), (300, 320)):
            for k in range(2 if (rc, lc) in ((9, 90), (27, 20)) else 1):
                entries.append((rc, lc, rng.random((rows + 2 * k, cols + 3 * k))))
    names = tdict_ref.build(tmp_path, entries)
    o = oracle.texture_dictionary(5)
    for rc, lc, tex in entries:
        o.add(rc, lc, tex)
    cls = {n: (rc, lc) for n, (rc, lc, _) in zip(names, entries)}
    sizes, lengths = (3, 9, 27), (20, 90, 300)
    avg_rows = [np.mean([t.shape[0] for r, _, t in entries if r == rc]) for rc in sizes]
    avg_cols = [[np.mean([t.shape[1] for r, l, t in entries if r == rc and l == lc])
                 for lc in lengths] for rc in sizes]
    cases = [(float(rng.uniform(1.0, 700.0)), float(rng.uniform(1.0, 90.0))) for _ in range(600)]
    for i0 in range(len(sizes)):  # lengths whose class depends on the abs() overload
        grid = [L for L in np.arange(1.0, 700.0, 0.05)
                if _length_class(avg_cols[i0], len(sizes), L, False) !=
                _length_class(avg_cols[i0], len(sizes), L, True)]
        cases += [(float(L), float(avg_rows[i0])) for L in grid[::max(1, len(grid) // 5)]]
    checked = ambiguous = 0
    for length, size in cases:
        path = np.array([[3.0, 4.0], [3.0 + length, 4.0]])
        src, tex = tdict_ref.lookup(path, size)
        mr, i0 = avg_rows[0], 0
        for i, a in enumerate(avg_rows):
            if abs(a - size) < mr:
                mr, i0 = abs(a - size), i
        wide = _length_class(avg_cols[i0], len(sizes), length, truncate=False)
        narrow = _length_class(avg_cols[i0], len(sizes), length, truncate=True)
        if wide != narrow:
            assert cls[src] == (sizes[i0], lengths[narrow]), (length, size)
            ambiguous += 1
            continue
        k = o.lookup(path, size)
        assert cls[src] == entries[k][:2] == (sizes[i0], lengths[wide]), (length, size)
        assert np.array_equal(tex, o.texture(names.index(src))), (length, size)
        checked += 1
    assert checked > 450 and ambiguous > 0


def test_strip_vertices_match_painty_spline(oracle, reference):
    """TextureBrushGpu's triangle strip (spine points and unit tangents from painty's own
    SplineEval, offset by the radius, as floats) equals the oracle's, bit for bit, for paths of
    2 to 9 points, straight, random and with repeated points."""
    rng = np.random.default_rng(41)
    paths = [np.array([[0.0, 0.0], [10.0, 0.0]]), np.array([[5.0, 5.0], [5.0, 5.0], [9.0, 2.0]])]
    paths += [rng.uniform(-50, 400, (int(rng.integers(2, 10)), 2)) for _ in range(40)]
    for path in paths:
        for radius in (0.5, 3.7, 25.0):
            xo, uo = oracle.gl_strip_vertices(path, radius)
            xr, ur = reference.gl_strip_vertices(path, radius)
            assert _same(xo, xr) and _same(uo, ur), (path, radius)
