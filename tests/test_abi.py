"""The C ABI library: it loads and exports every entry point the public header declares."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include/painty_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(painty_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "painty_compose_layers" in names and "painty_stamps" in names
    assert len(names) >= 40


def test_library_exports_all_declared(pg):
    lib = ctypes.CDLL(str(pg.LIB_PATH))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_status_strings(pg):
    assert pg.ABI_VERSION == 2
    lib = pg._lib
    for s in range(0, 9):
        assert lib.painty_status_string(s)


def test_invalid_arguments_rejected_without_gpu(pg):
    import numpy as np
    import pytest
    with pytest.raises(ValueError):
        pg.Canvas(0, 10)
    with pytest.raises(ValueError):
        pg.FootprintBrush(float("nan"), np.ones((4, 4)))
    with pytest.raises(ValueError):
        pg.mix_single_paint(np.ones(3), np.ones((2, 3)), np.ones((2, 3)))


def test_mix_paint_matches_reference_formula(pg, oracle):
    import numpy as np
    from painty_gb300 import workloads
    K, S = workloads.pigments()
    w = np.random.default_rng(3).dirichlet(np.full(14, 0.3))
    k1, s1 = pg.mix_single_paint(w, K, S)
    k2, s2 = oracle.mix_single_paint(w, K, S)
    assert np.array_equal(k1, k2) and np.array_equal(s1, s2)


def test_texture_and_gl_brush_arguments_rejected_without_gpu(pg):
    import numpy as np
    import pytest
    tex = np.random.default_rng(0).random((8, 16))
    with pytest.raises(ValueError):
        pg.TextureBrush(np.zeros((0, 4)))
    b = pg.TextureBrush(tex)
    for bad in (float("nan"), -1.0, 2e6):
        with pytest.raises(ValueError):
            b.setRadius(bad)
    with pytest.raises(ValueError):
        b.setThicknessScale(float("inf"))
    d = pg.TextureBrushDictionary(1)
    with pytest.raises(ValueError):
        d.add(1, 1, np.zeros((0, 3)))
    with pytest.raises(ValueError):
        d.add(1, 1, np.array([[1.0, float("nan")]]))
    with pytest.raises(ValueError):  # empty dictionary
        d.lookup(np.array([[0.0, 0.0], [5.0, 0.0]]), 4.0)
    d.add(4, 10, tex)
    assert d.lookup(np.array([[0.0, 0.0], [5.0, 0.0]]), 8.0) == 0
    g = pg.TextureBrushGpu(d)
    with pytest.raises(ValueError):
        g.setRadius(-3.0)
    with pytest.raises(pg.PaintyError):
        g.enableSmudge(True)
    assert g.lastTexture() == -1


def test_texture_dictionary_lookup_matches_oracle(pg, oracle):
    """The class choice of TextureBrushDictionary::lookup, including painty's initial length
    class 1 and its first-size-class distance, agrees with the oracle's restatement."""
    import numpy as np
    rng = np.random.default_rng(5)
    d, o = pg.TextureBrushDictionary(9), oracle.texture_dictionary(9)
    for rc, rows in ((3, 6), (9, 18), (27, 54)):
        for lc, cols in ((20, 30), (90, 100), (300, 320)):
            for k in range(2):
                t = rng.random((rows, cols))
                d.add(rc, lc, t)
                o.add(rc, lc, t)
    for trial in range(60):
        n = int(rng.integers(2, 6))
        path = rng.uniform(0, 400, (n, 2))
        size = float(rng.uniform(1, 80))
        assert d.lookup(path, size) == o.lookup(path, size)


def test_bounds_checked_build_exports_and_reports_itself(pg):
    """The bounds-checked twin library loads without a GPU, exports every declared entry and
    reports its build flag; the default library does not set it."""
    checked = pg.LIB_PATH.parent / "libpainty_gb300_checked.so"
    lib = ctypes.CDLL(str(checked))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    lib.painty_build_flags.restype = ctypes.c_int32
    assert lib.painty_build_flags() & 1
    assert pg.bounds_checked() == pg.BOUNDS_CHECKED


def test_phase_timing_build_exports_and_reports_itself(pg):
    """The phase-timing twin library loads without a GPU, exports every declared entry and
    reports its build flag; in the default build the phase counters are unsupported."""
    phases = pg.LIB_PATH.parent / "libpainty_gb300_phases.so"
    lib = ctypes.CDLL(str(phases))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    lib.painty_build_flags.restype = ctypes.c_int32
    assert lib.painty_build_flags() & 2 and not lib.painty_build_flags() & 1
    if not pg.PHASE_TIMERS:
        out = (ctypes.c_uint64 * 16)()
        assert pg._lib.painty_take_phase_cycles(out) == 4  # PAINTY_ERR_UNSUPPORTED


def test_brush_host_setup_matches_oracle_without_gpu(pg, oracle):
    """Brush setup is host code: the radius rule (changes below 0.5 ignored, so a brush created
    below 0.5 keeps an empty footprint, FootprintBrush.hxx:46-63), the resampled footprint and
    the map sizes agree with the oracle bit for bit, through a sequence of setRadius calls."""
    import numpy as np
    from painty_gb300 import workloads
    fp = workloads.footprint_image(seed=9)
    for r0, steps in ((0.0, (0.3, 0.6, 0.9, 1.2)), (0.3, (0.49, 3.0, 3.4, 2.4)),
                      (12.0, (12.45, 11.6, 64.0, 0.2))):
        b, ob = pg.FootprintBrush(r0, fp), oracle.brush(r0, fp)
        for r in (r0,) + steps:
            b.setRadius(r)
            ob.set_radius(r)
            assert b.info() == ob.info(), (r0, r)
            if b.info()[1]:
                assert np.array_equal(b.getFootprint(), ob.footprint()), (r0, r)
