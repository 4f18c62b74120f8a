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
    assert pg.ABI_VERSION == 1
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
