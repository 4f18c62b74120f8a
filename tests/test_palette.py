"""Palette JSON I/O (LoadPalette / SavePalette, Serialization.cxx:38-53) and the swatch image
(VisualizePalette, :64-137)."""
import io
import os
from pathlib import Path

import numpy as np
import pytest

from painty_gb300 import palette as P

# paints from painty's SerializationTest (SerializationTest.cxx:28-34), re-typed as data
SMALL = [(np.array([0.0, 0.5, 1.0]), np.array([0.2, 0.3, 0.4])),
         (np.array([0.22, 1.47, 0.57]), np.array([0.05, 0.003, 0.03]))]


def test_save_load_round_trip(tmp_path):
    f = tmp_path / "p.json"
    P.save_palette(f, SMALL)
    back = P.load_palette(f)
    assert len(back) == 2
    for (K, S), (K2, S2) in zip(SMALL, back):
        assert np.array_equal(K, K2) and np.array_equal(S, S2)


def test_compact_sorted_output():
    """nlohmann::json's `stream << j`: no spaces, object keys in sorted order."""
    assert P.dumps_palette(SMALL[:1]) == '[{"K":[0.0,0.5,1.0],"S":[0.2,0.3,0.4]}]'


def test_load_rejects_incomplete_entries():
    with pytest.raises(ValueError):
        P.load_palette(io.StringIO('[{"K":[1,2,3]}]'))
    with pytest.raises(ValueError):
        P.load_palette(io.StringIO('[{"K":[1,2],"S":[1,2,3]}]'))


def test_load_reference_palettes():
    """painty's own palette files, where the checkout is present (14-pigment measured set)."""
    root = Path(os.environ.get("PAINTY_REFERENCE_ROOT", "/root/reference")) / "data" / "paint_palettes"
    if not root.is_dir():
        pytest.skip("reference checkout not present")
    pal = P.load_palette(root / "lindemeier-measured.json")
    assert len(pal) == 14
    assert all(K.shape == (3,) and S.shape == (3,) for K, S in pal)
    assert len(P.load_palette(root / "curtis-watercolor.json")) == 13


def test_rgb2srgb():
    x = np.array([0.0, 0.002, 0.00313066844250063, 0.5, 1.0])
    s = P.rgb2srgb(x)
    assert s[0] == 0.0 and s[1] == 0.002 * 12.92 and s[-1] == pytest.approx(1.0, abs=1e-12)
    assert s[3] == 1.055 * 0.5 ** (1.0 / 2.4) - 0.055


@pytest.mark.gpu
def test_visualize_palette_vs_oracle(pg, oracle):
    img = P.visualize_palette(SMALL, 0.5)
    assert img.shape == (200, 200, 3)
    for c, (K, S) in enumerate(SMALL):
        ow = P.rgb2srgb(oracle.compute_reflectance(K, S, np.ones(3), 0.5))
        ob = P.rgb2srgb(oracle.compute_reflectance(K, S, np.zeros(3), 0.5))
        x = 100 * c + 50
        np.testing.assert_allclose(img[50, x], ow, rtol=1e-12)
        np.testing.assert_allclose(img[150, x], ob, rtol=1e-12)
        assert (img[:20, x] == 1.0).all() and (img[80:100, x] == 1.0).all()
        assert (img[100:120, x] == 0.0).all() and (img[180:, x] == 0.0).all()
        np.testing.assert_array_equal(img[20:80, x], np.broadcast_to(img[50, x], (60, 3)))


@pytest.fixture(scope="module")
def painty_ref():
    from oracle.oracle import Reference
    if not Reference.available():
        pytest.skip("reference checkout not present (oracle/_ref cannot be built here)")
    return Reference()


def test_load_palette_matches_painty(painty_ref):
    """painty's own LoadPalette (Serialization.cxx:38-44, its JSON library replaced by a
    stand-in that reads numbers as nlohmann does) and load_palette read the same paints, bit for
    bit: painty's palette files, and texts with integers, exponents, extra keys and spacing."""
    texts = ['[{"K":[1,2,3],"S":[4,5,6]}]',
             '[ {"S": [0.2, 3e-3, 1E2], "K": [0.1, -0.5, 7.25e+1], "name": "x"} ,\n'
             '  {"K":[0.30000000000000004,1e-320,123456789012],"S":[1,0.5,0.25]} ]',
             '[]']
    root = Path(os.environ.get("PAINTY_REFERENCE_ROOT", "/root/reference")) / "data" / "paint_palettes"
    if root.is_dir():
        texts += [f.read_text() for f in sorted(root.glob("*.json"))]
    for text in texts:
        ours = P.load_palette(io.StringIO(text))
        theirs = painty_ref.load_palette(text)
        assert len(ours) == len(theirs)
        for (K, S), (K2, S2) in zip(ours, theirs):
            assert np.array_equal(K, K2) and np.array_equal(S, S2), text[:60]


def test_visualize_palette_layout_matches_painty(painty_ref, oracle, monkeypatch):
    """visualize_palette's bands, widths and sRGB conversion against painty's own
    VisualizePalette (Serialization.cxx:64-137), bit for bit, with the reflectances taken from
    the oracle (painty's ComputeReflectance, bit for bit) instead of the GPU composite."""
    def reflectance(palette, thickness, background):
        bg = np.asarray(background, dtype=np.float64)
        return np.array([oracle.compute_reflectance(K, S, bg, thickness) for K, S in palette])

    monkeypatch.setattr(P, "palette_reflectance", reflectance)
    rng = np.random.default_rng(12)
    palettes = [SMALL, SMALL[:1],
                [(rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)) for _ in range(7)]]
    for pal in palettes:
        for t in (0.05, 0.5, 3.0):
            # NaN where K = 0: painty's formula (0 * coth 0) kept as it is
            assert np.array_equal(P.visualize_palette(pal, t), painty_ref.visualize_palette(pal, t),
                                  equal_nan=True)
