"""Paint palettes: painty's JSON palette files and the palette swatch image.

LoadPalette / SavePalette (painty/mixer/src/Serialization.cxx:38-53) read and write a JSON
array of {"K": [r, g, b], "S": [r, g, b]} objects (nlohmann::json, keys sorted, compact);
VisualizePalette (:64-137) paints each paint's Kubelka-Munk reflectance at a given thickness
on white and on black into a 200 x 100n swatch image (sRGB). The reflectances come from the
library's composite kernel on an F64 layer (painty's ComputeReflectance arithmetic).
"""
from __future__ import annotations

import io
import json
import math
import os
from typing import IO, Iterable

import numpy as np

Palette = list  # of (K (3,), S (3,)) pairs, painty::Palette of PaintCoeff


def _coeffs(v, key: str) -> np.ndarray:
    try:
        vals = [float(v[key][i]) for i in range(3)]  # nlohmann's j.at("K").at(0..2)
    except (KeyError, IndexError, TypeError) as e:
        raise ValueError(f"palette entry without three {key} coefficients") from e
    return np.array(vals)


def load_palette(src: str | os.PathLike | IO[str]) -> Palette:
    """LoadPalette (Serialization.cxx:38-44): the paints of a JSON palette, in file order."""
    if isinstance(src, (str, os.PathLike)):
        with open(src, "r", encoding="utf-8") as f:
            data = json.load(f)
    else:
        data = json.load(src)
    if not isinstance(data, (list, dict)):
        raise ValueError("a palette is a JSON array of {K, S} objects")
    items = data if isinstance(data, list) else list(data.values())
    return [(_coeffs(e, "K"), _coeffs(e, "S")) for e in items]


def save_palette(dst: str | os.PathLike | IO[str], palette: Iterable) -> None:
    """SavePalette (Serialization.cxx:46-53): compact JSON, keys in sorted order."""
    arr = [{"K": [float(x) for x in K], "S": [float(x) for x in S]} for K, S in palette]
    text = json.dumps(arr, separators=(",", ":"), sort_keys=True)
    if isinstance(dst, (str, os.PathLike)):
        with open(dst, "w", encoding="utf-8") as f:
            f.write(text)
    else:
        dst.write(text)


def dumps_palette(palette: Iterable) -> str:
    buf = io.StringIO()
    save_palette(buf, palette)
    return buf.getvalue()


def rgb2srgb(lin: np.ndarray) -> np.ndarray:
    """ColorConverter::rgb2srgb (painty/core/Color.hxx:198-206), value by value with the C
    library's pow (math.pow), as painty's std::pow: numpy's vectorised power can differ from it
    in the last bit. NaN stays NaN."""
    lin = np.asarray(lin, dtype=np.float64)
    out = np.empty_like(lin)
    flat, res = lin.reshape(-1), out.reshape(-1)
    for i, v in enumerate(flat.tolist()):
        if v <= 0.00313066844250063:
            res[i] = v * 12.92
        elif v == v:
            res[i] = 1.055 * math.pow(v, 1.0 / 2.4) - 0.055
        else:
            res[i] = v
    return out


def palette_reflectance(palette: Palette, thickness: float, background) -> np.ndarray:
    """(n, 3) reflectance of each paint at `thickness` over `background` (linear RGB), by the
    library's composite (one F64 layer of n pixels)."""
    from . import Image, PaintLayer, compose_layers

    n = len(palette)
    lay = PaintLayer(1, n, "f64")
    lay.upload("K", np.array([K for K, _ in palette], dtype=np.float64).reshape(1, n, 3))
    lay.upload("S", np.array([S for _, S in palette], dtype=np.float64).reshape(1, n, 3))
    lay.upload("V", np.full((1, n), float(thickness)))
    r0 = Image(1, n, "f64")
    r0.upload(np.broadcast_to(np.asarray(background, dtype=np.float64), (1, n, 3)).copy())
    out = Image(1, n, "f64")
    compose_layers([lay], r0, out)
    return out.download(dtype=np.float64).reshape(n, 3)


def visualize_palette(palette: Palette, applied_thickness: float) -> np.ndarray:
    """VisualizePalette (Serialization.cxx:64-137): (200, 100 n, 3) sRGB swatches -- per paint
    a white band, the paint on white, white, black, the paint on black, black."""
    n = len(palette)
    img = np.zeros((200, 100 * n, 3))
    if n == 0:
        return img
    on_white = rgb2srgb(palette_reflectance(palette, applied_thickness, [1.0, 1.0, 1.0]))
    on_black = rgb2srgb(palette_reflectance(palette, applied_thickness, [0.0, 0.0, 0.0]))
    h = float(img.shape[0])
    width = img.shape[1] // n
    # band edges: painty's loops run y from int(f0 * h) while y < f1 * h
    bands = [(0.0, 0.1, None), (0.1, 0.4, "white"), (0.4, 0.5, 1.0), (0.5, 0.6, 0.0),
             (0.6, 0.9, "black"), (0.9, 1.0, 0.0)]
    for c in range(n):
        cols = slice(c * width, (c + 1) * width)
        for f0, f1, what in bands:
            y0 = int(f0 * h)
            y1 = int(np.ceil(f1 * h))
            if what is None:
                val = 1.0
            elif what == "white":
                val = on_white[c]
            elif what == "black":
                val = on_black[c]
            else:
                val = what
            img[y0:y1, cols] = val
    return img
