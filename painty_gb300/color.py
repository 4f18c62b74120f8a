"""CIELab and CIEDE2000 colour differences, vectorised (the reporting side of the paint path).

painty's ColorConverter (painty/core/Color.hxx) converts linear RGB to XYZ with the sRGB D65
matrix (Color.hxx:186-198), XYZ to Lab with the D65 white (Color.hxx:49-51, 77-81), and
measures CIEDE2000 (Color.hxx:658-763; Sharma, Wu and Dalal 2005) with its own conventions:
the second colour's hue is 0 when its a' and b are both (near) zero, and hue difference and
mean hue fall back to 0 and h1 + h2 when the chroma product is (near) zero.
"""
from __future__ import annotations

import numpy as np

_RGB2XYZ = np.array([[0.4124564, 0.3575761, 0.1804375],
                     [0.2126729, 0.7151522, 0.0721750],
                     [0.0193339, 0.1191920, 0.9503041]])
_WHITE = np.array([0.95047, 1.0, 1.08883])


def linear_rgb_to_lab(rgb: np.ndarray) -> np.ndarray:
    """(..., 3) linear RGB -> (..., 3) CIELab (D65)."""
    rgb = np.asarray(rgb, dtype=np.float64)
    xyz = rgb @ _RGB2XYZ.T / _WHITE
    t0 = (6.0 / 29.0) ** 3
    f = np.where(xyz > t0, np.cbrt(xyz), (1.0 / 3.0) * (29.0 / 6.0) ** 2 * xyz + 4.0 / 29.0)
    L = 116.0 * f[..., 1] - 16.0
    a = 500.0 * (f[..., 0] - f[..., 1])
    b = 200.0 * (f[..., 1] - f[..., 2])
    return np.stack([L, a, b], axis=-1)


def ciede2000(lab1: np.ndarray, lab2: np.ndarray) -> np.ndarray:
    """CIEDE2000 between (..., 3) Lab arrays."""
    lab1 = np.asarray(lab1, dtype=np.float64)
    lab2 = np.asarray(lab2, dtype=np.float64)
    pi = np.pi
    eps = np.finfo(np.float64).eps * 1000.0
    L1, A1, B1 = lab1[..., 0], lab1[..., 1], lab1[..., 2]
    L2, A2, B2 = lab2[..., 0], lab2[..., 1], lab2[..., 2]
    C1 = np.sqrt(A1 * A1 + B1 * B1)
    C2 = np.sqrt(A2 * A2 + B2 * B2)
    Cm7 = ((C1 + C2) / 2.0) ** 7
    G = 0.5 * (1.0 - np.sqrt(Cm7 / (Cm7 + 25.0 ** 7)))
    a1 = (1.0 + G) * A1
    a2 = (1.0 + G) * A2
    Cp1 = np.sqrt(a1 * a1 + B1 * B1)
    Cp2 = np.sqrt(a2 * a2 + B2 * B2)
    Cprod = Cp1 * Cp2
    h1 = np.arctan2(B1, a1)
    h1 = np.where(h1 < 0, h1 + 2 * pi, h1)
    h2 = np.arctan2(B2, a2)
    h2 = np.where(h2 < 0, h2 + 2 * pi, h2)
    h2 = np.where(np.abs(np.abs(a2) + np.abs(B2)) < eps, 0.0, h2)
    dL = L2 - L1
    dC = Cp2 - Cp1
    dh = h2 - h1
    dh = np.where(dh > pi, dh - 2 * pi, dh)
    dh = np.where(dh < -pi, dh + 2 * pi, dh)
    dh = np.where(np.abs(Cprod) < eps, 0.0, dh)
    dH = 2.0 * np.sqrt(Cprod) * np.sin(dh / 2.0)
    Lp = (L1 + L2) / 2.0
    Cp = (Cp1 + Cp2) / 2.0
    hp = (h1 + h2) / 2.0
    hp = np.where(np.abs(h1 - h2) > pi, hp - pi, hp)
    hp = np.where(hp < 0, hp + 2 * pi, hp)
    hp = np.where(np.abs(Cprod) < eps, h1 + h2, hp)
    L50 = (Lp - 50.0) ** 2
    Sl = 1.0 + 0.015 * L50 / np.sqrt(20.0 + L50)
    Sc = 1.0 + 0.045 * Cp
    Tt = (1.0 - 0.17 * np.cos(hp - pi / 6.0) + 0.24 * np.cos(2.0 * hp)
          + 0.32 * np.cos(3.0 * hp + pi / 30.0) - 0.20 * np.cos(4.0 * hp - 63.0 * pi / 180.0))
    Sh = 1.0 + 0.015 * Cp * Tt
    dtheta = (30.0 * pi / 180.0) * np.exp(-(((180.0 / pi * hp - 275.0) / 25.0) ** 2))
    Cp7 = Cp ** 7
    Rc = 2.0 * np.sqrt(Cp7 / (Cp7 + 25.0 ** 7))
    RT = -np.sin(2.0 * dtheta) * Rc
    return np.sqrt((dL / Sl) ** 2 + (dC / Sc) ** 2 + (dH / Sh) ** 2 + RT * (dC / Sc) * (dH / Sh))


def delta_e(rgb_ref: np.ndarray, rgb: np.ndarray) -> np.ndarray:
    """Per-pixel CIEDE2000 between two (..., 3) linear-RGB reflectance images."""
    return ciede2000(linear_rgb_to_lab(rgb_ref), linear_rgb_to_lab(rgb))
