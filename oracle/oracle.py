"""Python binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, to check
results. It loads oracle/_build/liboracle.so (the double-precision restatement of painty's
paint path, oracle/painty_oracle.cpp) and, where they were built, oracle/_ref/libpainty_ref.so
(painty's own headers compiled against the repository's Eigen/OpenCV stand-ins) and
oracle/_ref/libglsl_ref.so (painty's GL compute shaders compiled as C++, oracle/glsl_ref.cpp)
and oracle/_ref/libtdict_ref.so (painty's TextureBrushDictionary.cxx, oracle/tdict_ref.cpp).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libpainty_ref.so"
GLSL_LIB = HERE / "_ref" / "libglsl_ref.so"
TDICT_LIB = HERE / "_ref" / "libtdict_ref.so"
# the reference checkout (only the reference-header build reads it)
REFERENCE_ROOT = Path(os.environ.get("PAINTY_REFERENCE_ROOT", "/root/reference"))

_P, _I32, _I64, _D = C.c_void_p, C.c_int32, C.c_int64, C.c_double


def build(ref: bool = False) -> None:
    """make -C oracle (and `make ref` when the reference checkout is present)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if ref and (REFERENCE_ROOT / "painty").is_dir():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REFERENCE_ROOT}"], check=True)


def _load(path: Path):
    if not path.exists():
        build(ref=path in (REF_LIB, GLSL_LIB, TDICT_LIB))
    return C.CDLL(str(path))


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class _Lib:
    def __init__(self, lib, pre: str):
        self.lib, self.pre = lib, pre

    def f(self, name, *args, res=None):
        fn = getattr(self.lib, f"{self.pre}_{name}")
        fn.argtypes = list(args)
        fn.restype = res
        return fn


class Oracle:
    """The restated oracle (prefix orc_)."""

    def __init__(self):
        self.lib = _load(LIB)
        L = _Lib(self.lib, "orc")
        self.coth = L.f("coth", _D, res=_D)
        self._cr = L.f("compute_reflectance", _P, _P, _P, _D, _P)
        self._km64 = L.f("km_fp64", _P, _P, _P, _D, _P, _P)
        self.catmull_rom_1d = L.f("catmull_rom_1d", _D, _D, _D, _D, _D, res=_D)
        self._spline = L.f("spline_catmull_rom", _P, _I32, _D, _P)
        self._interp = L.f("interpolate", _P, _I32, _I32, _D, _D, res=_D)
        self._compose = L.f("compose_layers", _I64, _I32, _P, _P, _P, _P, _P, _I32, _I32)
        self._compose32 = L.f("compose_layers_f32_soa", _I64, _I32, _P, _P, _P, _P, _P, _I32)
        self._compose32d = L.f("compose_layers_f32_soa_f64", _I64, _I32, _P, _P, _P, _P, _P, _I32)
        self._cc = L.f("canvas_create", _I32, _I32, res=_P)
        self._cd = L.f("canvas_destroy", _P)
        self._cp = L.f("canvas_plane", _P, _I32, res=_P)
        self._cdry = L.f("canvas_dry", _P)
        self._ccomp = L.f("canvas_compose", _P, _P)
        self._crender = L.f("canvas_render", _P, _P)
        self._bc = L.f("brush_create", _D, _P, _I32, _I32, res=_P)
        self._bd = L.f("brush_destroy", _P)
        self._bsr = L.f("brush_set_radius", _P, _D)
        self._brates = L.f("brush_set_rates", _P, _D, _D)
        self._bsnap = L.f("brush_set_snapshot", _P, _I32)
        self._bdip = L.f("brush_dip", _P, _P, _P)
        self._bupd = L.f("brush_update_snapshot", _P, _P)
        self._bimp = L.f("brush_imprint", _P, _P, _D, _D, _D)
        self._bstamps = L.f("brush_stamps", _P, _P, _P, _I64)
        self._bstroke = L.f("brush_paint_stroke", _P, _P, _P, _I32, _D, res=_I64)
        self._sstamps = L.f("stroke_stamps", _P, _I32, _D, _P, _I64, res=_I64)
        self._binfo = L.f("brush_info", _P, C.POINTER(_I32), C.POINTER(_I32), res=_D)
        self._bfp = L.f("brush_footprint", _P, res=_P)
        self._bpick = L.f("brush_pickup", _P, _I32, res=_P)
        self._bsnapget = L.f("brush_snapshot", _P, _I32, C.POINTER(_I32), C.POINTER(_I32), res=_P)
        self._mix = L.f("mix_single_paint", _P, _I32, _P, _P, _P, _P)
        self._lab = L.f("rgb2lab", _P, _P)
        self._de = L.f("ciede2000", _P, _P, res=_D)
        self._deimg = L.f("delta_e_images", _I64, _P, _P, C.POINTER(_D), _I32, res=_D)
        self._resample = L.f("resample", _P, _I32, _I32, _I32, _I32, _P)

    # -- math
    def compute_reflectance(self, K, S, R0, d):
        K, S, R0 = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S, R0))
        out = np.zeros(3)
        self._cr(_p(K), _p(S), _p(R0), float(d), _p(out))
        return out

    def km_fp64(self, K, S, R0, d):
        K, S, R0 = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S, R0))
        R, T = np.zeros(3), np.zeros(3)
        self._km64(_p(K), _p(S), _p(R0), float(d), _p(R), _p(T))
        return R, T

    def spline_catmull_rom(self, pts, u):
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        out = np.zeros(2)
        self._spline(_p(pts), len(pts), float(u), _p(out))
        return out

    def interpolate(self, img, x, y):
        img = np.ascontiguousarray(img, dtype=np.float64)
        return self._interp(_p(img), img.shape[0], img.shape[1], float(x), float(y))

    def resample(self, img, rows, cols):
        img = np.ascontiguousarray(img, dtype=np.float64)
        out = np.zeros((rows, cols))
        self._resample(_p(img), img.shape[0], img.shape[1], rows, cols, _p(out))
        return out

    def compose_layers(self, K, S, V, R0, mode: int = 0, threads: int = 1):
        """K, S: (L, npix, 3); V: (L, npix); R0: (npix, 3) -> (npix, 3). mode 1 = FP64 oracle."""
        K, S, V, R0 = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S, V, R0))
        L, npix = V.shape
        out = np.zeros((npix, 3))
        self._compose(npix, L, _p(K), _p(S), _p(V), _p(R0), _p(out), mode, threads)
        return out

    def compose_layers_f32_planar(self, K, S, V, R0, threads: int = 1):
        """The reference composite over float32 planar stacks (timed CPU baseline)."""
        L = V.shape[0]
        npix = V[0].size
        out = np.empty((3,) + V.shape[1:], dtype=np.float32)
        self._compose32(npix, L, _p(K), _p(S), _p(V), _p(R0), _p(out), threads)
        return out

    def compose_layers_f32_planar_f64(self, K, S, V, R0, threads: int = 1):
        """The reference composite over float32 planar stacks K, S (L, 3, rows, cols),
        V (L, rows, cols), R0 (3, rows, cols), kept in double: (rows, cols, 3)."""
        K, S, V, R0 = (np.ascontiguousarray(x, dtype=np.float32) for x in (K, S, V, R0))
        L = V.shape[0]
        npix = V[0].size
        out = np.empty(V.shape[1:] + (3,), dtype=np.float64)
        self._compose32d(npix, L, _p(K), _p(S), _p(V), _p(R0), _p(out), threads)
        return out

    def mix_single_paint(self, w, K, S):
        w, K, S = (np.ascontiguousarray(x, dtype=np.float64) for x in (w, K, S))
        k, s = np.zeros(3), np.zeros(3)
        self._mix(_p(w), len(w), _p(K), _p(S), _p(k), _p(s))
        return k, s

    def rgb2lab(self, rgb):
        rgb = np.ascontiguousarray(rgb, dtype=np.float64)
        out = np.zeros(3)
        self._lab(_p(rgb), _p(out))
        return out

    def ciede2000(self, a, b):
        a, b = (np.ascontiguousarray(x, dtype=np.float64) for x in (a, b))
        return self._de(_p(a), _p(b))

    def delta_e(self, rgb_a, rgb_b, threads: int = 8):
        """(max, mean) CIEDE2000 between two linear-RGB images (..., 3)."""
        a = np.ascontiguousarray(rgb_a, dtype=np.float64).reshape(-1, 3)
        b = np.ascontiguousarray(rgb_b, dtype=np.float64).reshape(-1, 3)
        mean = _D()
        mx = self._deimg(a.shape[0], _p(a), _p(b), C.byref(mean), threads)
        return mx, mean.value

    def stroke_stamps(self, path, spacing):
        path = np.ascontiguousarray(path, dtype=np.float64)
        n = self._sstamps(_p(path), len(path), float(spacing), None, 0)
        out = np.zeros((max(n, 1), 3))
        self._sstamps(_p(path), len(path), float(spacing), _p(out), n)
        return out[:n]

    # -- objects
    def canvas(self, rows, cols):
        return OCanvas(self, rows, cols)

    def brush(self, radius, footprint):
        return OBrush(self, radius, footprint)

    # -- the GL canvas path (float; K4 / S4 / R4: (rows, cols, 4) float32)
    def glsl_compose(self, K4, S4, R4):
        """CanvasGpu::getComposed: ComposeLayerOnSubstrate over a copy of R0."""
        K4, S4, R4 = (np.ascontiguousarray(x, dtype=np.float32) for x in (K4, S4, R4))
        out = np.empty_like(R4)
        f = _Lib(self.lib, "orc").f("glsl_compose", _I64, _P, _P, _P, _P)
        f(K4.size // 4, _p(K4), _p(S4), _p(R4), _p(out))
        return out

    def glsl_dry_step(self, K4, S4, R4, portion):
        """CanvasGpu::dryStep on copies; returns (K4, R4)."""
        K4, R4 = (np.array(x, dtype=np.float32, order="C") for x in (K4, R4))
        S4 = np.ascontiguousarray(S4, dtype=np.float32)
        f = _Lib(self.lib, "orc").f("glsl_dry_step", _I64, _P, _P, _P, C.c_float)
        f(K4.size // 4, _p(K4), _p(S4), _p(R4), float(portion))
        return K4, R4

    def glsl_imprint(self, warped, K4, S4, x0, y0, aoi_w, aoi_h, Kb, Sb, scale):
        """TextureBrushGpu's imprint pass on copies of K4 / S4; returns (K4, S4)."""
        return _glsl_imprint(_Lib(self.lib, "orc"), "glsl_imprint", warped, K4, S4, x0, y0,
                             aoi_w, aoi_h, Kb, Sb, scale)

    def glsl_clear(self, warped, x0, y0, aoi_w, aoi_h):
        """TextureBrushGpu's clear pass on a copy of the warped texture."""
        return _glsl_clear(_Lib(self.lib, "orc"), "glsl_clear", warped, x0, y0, aoi_w, aoi_h)

    def gl_strip_vertices(self, path, radius):
        """TextureBrushGpu's triangle strip: ((2n, 2) float32 vertices, (2n, 2) texcoords)."""
        return _strip(_Lib(self.lib, "orc"), path, radius)

    def texture_dictionary(self, seed: int):
        return _TDict(self.lib, seed)

    def gpu_texture_brush(self):
        return _GTBrush(self.lib)

    def texture_brush(self, texture):
        return _TBrush(self.lib, "orc", texture)


class _TBrush:
    """TextureBrush<vec3> with the given thickness texture (orc_ or ref_ prefix)."""

    def __init__(self, lib, pre: str, texture):
        L = _Lib(lib, pre)
        self._create = L.f("tbrush_create", _P, _I32, _I32, res=_P)
        self._destroy = L.f("tbrush_destroy", _P)
        self._radius = L.f("tbrush_set_radius", _P, _D)
        self._dip = L.f("tbrush_dip", _P, _P, _P)
        self._smudge = L.f("tbrush_set_smudge", _P, _I32)
        self._scale = L.f("tbrush_set_thickness_scale", _P, _D)
        self._stroke = L.f("tbrush_paint_stroke", _P, _P, _P, _I32,
                           res=_I64 if pre == "orc" else None)
        self.pre = pre
        if pre == "orc":
            self._map = L.f("tbrush_smudge_map", _P, _I32, C.POINTER(_I32), res=_P)
        tex = np.ascontiguousarray(texture, dtype=np.float64)
        self.h = self._create(_p(tex), tex.shape[0], tex.shape[1])

    def __del__(self):
        if getattr(self, "h", None):
            self._destroy(self.h)
            self.h = None

    def set_radius(self, r):
        self._radius(self.h, float(r))

    def dip(self, K, S):
        K, S = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S))
        self._dip(self.h, _p(K), _p(S))

    def enable_smudge(self, on: bool):
        self._smudge(self.h, 1 if on else 0)

    def set_thickness_scale(self, s):
        self._scale(self.h, float(s))

    def paint_stroke(self, canvas, path):
        path = np.ascontiguousarray(path, dtype=np.float64)
        return self._stroke(self.h, canvas.h, _p(path), len(path))

    def smudge_map(self, which: str):
        side = _I32()
        idx = {"K": 0, "S": 1, "V": 2}[which]
        ptr = self._map(self.h, idx, C.byref(side))
        n = side.value
        if n == 0:
            return np.zeros((0, 0) if which == "V" else (0, 0, 3))
        a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(_D)), (n * n * (1 if which == "V" else 3),))
        return a.reshape((n, n) if which == "V" else (n, n, 3)).copy()


class _TDict:
    """TextureBrushDictionary with a seeded pick (orc_tdict)."""

    def __init__(self, lib, seed: int):
        L = _Lib(lib, "orc")
        self._lib = lib
        self._destroy = L.f("tdict_destroy", _P)
        self._add = L.f("tdict_add", _P, C.c_uint32, C.c_uint32, _P, _I32, _I32, res=_I32)
        self._lookup = L.f("tdict_lookup", _P, _P, _I32, _D, res=_I32)
        self.h = L.f("tdict_create", C.c_uint32, res=_P)(seed)

    def __del__(self):
        if getattr(self, "h", None):
            self._destroy(self.h)
            self.h = None

    def add(self, radius_class, length_class, height):
        h = np.ascontiguousarray(height, dtype=np.float64)
        return self._add(self.h, radius_class, length_class, _p(h), h.shape[0], h.shape[1])

    def lookup(self, path, brush_size):
        p = np.ascontiguousarray(path, dtype=np.float64)
        return self._lookup(self.h, _p(p), len(p), float(brush_size))

    def texture(self, index):
        """Entry `index`'s GL texture (float32, GL row order)."""
        f = _Lib(self._lib, "orc").f("tdict_texture", _P, _I32, C.POINTER(_I32),
                                     C.POINTER(_I32), _P, res=_I32)
        rows, cols = _I32(0), _I32(0)
        if f(self.h, int(index), C.byref(rows), C.byref(cols), None) != 0:
            raise IndexError(index)
        out = np.empty((rows.value, cols.value), np.float32)
        f(self.h, int(index), C.byref(rows), C.byref(cols), _p(out))
        return out


class _GTBrush:
    """TextureBrushGpu, smudge off (orc_gtbrush); paints float K4 / S4 arrays in place."""

    def __init__(self, lib):
        L = _Lib(lib, "orc")
        self._destroy = L.f("gtbrush_destroy", _P)
        self._radius = L.f("gtbrush_set_radius", _P, _D)
        self._dip = L.f("gtbrush_dip", _P, _P, _P)
        self._scale = L.f("gtbrush_set_thickness_scale", _P, _D)
        self._last = L.f("gtbrush_last_texture", _P, res=_I32)
        self._warped = L.f("gtbrush_warped", _P, res=_P)
        self._stroke = L.f("gtbrush_paint_stroke", _P, _P, _I32, _I32, _P, _P, _P, _I32,
                           res=_I32)
        self.h = L.f("gtbrush_create", res=_P)()

    def __del__(self):
        if getattr(self, "h", None):
            self._destroy(self.h)
            self.h = None

    def set_radius(self, r):
        self._radius(self.h, float(r))

    def dip(self, K, S):
        K, S = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S))
        self._dip(self.h, _p(K), _p(S))

    def set_thickness_scale(self, s):
        self._scale(self.h, float(s))

    def last_texture(self):
        return self._last(self.h)

    def paint_stroke(self, dictionary, K4, S4, path):
        """K4, S4: C-contiguous float32 (rows, cols, 4), painted in place."""
        assert K4.dtype == np.float32 and K4.flags.c_contiguous and S4.flags.c_contiguous
        p = np.ascontiguousarray(path, dtype=np.float64)
        return self._stroke(self.h, dictionary.h, K4.shape[0], K4.shape[1], _p(K4), _p(S4),
                            _p(p), len(p))


class OCanvas:
    def __init__(self, o: Oracle, rows: int, cols: int):
        self.o, self.rows, self.cols = o, rows, cols
        self.h = o._cc(rows, cols)

    def __del__(self):
        if getattr(self, "h", None):
            self.o._cd(self.h)
            self.h = None

    def plane(self, which: str) -> np.ndarray:
        idx = {"K": 0, "S": 1, "V": 2, "R0": 3, "h": 4}[which]
        n = self.rows * self.cols * (1 if which in ("V", "h") else 3)
        arr = np.ctypeslib.as_array(C.cast(self.o._cp(self.h, idx), C.POINTER(_D)), (n,))
        return arr.reshape((self.rows, self.cols) if which in ("V", "h") else
                           (self.rows, self.cols, 3))

    def set(self, which: str, data) -> None:
        self.plane(which)[...] = data

    def get(self, which: str) -> np.ndarray:
        return self.plane(which).copy()

    def dry(self) -> None:
        self.o._cdry(self.h)

    def compose(self) -> np.ndarray:
        out = np.zeros((self.rows, self.cols, 3))
        self.o._ccomp(self.h, _p(out))
        return out

    def render(self) -> np.ndarray:
        """Renderer::render: the lit canvas (rows, cols, 3)."""
        out = np.zeros((self.rows, self.cols, 3))
        self.o._crender(self.h, _p(out))
        return out


class OBrush:
    def __init__(self, o: Oracle, radius: float, footprint: np.ndarray):
        self.o = o
        fp = np.ascontiguousarray(footprint, dtype=np.float64)
        self.h = o._bc(float(radius), _p(fp), fp.shape[0], fp.shape[1])

    def __del__(self):
        if getattr(self, "h", None):
            self.o._bd(self.h)
            self.h = None

    def set_radius(self, r):
        self.o._bsr(self.h, float(r))

    def set_rates(self, pickup, deposition):
        self.o._brates(self.h, float(pickup), float(deposition))

    def set_snapshot(self, use: bool):
        self.o._bsnap(self.h, 1 if use else 0)

    def dip(self, K, S):
        K, S = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S))
        self.o._bdip(self.h, _p(K), _p(S))

    def update_snapshot(self, canvas: OCanvas):
        self.o._bupd(self.h, canvas.h)

    def imprint(self, canvas: OCanvas, cx, cy, theta):
        self.o._bimp(self.h, canvas.h, float(cx), float(cy), float(theta))

    def stamps(self, canvas: OCanvas, s):
        s = np.ascontiguousarray(s, dtype=np.float64).reshape(-1, 3)
        self.o._bstamps(self.h, canvas.h, _p(s), s.shape[0])

    def paint_stroke(self, canvas: OCanvas, path, spacing=1.0) -> int:
        path = np.ascontiguousarray(path, dtype=np.float64)
        return self.o._bstroke(self.h, canvas.h, _p(path), len(path), float(spacing))

    def info(self):
        F, S = _I32(), _I32()
        r = self.o._binfo(self.h, C.byref(F), C.byref(S))
        return r, F.value, S.value

    def footprint(self):
        _, F, _ = self.info()
        return np.ctypeslib.as_array(C.cast(self.o._bfp(self.h), C.POINTER(_D)), (F, F)).copy()

    def pickup(self, which: str):
        _, _, S = self.info()
        idx = {"K": 0, "S": 1, "V": 2}[which]
        n = S * S * (1 if which == "V" else 3)
        a = np.ctypeslib.as_array(C.cast(self.o._bpick(self.h, idx), C.POINTER(_D)), (n,))
        return a.reshape((S, S) if which == "V" else (S, S, 3)).copy()

    def snapshot(self, which: str):
        """The brush's snapshot buffer (FootprintBrush::_snapshotBuffer) plane K, S or V;
        None before the brush's first snapshot."""
        idx = {"K": 0, "S": 1, "V": 2}[which]
        rows, cols = _I32(0), _I32(0)
        ptr = self.o._bsnapget(self.h, idx, C.byref(rows), C.byref(cols))
        if not ptr or rows.value * cols.value == 0:
            return None
        n = rows.value * cols.value * (1 if which == "V" else 3)
        a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(_D)), (n,))
        shape = (rows.value, cols.value) if which == "V" else (rows.value, cols.value, 3)
        return a.reshape(shape).copy()


def _strip(L, path, radius):
    p = np.ascontiguousarray(path, dtype=np.float64)
    n = len(p)
    xy, uv = np.empty((2 * n, 2), np.float32), np.empty((2 * n, 2), np.float32)
    L.f("gl_strip_vertices", _P, _I32, _D, _P, _P)(_p(p), n, float(radius), _p(xy), _p(uv))
    return xy, uv


def _glsl_imprint(L, name, warped, K4, S4, x0, y0, aoi_w, aoi_h, Kb, Sb, scale):
    warped = np.ascontiguousarray(warped, dtype=np.float32)
    K4, S4 = (np.array(x, dtype=np.float32, order="C") for x in (K4, S4))
    Kb, Sb = (np.ascontiguousarray(x, dtype=np.float32) for x in (Kb, Sb))
    rows, cols = warped.shape
    f = L.f(name, _I32, _I32, _P, _P, _P, _I32, _I32, _I32, _I32, _P, _P, C.c_float)
    f(rows, cols, _p(warped), _p(K4), _p(S4), int(x0), int(y0), int(aoi_w), int(aoi_h), _p(Kb),
      _p(Sb), float(scale))
    return K4, S4


def _glsl_clear(L, name, warped, x0, y0, aoi_w, aoi_h):
    warped = np.array(warped, dtype=np.float32, order="C")
    rows, cols = warped.shape
    f = L.f(name, _I32, _I32, _P, _I32, _I32, _I32, _I32)
    f(rows, cols, _p(warped), int(x0), int(y0), int(aoi_w), int(aoi_h))
    return warped


class GlslReference:
    """painty's GL compute shaders compiled as C++ (oracle/glsl_ref.cpp, prefix glref_):
    the reference the GL-path restatement is pinned to. Arrays are (rows, cols, 4) float32
    (K4 / S4 / R4) or (rows, cols) float32 (the warped brush texture)."""

    def __init__(self):
        self.L = _Lib(_load(GLSL_LIB), "glref")

    @staticmethod
    def available() -> bool:
        if GLSL_LIB.exists():
            return True
        if not (REFERENCE_ROOT / "painty").is_dir():
            return False
        try:
            build(ref=True)
        except Exception:
            return False
        return GLSL_LIB.exists()

    def compose(self, K4, S4, R4):
        """ComposeLayerOnSubstrate over a copy of R4."""
        K4, S4 = (np.ascontiguousarray(x, dtype=np.float32) for x in (K4, S4))
        out = np.array(R4, dtype=np.float32, order="C")
        rows, cols = out.shape[:2]
        self.L.f("compose", _I32, _I32, _P, _P, _P)(rows, cols, _p(K4), _p(S4), _p(out))
        return out

    def dry_step(self, K4, S4, R4, portion):
        """DryingStep on copies; returns (K4, R4)."""
        K4, S4, R4 = (np.array(x, dtype=np.float32, order="C") for x in (K4, S4, R4))
        rows, cols = K4.shape[:2]
        self.L.f("dry_step", _I32, _I32, _P, _P, _P, C.c_float)(
            rows, cols, _p(K4), _p(S4), _p(R4), float(portion))
        return K4, R4

    def imprint(self, warped, K4, S4, x0, y0, aoi_w, aoi_h, Kb, Sb, scale):
        """PaintTextureFootprintOnCanvas on copies of K4 / S4; returns (K4, S4)."""
        return _glsl_imprint(self.L, "imprint", warped, K4, S4, x0, y0, aoi_w, aoi_h, Kb, Sb,
                             scale)

    def clear(self, warped, x0, y0, aoi_w, aoi_h):
        """ClearTextureFootprint on a copy of the warped texture."""
        return _glsl_clear(self.L, "clear", warped, x0, y0, aoi_w, aoi_h)


class TDictReference:
    """painty's own TextureBrushDictionary.cxx (oracle/tdict_ref.cpp, prefix tref_). `build`
    writes empty files <radius>_<length>_<k>.tex into root/data/textures, registers each one's
    height map for painty's imRead and lets painty's constructor scan the folder."""

    def __init__(self):
        self.L = _Lib(_load(TDICT_LIB), "tref")
        self.h = None

    @staticmethod
    def available() -> bool:
        if TDICT_LIB.exists():
            return True
        if not (REFERENCE_ROOT / "painty").is_dir():
            return False
        try:
            build(ref=True)
        except Exception:
            return False
        return TDICT_LIB.exists()

    def build(self, root: Path, entries):
        """entries: (radius_class, length_class, height map) in insertion order. Returns the
        relative path painty reads for each entry."""
        folder = Path(root) / "data" / "textures"
        folder.mkdir(parents=True, exist_ok=True)
        self.L.f("clear_registry")()
        reg = self.L.f("register", C.c_char_p, _P, _I32, _I32)
        names = []
        for k, (rc, lc, tex) in enumerate(entries):
            rel = f"data/textures/{int(rc)}_{int(lc)}_{k}.tex"
            (Path(root) / rel).write_bytes(b"")
            h = np.ascontiguousarray(tex, dtype=np.float64)
            reg(rel.encode(), _p(h), h.shape[0], h.shape[1])
            names.append(rel)
        self.h = self.L.f("create", C.c_char_p, res=_P)(str(root).encode())
        if not self.h:
            raise RuntimeError("painty's TextureBrushDictionary could not be built")
        return names

    def __del__(self):
        if getattr(self, "h", None):
            self.L.f("destroy", _P)(self.h)
            self.h = None

    def lookup(self, path, brush_size):
        """(source path, GL texture) of painty's pick."""
        p = np.ascontiguousarray(path, dtype=np.float64)
        f = self.L.f("lookup", _P, _P, _I32, _D, C.c_char_p, _I32, C.POINTER(_I32),
                     C.POINTER(_I32), _P, res=_I32)
        src = C.create_string_buffer(512)
        rows, cols = _I32(0), _I32(0)
        buf = np.empty(1 << 20, np.float32)
        if f(self.h, _p(p), len(p), float(brush_size), src, 512, C.byref(rows), C.byref(cols),
             _p(buf)) != 0:
            raise RuntimeError("painty's lookup threw")
        return src.value.decode(), buf[:rows.value * cols.value].reshape(rows.value, cols.value)


class Reference:
    """painty's own headers compiled against the stand-ins (prefix ref_); None if unbuilt."""

    def __init__(self):
        self.lib = _load(REF_LIB)
        L = _Lib(self.lib, "ref")
        self.coth = L.f("coth", _D, res=_D)
        self._cr = L.f("compute_reflectance", _P, _P, _P, _D, _P)
        self.catmull_rom_1d = L.f("catmull_rom_1d", _D, _D, _D, _D, _D, res=_D)
        self._spline = L.f("spline_catmull_rom", _P, _I32, _D, _P)
        self._interp = L.f("interpolate", _P, _I32, _I32, _D, _D, res=_D)
        self._lab = L.f("rgb2lab", _P, _P)
        self._de = L.f("ciede2000", _P, _P, res=_D)
        self._cc = L.f("canvas_create", _I32, _I32, res=_P)
        self._cd = L.f("canvas_destroy", _P)
        self._cget = L.f("canvas_get", _P, _I32, _P)
        self._cset = L.f("canvas_set", _P, _I32, _P)
        self._cdry = L.f("canvas_dry", _P)
        self._ccomp = L.f("canvas_compose", _P, _P)
        self._crender = L.f("canvas_render", _P, _P)
        self._bc = L.f("brush_create", _D, _P, _I32, _I32, res=_P)
        self._bd = L.f("brush_destroy", _P)
        self._bsr = L.f("brush_set_radius", _P, _D)
        self._brates = L.f("brush_set_rates", _P, _D, _D)
        self._bsnap = L.f("brush_set_snapshot", _P, _I32)
        self._bdip = L.f("brush_dip", _P, _P, _P)
        self._bupd = L.f("brush_update_snapshot", _P, _P)
        self._bimp = L.f("brush_imprint", _P, _P, _D, _D, _D)
        self._bstamps = L.f("brush_stamps", _P, _P, _P, _I64)
        self._bstroke = L.f("brush_paint_stroke", _P, _P, _P, _I32, res=_I64)
        self._binfo = L.f("brush_info", _P, C.POINTER(_I32), C.POINTER(_I32))
        self._bfp = L.f("brush_footprint", _P, _P)
        self._bpick = L.f("brush_pickup", _P, _I32, _P)

    @staticmethod
    def available() -> bool:
        if REF_LIB.exists():
            return True
        if not (REFERENCE_ROOT / "painty").is_dir():
            return False
        try:
            build(ref=True)
        except Exception:
            return False
        return REF_LIB.exists()

    def load_palette(self, text: str):
        """painty's LoadPalette of a JSON text: [(K, S)] as float64 arrays."""
        f = _Lib(self.lib, "ref").f("load_palette", C.c_char_p, _P, _P, _I32, res=_I32)
        cap = 4096
        K, S = np.zeros((cap, 3)), np.zeros((cap, 3))
        n = f(text.encode(), _p(K), _p(S), cap)
        if n < 0:
            raise ValueError("painty's LoadPalette threw")
        return [(K[i].copy(), S[i].copy()) for i in range(min(n, cap))]

    def visualize_palette(self, palette, thickness):
        """painty's VisualizePalette: (200, 100 n, 3) float64 sRGB."""
        n = len(palette)
        K = np.ascontiguousarray([k for k, _ in palette], dtype=np.float64).reshape(n, 3)
        S = np.ascontiguousarray([s for _, s in palette], dtype=np.float64).reshape(n, 3)
        out = np.zeros((200, 100 * n, 3))
        f = _Lib(self.lib, "ref").f("visualize_palette", _P, _P, _I32, _D, _P)
        f(_p(K), _p(S), n, float(thickness), _p(out))
        return out

    def mix_single_paint(self, weights, K, S):
        """painty's own PaintMixer::mixSinglePaint over the palette (K, S: n x 3)."""
        w = np.ascontiguousarray(weights, dtype=np.float64)
        K, S = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S))
        ok, os_ = np.zeros(3), np.zeros(3)
        f = _Lib(self.lib, "ref").f("mix_single_paint", _P, _I32, _P, _P, _P, _P, res=_I32)
        if f(_p(w), len(w), _p(K), _p(S), _p(ok), _p(os_)) != 0:
            raise ValueError("painty's mixSinglePaint threw")
        return ok, os_

    def gl_strip_vertices(self, path, radius):
        """TextureBrushGpu's triangle strip over painty's SplineEval."""
        return _strip(_Lib(self.lib, "ref"), path, radius)

    def compute_reflectance(self, K, S, R0, d):
        K, S, R0 = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S, R0))
        out = np.zeros(3)
        self._cr(_p(K), _p(S), _p(R0), float(d), _p(out))
        return out

    def spline_catmull_rom(self, pts, u):
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        out = np.zeros(2)
        self._spline(_p(pts), len(pts), float(u), _p(out))
        return out

    def interpolate(self, img, x, y):
        img = np.ascontiguousarray(img, dtype=np.float64)
        return self._interp(_p(img), img.shape[0], img.shape[1], float(x), float(y))

    def rgb2lab(self, rgb):
        rgb = np.ascontiguousarray(rgb, dtype=np.float64)
        out = np.zeros(3)
        self._lab(_p(rgb), _p(out))
        return out

    def ciede2000(self, a, b):
        a, b = (np.ascontiguousarray(x, dtype=np.float64) for x in (a, b))
        return self._de(_p(a), _p(b))

    def canvas(self, rows, cols):
        return RCanvas(self, rows, cols)

    def brush(self, radius, footprint):
        return RBrush(self, radius, footprint)

    def texture_brush(self, texture):
        return _TBrush(self.lib, "ref", texture)


class RCanvas:
    def __init__(self, r: Reference, rows: int, cols: int):
        self.r, self.rows, self.cols = r, rows, cols
        self.h = r._cc(rows, cols)

    def __del__(self):
        if getattr(self, "h", None):
            self.r._cd(self.h)
            self.h = None

    def get(self, which: str) -> np.ndarray:
        idx = {"K": 0, "S": 1, "V": 2, "R0": 3, "h": 4}[which]
        one = which in ("V", "h")
        out = np.zeros((self.rows, self.cols) if one else (self.rows, self.cols, 3))
        self.r._cget(self.h, idx, _p(out))
        return out

    def set(self, which: str, data) -> None:
        idx = {"K": 0, "S": 1, "V": 2, "R0": 3, "h": 4}[which]
        d = np.ascontiguousarray(data, dtype=np.float64)
        self.r._cset(self.h, idx, _p(d))

    def dry(self):
        self.r._cdry(self.h)

    def compose(self):
        out = np.zeros((self.rows, self.cols, 3))
        self.r._ccomp(self.h, _p(out))
        return out

    def render(self):
        out = np.zeros((self.rows, self.cols, 3))
        self.r._crender(self.h, _p(out))
        return out


class RBrush:
    def __init__(self, r: Reference, radius: float, footprint: np.ndarray):
        self.r = r
        fp = np.ascontiguousarray(footprint, dtype=np.float64)
        self.h = r._bc(float(radius), _p(fp), fp.shape[0], fp.shape[1])

    def __del__(self):
        if getattr(self, "h", None):
            self.r._bd(self.h)
            self.h = None

    def set_radius(self, v):
        self.r._bsr(self.h, float(v))

    def set_rates(self, p, d):
        self.r._brates(self.h, float(p), float(d))

    def set_snapshot(self, use):
        self.r._bsnap(self.h, 1 if use else 0)

    def dip(self, K, S):
        K, S = (np.ascontiguousarray(x, dtype=np.float64) for x in (K, S))
        self.r._bdip(self.h, _p(K), _p(S))

    def update_snapshot(self, canvas):
        self.r._bupd(self.h, canvas.h)

    def imprint(self, canvas, cx, cy, theta):
        self.r._bimp(self.h, canvas.h, float(cx), float(cy), float(theta))

    def stamps(self, canvas, s):
        s = np.ascontiguousarray(s, dtype=np.float64).reshape(-1, 3)
        self.r._bstamps(self.h, canvas.h, _p(s), s.shape[0])

    def paint_stroke(self, canvas, path) -> int:
        path = np.ascontiguousarray(path, dtype=np.float64)
        return self.r._bstroke(self.h, canvas.h, _p(path), len(path))

    def info(self):
        F, S = _I32(), _I32()
        self.r._binfo(self.h, C.byref(F), C.byref(S))
        return F.value, S.value

    def footprint(self):
        F, _ = self.info()
        out = np.zeros((F, F))
        self.r._bfp(self.h, _p(out))
        return out

    def pickup(self, which):
        _, S = self.info()
        idx = {"K": 0, "S": 1, "V": 2}[which]
        out = np.zeros((S, S) if which == "V" else (S, S, 3))
        self.r._bpick(self.h, idx, _p(out))
        return out
