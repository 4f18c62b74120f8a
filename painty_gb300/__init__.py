"""painty_gb300 -- GB300-native Kubelka-Munk paint path (Python host mirror of the C ABI).

Mirrors lindemeier/painty's renderer classes over the C ABI in include/painty_gb300.h:

    Canvas          painty/renderer/Canvas.hxx        (wet layer, substrate R0, height map)
    PaintLayer      painty/renderer/PaintLayer.hxx    (K, S, V planes)
    Image           Mat<vec3> reflectance on the device (R0 / composite output)
    FootprintBrush  painty/renderer/FootprintBrush.hxx
    Renderer        painty/renderer/Renderer.hxx      (compose)
    mix_single_paint painty/mixer/src/PaintMixer.cxx:327-355

Errors map to painty's exception types: invalid arguments raise ValueError (painty throws
std::invalid_argument), CUDA failures raise RuntimeError, allocation failures MemoryError.

The compiled library is required: importing this package without it raises ImportError.
There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
# PAINTY_BOUNDS_CHECK=1 loads the bounds-checked build of the library (the stamp kernels test
# every computed index before the access and raise instead of faulting)
BOUNDS_CHECKED = os.environ.get("PAINTY_BOUNDS_CHECK", "") not in ("", "0")
# PAINTY_PHASE_TIMERS=1 loads the phase-timing build (per-phase clock counters of the stamp
# loop, read with take_phase_cycles)
PHASE_TIMERS = os.environ.get("PAINTY_PHASE_TIMERS", "") not in ("", "0")
LIB_PATH = _HERE / "_lib" / ("libpainty_gb300_checked.so" if BOUNDS_CHECKED
                             else "libpainty_gb300_phases.so" if PHASE_TIMERS
                             else "libpainty_gb300.so")

if not LIB_PATH.exists():
    raise ImportError(
        f"painty_gb300 native library not found at {LIB_PATH}; build it with "
        "`python painty_gb300/build.py` (CUDA toolkit required; there is no CPU fallback)")

_lib = C.CDLL(str(LIB_PATH))

STORAGE = {"f32": 0, "f16": 1, "bf16": 2, "f64": 3}
HOST_F64_INTERLEAVED, HOST_F32_INTERLEAVED, HOST_F64_PLANAR, HOST_F32_PLANAR = 0, 1, 2, 3
PLANE = {"K": 0, "S": 1, "V": 2, "R0": 3, "h": 4, "VL": 5}

_P, _I32, _I64, _D = C.c_void_p, C.c_int32, C.c_int64, C.c_double


def _sig(name, *args, res=C.c_int):
    f = getattr(_lib, name)
    f.argtypes = list(args)
    f.restype = res
    return f


_sig("painty_abi_version", res=_I32)
_sig("painty_build_flags", res=_I32)
_sig("painty_status_string", C.c_int, res=C.c_char_p)
_sig("painty_last_error", res=C.c_char_p)
_sig("painty_kernel_launch_count", res=_I64)
_sig("painty_take_device_faults", C.POINTER(C.c_uint32))
_sig("painty_take_phase_cycles", C.POINTER(C.c_uint64))
_sig("painty_layer_create", _I32, _I32, C.c_int, C.POINTER(_P))
_sig("painty_layer_destroy", _P)
_sig("painty_layer_clear", _P, _P)
_sig("painty_layer_upload", _P, C.c_int, _P, C.c_int, _P)
_sig("painty_layer_download", _P, C.c_int, _P, C.c_int, _P)
_sig("painty_layer_copy", _P, _P, _P)
_sig("painty_layer_set_cells", _P, _I64, _P, _P, _P, _P, _P)
_sig("painty_layer_info", _P, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(C.c_int))
_sig("painty_image_create", _I32, _I32, C.c_int, C.POINTER(_P))
_sig("painty_image_destroy", _P)
_sig("painty_image_fill", _P, _D, _D, _D, _P)
_sig("painty_image_upload", _P, _P, C.c_int, _P)
_sig("painty_image_download", _P, _P, C.c_int, _P)
_sig("painty_compose_layers", _P, _I32, _P, _P, _P)
_sig("painty_compose_layers_unfused", _P, _I32, _P, _P, _P)
_sig("painty_compose_layers_host", _P, _P, _P, _I32, _P, _P, _I32, _I32, _P)
_sig("painty_canvas_create", _I32, _I32, C.c_int, C.POINTER(_P))
_sig("painty_canvas_destroy", _P)
_sig("painty_canvas_clear", _P, _P)
_sig("painty_canvas_upload", _P, C.c_int, _P, C.c_int, _P)
_sig("painty_canvas_download", _P, C.c_int, _P, C.c_int, _P)
_sig("painty_canvas_layer", _P, C.POINTER(_P))
_sig("painty_canvas_r0", _P, C.POINTER(_P))
_sig("painty_canvas_info", _P, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(C.c_int))
_sig("painty_canvas_compose", _P, _P, _P)
_sig("painty_canvas_dry", _P, _P)
_sig("painty_brush_create", _D, _P, _I32, _I32, C.POINTER(_P))
_sig("painty_brush_destroy", _P)
_sig("painty_brush_set_radius", _P, _D)
_sig("painty_brush_set_rates", _P, _D, _D)
_sig("painty_brush_get_rates", _P, C.POINTER(_D), C.POINTER(_D))
_sig("painty_brush_set_snapshot", _P, _I32)
_sig("painty_brush_dip", _P, _P, _P, _P)
_sig("painty_brush_update_snapshot", _P, _P, _P)
_sig("painty_brush_info", _P, C.POINTER(_D), C.POINTER(_I32), C.POINTER(_I32))
_sig("painty_brush_footprint", _P, _P)
_sig("painty_brush_download_pickup", _P, C.c_int, _P, C.c_int, _P)
_sig("painty_imprint", _P, _P, _D, _D, _D, _P)
_sig("painty_stamps", _P, _P, _P, _I64, _P)
_sig("painty_stroke", _P, _P, _P, _I32, _D, C.POINTER(_I64), _P)
_sig("painty_mix_paint", _P, _I32, _P, _P, _P, _P)
_sig("painty_paint_batch", _P, _P, _I32, _P, _I64, _P, _I64, C.POINTER(_I64), _P)
_sig("painty_batch_last_shape", C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32))
_sig("painty_batch_last_split", C.POINTER(_I32), C.POINTER(_I32))
_sig("painty_texture_brush_create", _P, _I32, _I32, C.POINTER(_P))
_sig("painty_texture_brush_destroy", _P)
_sig("painty_texture_brush_set_radius", _P, _D)
_sig("painty_texture_brush_dip", _P, _P, _P)
_sig("painty_texture_brush_set_smudge", _P, _I32)
_sig("painty_texture_brush_set_thickness_scale", _P, _D)
_sig("painty_texture_brush_paint_stroke", _P, _P, _P, _I32, C.POINTER(_I64), _P)
_sig("painty_texture_brush_smudge_map", _P, C.c_int, _P, C.POINTER(_I32), _P)
_sig("painty_canvas_compose_glsl", _P, _P, _P)
_sig("painty_canvas_render", _P, _P, _P)
_sig("painty_canvas_dry_step", _P, C.c_float, _P)
_sig("painty_texture_dictionary_create", C.c_uint32, C.POINTER(_P))
_sig("painty_texture_dictionary_destroy", _P)
_sig("painty_texture_dictionary_add", _P, C.c_uint32, C.c_uint32, _P, _I32, _I32, C.POINTER(_I32))
_sig("painty_texture_dictionary_lookup", _P, _P, _I32, _D, C.POINTER(_I32))
_sig("painty_gpu_texture_brush_create", _P, C.POINTER(_P))
_sig("painty_gpu_texture_brush_destroy", _P)
_sig("painty_gpu_texture_brush_set_radius", _P, _D)
_sig("painty_gpu_texture_brush_dip", _P, _P, _P)
_sig("painty_gpu_texture_brush_set_thickness_scale", _P, _D)
_sig("painty_gpu_texture_brush_set_smudge", _P, _I32)
_sig("painty_gpu_texture_brush_last_texture", _P, C.POINTER(_I32))
_sig("painty_gpu_texture_brush_paint_stroke", _P, _P, _P, _I32, _P)

# painty_stroke_desc (include/painty_gb300.h)
STROKE_DESC = np.dtype([("canvas", np.int32), ("npoints", np.int32), ("first_point", np.int64),
                        ("radius", np.float64), ("spacing", np.float64),
                        ("K", np.float64, 3), ("S", np.float64, 3)])

ABI_VERSION = _lib.painty_abi_version()


class PaintyError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


class PaintyValueError(PaintyError, ValueError):
    pass


def _check(status: int) -> None:
    if status == 0:
        return
    msg = f"{_lib.painty_status_string(status).decode()}: {_lib.painty_last_error().decode()}"
    if status == 1:
        raise PaintyValueError(status, msg)
    if status == 2:
        raise MemoryError(msg)
    raise PaintyError(status, msg)


def bounds_checked() -> bool:
    """Whether the loaded library is the bounds-checked build."""
    return bool(_lib.painty_build_flags() & 1)


def kernel_launch_count() -> int:
    """Kernel launches this library has issued in this process."""
    return int(_lib.painty_kernel_launch_count())


PHASES = ("paint", "refresh", "classify", "derive", "setup", "cta_barrier", "cluster_barrier",
          "waves")


def take_phase_cycles() -> dict:
    """Phase-timing build: reads and clears the stamp loop's counters. Returns the stamps
    (summed over CTAs) and, per phase, the clock cycles a warp spent in it per stamp."""
    v = (C.c_uint64 * 16)()
    _check(_lib.painty_take_phase_cycles(v))
    ws = max(int(v[9]), 1)  # warp-stamps: lane 0 of each warp records its warp
    return {"stamps": int(v[8]),
            "cycles_per_stamp": {p: round(v[i] / ws, 1) for i, p in enumerate(PHASES)}}


def take_device_faults() -> int:
    """Reads and clears the device's pipeline-fault word (nonzero: a kernel's copy pipeline
    stalled past its wait limit and wrote NaN instead of hanging)."""
    v = C.c_uint32()
    _check(_lib.painty_take_device_faults(C.byref(v)))
    return int(v.value)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


def _host_fmt(a: np.ndarray, planar: bool) -> int:
    if a.dtype == np.float64:
        return HOST_F64_PLANAR if planar else HOST_F64_INTERLEAVED
    if a.dtype == np.float32:
        return HOST_F32_PLANAR if planar else HOST_F32_INTERLEAVED
    raise TypeError("host buffers are float32 or float64")


def _shape3(rows, cols, planar):
    return (3, rows, cols) if planar else (rows, cols, 3)


class PaintLayer:
    """painty::PaintLayer<vec3> on the device (PaintLayer.hxx:21-145)."""

    def __init__(self, rows: int, cols: int, storage: str = "f32", *, _handle=None, _owner=None):
        self.storage = storage
        if _handle is not None:
            self._h = _handle
            self._owned = False
            self._owner = _owner
        else:
            h = _P()
            _check(_lib.painty_layer_create(rows, cols, STORAGE[storage], C.byref(h)))
            self._h = h.value
            self._owned = True
        r, c, s = _I32(), _I32(), C.c_int()
        _check(_lib.painty_layer_info(self._h, C.byref(r), C.byref(c), C.byref(s)))
        self.rows, self.cols = r.value, c.value

    def __del__(self):
        if getattr(self, "_owned", False) and self._h:
            _lib.painty_layer_destroy(self._h)
            self._h = None

    def getRows(self) -> int:
        return self.rows

    def getCols(self) -> int:
        return self.cols

    def clear(self, stream=None) -> None:
        _check(_lib.painty_layer_clear(self._h, _stream(stream)))

    def upload(self, plane: str, data: np.ndarray, planar: bool = False, stream=None) -> None:
        data = np.ascontiguousarray(data)
        _check(_lib.painty_layer_upload(self._h, PLANE[plane], _ptr(data),
                                        _host_fmt(data, planar), _stream(stream)))

    def download(self, plane: str, dtype=np.float64, planar: bool = False, stream=None):
        shape = (self.rows, self.cols) if plane == "V" else _shape3(self.rows, self.cols, planar)
        out = np.empty(shape, dtype=dtype)
        _check(_lib.painty_layer_download(self._h, PLANE[plane], _ptr(out),
                                          _host_fmt(out, planar), _stream(stream)))
        return out

    def set(self, K: np.ndarray, S: np.ndarray, V: np.ndarray, stream=None) -> None:
        self.upload("K", K, stream=stream)
        self.upload("S", S, stream=stream)
        self.upload("V", V, stream=stream)

    def setCells(self, rows_cols, K, S, V, stream=None) -> None:
        """PaintLayer::set(i, j, k, s, v) (PaintLayer.hxx:122-127) for many cells, in order."""
        rc = np.ascontiguousarray(rows_cols, dtype=np.int32).reshape(-1, 2)
        K = np.ascontiguousarray(K, dtype=np.float64).reshape(-1, 3)
        S = np.ascontiguousarray(S, dtype=np.float64).reshape(-1, 3)
        V = np.ascontiguousarray(V, dtype=np.float64).reshape(-1)
        n = rc.shape[0]
        if not (K.shape[0] == S.shape[0] == V.shape[0] == n):
            raise ValueError("rows_cols, K, S and V describe different numbers of cells")
        _check(_lib.painty_layer_set_cells(self._h, n, _ptr(rc), _ptr(K), _ptr(S), _ptr(V),
                                           _stream(stream)))

    def setCell(self, i: int, j: int, k, s, v: float) -> None:
        """PaintLayer::set(i, j, k, s, v)."""
        self.setCells([[i, j]], [k], [s], [v])

    def getK_buffer(self):
        return self.download("K")

    def getS_buffer(self):
        return self.download("S")

    def getV_buffer(self):
        return self.download("V")

    def copyTo(self, other: "PaintLayer", stream=None) -> None:
        _check(_lib.painty_layer_copy(self._h, other._h, _stream(stream)))

    def composeOnto(self, R0: "Image", stream=None) -> None:
        """PaintLayer::composeOnto (PaintLayer.hxx:81-96): R0 <- KM(K, S, R0, V) in place."""
        compose_layers([self], R0, R0, stream=stream)


class Image:
    """A 3-channel reflectance image (painty Mat<vec3>) on the device; F32 or F64."""

    def __init__(self, rows: int, cols: int, storage: str = "f32", *, _handle=None, _owner=None):
        self.rows, self.cols, self.storage = rows, cols, storage
        if _handle is not None:
            self._h, self._owned, self._owner = _handle, False, _owner
        else:
            h = _P()
            _check(_lib.painty_image_create(rows, cols, STORAGE[storage], C.byref(h)))
            self._h, self._owned = h.value, True

    def __del__(self):
        if getattr(self, "_owned", False) and self._h:
            _lib.painty_image_destroy(self._h)
            self._h = None

    def fill(self, r: float, g: float, b: float, stream=None) -> None:
        _check(_lib.painty_image_fill(self._h, r, g, b, _stream(stream)))

    def upload(self, data: np.ndarray, planar: bool = False, stream=None) -> None:
        data = np.ascontiguousarray(data)
        _check(_lib.painty_image_upload(self._h, _ptr(data), _host_fmt(data, planar),
                                        _stream(stream)))

    def download(self, dtype=np.float64, planar: bool = False, out=None, stream=None):
        if out is None:
            out = np.empty(_shape3(self.rows, self.cols, planar), dtype=dtype)
        _check(_lib.painty_image_download(self._h, _ptr(out), _host_fmt(out, planar),
                                          _stream(stream)))
        return out


def compose_layers(layers, r0: Image, out: Image, fused: bool = True, stream=None) -> None:
    """out = KM(layer L-1, ... KM(layer 0, r0)) -- PaintLayer::composeOnto over a stack."""
    arr = (_P * max(1, len(layers)))(*[l._h for l in layers])
    fn = _lib.painty_compose_layers if fused else _lib.painty_compose_layers_unfused
    _check(fn(arr, len(layers), r0._h, out._h, _stream(stream)))


def compose_layers_host(K: np.ndarray, S: np.ndarray, V: np.ndarray, R0: np.ndarray,
                        out: np.ndarray | None = None, stream=None) -> np.ndarray:
    """Renderer::compose of host layer stacks into a host image in one call, the transfers
    pipelined in row bands: K, S float32 (L, 3, rows, cols), V (L, rows, cols), R0 and the
    result (3, rows, cols). Pinned host arrays give full host-link speed."""
    R0 = np.ascontiguousarray(R0, dtype=np.float32)
    if R0.ndim != 3 or R0.shape[0] != 3:
        raise ValueError("R0 must be (3, rows, cols)")
    rows, cols = R0.shape[1:]
    L = V.shape[0]
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (K, S, V)]
    if arrs[0].shape != (L, 3, rows, cols) or arrs[1].shape != (L, 3, rows, cols) or \
            arrs[2].shape != (L, rows, cols):
        raise ValueError("K, S must be (L, 3, rows, cols) and V (L, rows, cols)")
    if out is None:
        out = np.empty((3, rows, cols), dtype=np.float32)
    elif out.shape != (3, rows, cols) or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
        raise ValueError("out must be a C-contiguous float32 array of (3, rows, cols)")
    _check(_lib.painty_compose_layers_host(_ptr(arrs[0]), _ptr(arrs[1]), _ptr(arrs[2]), L,
                                           _ptr(R0), _ptr(out), rows, cols, _stream(stream)))
    return out


class Canvas:
    """painty::Canvas<vec3> (Canvas.hxx:20-198) on the device."""

    def __init__(self, rows: int, cols: int, storage: str = "f32"):
        h = _P()
        _check(_lib.painty_canvas_create(rows, cols, STORAGE[storage], C.byref(h)))
        self._h = h.value
        self.rows, self.cols, self.storage = rows, cols, storage

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.painty_canvas_destroy(self._h)
            self._h = None

    def clear(self, stream=None) -> None:
        _check(_lib.painty_canvas_clear(self._h, _stream(stream)))

    def upload(self, plane: str, data: np.ndarray, planar: bool = False, stream=None) -> None:
        data = np.ascontiguousarray(data)
        _check(_lib.painty_canvas_upload(self._h, PLANE[plane], _ptr(data),
                                         _host_fmt(data, planar), _stream(stream)))

    def download(self, plane: str, dtype=np.float64, planar: bool = False, stream=None):
        one = plane in ("V", "h", "VL")
        shape = (self.rows, self.cols) if one else _shape3(self.rows, self.cols, planar)
        out = np.empty(shape, dtype=dtype)
        _check(_lib.painty_canvas_download(self._h, PLANE[plane], _ptr(out),
                                           _host_fmt(out, planar), _stream(stream)))
        return out

    def setBackground(self, background: np.ndarray) -> None:
        """Canvas::setBackground (Canvas.hxx:80-87): clear, then R0 = background."""
        self.clear()
        self.upload("R0", background)

    def getR0(self):
        return self.download("R0")

    def get_h(self):
        return self.download("h")

    def getComposedGlsl(self, out: Image | None = None, stream=None) -> Image:
        """CanvasGpu::getComposed (CanvasGpu.cxx:91-95): the GL path's composite."""
        if out is None:
            out = Image(self.rows, self.cols, "f32")
        _check(_lib.painty_canvas_compose_glsl(self._h, out._h, _stream(stream)))
        return out

    def dryStep(self, step: float = 0.01, stream=None) -> None:
        """CanvasGpu::dryStep (CanvasGpu.cxx:112-128)."""
        _check(_lib.painty_canvas_dry_step(self._h, float(step), _stream(stream)))

    def getPaintLayer(self) -> PaintLayer:
        h = _P()
        _check(_lib.painty_canvas_layer(self._h, C.byref(h)))
        return PaintLayer(0, 0, self.storage, _handle=h.value, _owner=self)

    def r0_image(self) -> Image:
        h = _P()
        _check(_lib.painty_canvas_r0(self._h, C.byref(h)))
        return Image(self.rows, self.cols, "f64" if self.storage == "f64" else "f32",
                     _handle=h.value, _owner=self)

    def dryCanvas(self, stream=None) -> None:
        _check(_lib.painty_canvas_dry(self._h, _stream(stream)))


class Renderer:
    """painty::Renderer<vec3>::compose (Renderer.hxx:26-53)."""

    def compose(self, canvas: Canvas, out: Image | None = None, stream=None) -> Image:
        if out is None:
            out = Image(canvas.rows, canvas.cols, "f64" if canvas.storage == "f64" else "f32")
        _check(_lib.painty_canvas_compose(canvas._h, out._h, _stream(stream)))
        return out

    def render(self, canvas: Canvas, out: Image | None = None, stream=None) -> Image:
        """Renderer::render (Renderer.hxx:60-156): the composite lit by a point light."""
        if out is None:
            out = Image(canvas.rows, canvas.cols, "f64" if canvas.storage == "f64" else "f32")
        _check(_lib.painty_canvas_render(canvas._h, out._h, _stream(stream)))
        return out


class FootprintBrush:
    """painty::FootprintBrush<vec3> (FootprintBrush.hxx:22-502).

    `footprint` is the full-size footprint image (values in [0, 1]) that stands in for
    data/footprint/footprint.png.
    """

    def __init__(self, radius: float, footprint: np.ndarray):
        fp = np.ascontiguousarray(footprint, dtype=np.float64)
        h = _P()
        _check(_lib.painty_brush_create(float(radius), _ptr(fp), fp.shape[0], fp.shape[1],
                                        C.byref(h)))
        self._h = h.value

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.painty_brush_destroy(self._h)
            self._h = None

    def setRadius(self, radius: float) -> None:
        _check(_lib.painty_brush_set_radius(self._h, float(radius)))

    def setPickupRate(self, rate: float) -> None:
        _, dep = self.rates()
        _check(_lib.painty_brush_set_rates(self._h, float(rate), dep))

    def setDepositionRate(self, rate: float) -> None:
        pick, _ = self.rates()
        _check(_lib.painty_brush_set_rates(self._h, pick, float(rate)))

    def rates(self):
        p, d = _D(), _D()
        _check(_lib.painty_brush_get_rates(self._h, C.byref(p), C.byref(d)))
        return p.value, d.value

    def getPickupRate(self) -> float:
        return self.rates()[0]

    def getDepositionRate(self) -> float:
        return self.rates()[1]

    def setUseSnapshotBuffer(self, use: bool) -> None:
        _check(_lib.painty_brush_set_snapshot(self._h, 1 if use else 0))

    def dip(self, paint) -> None:
        K = np.ascontiguousarray(paint[0], dtype=np.float64)
        S = np.ascontiguousarray(paint[1], dtype=np.float64)
        _check(_lib.painty_brush_dip(self._h, _ptr(K), _ptr(S), None))

    def updateSnapshot(self, canvas: Canvas, stream=None) -> None:
        _check(_lib.painty_brush_update_snapshot(self._h, canvas._h, _stream(stream)))

    def info(self):
        r, F, S = _D(), _I32(), _I32()
        _check(_lib.painty_brush_info(self._h, C.byref(r), C.byref(F), C.byref(S)))
        return r.value, F.value, S.value

    def getFootprint(self) -> np.ndarray:
        _, F, _ = self.info()
        out = np.empty((F, F), dtype=np.float64)
        _check(_lib.painty_brush_footprint(self._h, _ptr(out)))
        return out

    def getPickupMap(self, plane: str, dtype=np.float64) -> np.ndarray:
        _, _, S = self.info()
        shape = (S, S) if plane == "V" else (S, S, 3)
        out = np.empty(shape, dtype=dtype)
        _check(_lib.painty_brush_download_pickup(self._h, PLANE[plane], _ptr(out),
                                                 _host_fmt(out, False), None))
        return out

    def imprint(self, center, theta: float, canvas: Canvas, stream=None) -> None:
        _check(_lib.painty_imprint(canvas._h, self._h, float(center[0]), float(center[1]),
                                   float(theta), _stream(stream)))

    def stamps(self, cx_cy_theta: np.ndarray, canvas: Canvas, stream=None) -> None:
        s = np.ascontiguousarray(cx_cy_theta, dtype=np.float64).reshape(-1, 3)
        _check(_lib.painty_stamps(canvas._h, self._h, _ptr(s), s.shape[0], _stream(stream)))

    def paintStroke(self, path: np.ndarray, canvas: Canvas, spacing: float = 1.0,
                    stream=None) -> int:
        p = np.ascontiguousarray(path, dtype=np.float64).reshape(-1, 2)
        n = _I64()
        _check(_lib.painty_stroke(canvas._h, self._h, _ptr(p), p.shape[0], float(spacing),
                                  C.byref(n), _stream(stream)))
        return n.value


class TextureBrush:
    """painty::TextureBrush<vec3> (TextureBrush.hxx:20-237) with its Smudge (Smudge.hxx).

    `texture` is the brush-stroke sample's thickness map (rows x cols, values >= 0) that
    stands in for the sample directory painty's constructor reads.
    """

    def __init__(self, texture: np.ndarray):
        t = np.ascontiguousarray(texture, dtype=np.float64)
        h = _P()
        _check(_lib.painty_texture_brush_create(_ptr(t), t.shape[0], t.shape[1], C.byref(h)))
        self._h = h.value

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.painty_texture_brush_destroy(self._h)
            self._h = None

    def setRadius(self, radius: float) -> None:
        _check(_lib.painty_texture_brush_set_radius(self._h, float(radius)))

    def dip(self, paint) -> None:
        K = np.ascontiguousarray(paint[0], dtype=np.float64)
        S = np.ascontiguousarray(paint[1], dtype=np.float64)
        _check(_lib.painty_texture_brush_dip(self._h, _ptr(K), _ptr(S)))

    def enableSmudge(self, enable: bool) -> None:
        _check(_lib.painty_texture_brush_set_smudge(self._h, 1 if enable else 0))

    def setThicknessScale(self, scale: float) -> None:
        _check(_lib.painty_texture_brush_set_thickness_scale(self._h, float(scale)))

    def paintStroke(self, path: np.ndarray, canvas: Canvas, stream=None) -> int:
        """Paints the stroke; returns the number of pixels it deposited on."""
        p = np.ascontiguousarray(path, dtype=np.float64).reshape(-1, 2)
        n = _I64()
        _check(_lib.painty_texture_brush_paint_stroke(canvas._h, self._h, _ptr(p), p.shape[0],
                                                      C.byref(n), _stream(stream)))
        return n.value

    def getSmudgeMap(self, plane: str) -> np.ndarray:
        """The smudge pickup map's K / S (side, side, 3) or V (side, side)."""
        side = _I32()
        _check(_lib.painty_texture_brush_smudge_map(self._h, PLANE[plane], None, C.byref(side),
                                                    None))
        n = side.value
        out = np.empty((n, n) if plane == "V" else (n, n, 3), dtype=np.float64)
        if n:
            _check(_lib.painty_texture_brush_smudge_map(self._h, PLANE[plane], _ptr(out),
                                                        C.byref(side), None))
        return out


class TextureBrushDictionary:
    """painty::TextureBrushDictionary (TextureBrushDictionary.hxx:17-39) with a seeded pick."""

    def __init__(self, seed: int = 0):
        h = _P()
        _check(_lib.painty_texture_dictionary_create(int(seed) & 0xffffffff, C.byref(h)))
        self._h = h.value

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.painty_texture_dictionary_destroy(self._h)
            self._h = None

    def add(self, radius_class: int, length_class: int, height: np.ndarray) -> int:
        """One texture of class (radius token, length token); returns its index."""
        t = np.ascontiguousarray(height, dtype=np.float64)
        i = _I32()
        _check(_lib.painty_texture_dictionary_add(self._h, radius_class, length_class, _ptr(t),
                                                  t.shape[0], t.shape[1], C.byref(i)))
        return i.value

    def lookup(self, path: np.ndarray, brush_size: float) -> int:
        p = np.ascontiguousarray(path, dtype=np.float64).reshape(-1, 2)
        i = _I32()
        _check(_lib.painty_texture_dictionary_lookup(self._h, _ptr(p), p.shape[0],
                                                     float(brush_size), C.byref(i)))
        return i.value


class TextureBrushGpu:
    """painty::TextureBrushGpu (TextureBrushGpu.hxx:21-64) painting the GL canvas path."""

    def __init__(self, dictionary: TextureBrushDictionary):
        h = _P()
        _check(_lib.painty_gpu_texture_brush_create(dictionary._h, C.byref(h)))
        self._h = h.value
        self._dict = dictionary  # the brush borrows it

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.painty_gpu_texture_brush_destroy(self._h)
            self._h = None

    def setRadius(self, radius: float) -> None:
        _check(_lib.painty_gpu_texture_brush_set_radius(self._h, float(radius)))

    def dip(self, paint) -> None:
        K = np.ascontiguousarray(paint[0], dtype=np.float64)
        S = np.ascontiguousarray(paint[1], dtype=np.float64)
        _check(_lib.painty_gpu_texture_brush_dip(self._h, _ptr(K), _ptr(S)))

    def setThicknessScale(self, scale: float) -> None:
        _check(_lib.painty_gpu_texture_brush_set_thickness_scale(self._h, float(scale)))

    def enableSmudge(self, enable: bool) -> None:
        _check(_lib.painty_gpu_texture_brush_set_smudge(self._h, 1 if enable else 0))

    def lastTexture(self) -> int:
        i = _I32()
        _check(_lib.painty_gpu_texture_brush_last_texture(self._h, C.byref(i)))
        return i.value

    def paintStroke(self, path: np.ndarray, canvas: Canvas, stream=None) -> None:
        p = np.ascontiguousarray(path, dtype=np.float64).reshape(-1, 2)
        _check(_lib.painty_gpu_texture_brush_paint_stroke(canvas._h, self._h, _ptr(p),
                                                          p.shape[0], _stream(stream)))


class SbrRenderThread:
    """painty::SbrRenderThread (SbrRenderThread.hxx:19-116): one worker thread owns a canvas
    and a TextureBrushGpu (the GL canvas path) and runs requests in order; calls return
    concurrent.futures futures. The worker dries the canvas by Canvas.dryStep() every
    `dry_interval` seconds (0.25 in painty; 0 turns it off). No window is shown."""

    def __init__(self, rows: int, cols: int, dictionary: TextureBrushDictionary,
                 background: np.ndarray | None = None, dry_interval: float = 0.25):
        import concurrent.futures as cf
        import threading

        self._rows, self._cols = rows, cols
        self._dict = dictionary
        self._scale = 1.0
        self._pool = cf.ThreadPoolExecutor(max_workers=1)

        def make():
            self._brush = TextureBrushGpu(dictionary)
            self._canvas = Canvas(rows, cols, "f32")
            if background is not None:
                self._canvas.setBackground(background)

        self._pool.submit(make).result()
        self._stop = threading.Event()
        self._timer = None
        if dry_interval > 0:
            def tick():
                while not self._stop.wait(dry_interval):
                    try:
                        self._pool.submit(self._canvas.dryStep)
                    except RuntimeError:  # the pool has shut down
                        return
            self._timer = threading.Thread(target=tick, daemon=True)
            self._timer.start()

    def close(self) -> None:
        if self._pool is None:
            return
        self._stop.set()
        if self._timer is not None:
            self._timer.join()

        def release():
            self._brush = None
            self._canvas = None

        self._pool.submit(release).result()
        self._pool.shutdown(wait=True)
        self._pool = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def getSize(self):
        return self._rows, self._cols

    def getBrushThicknessScale(self) -> float:
        return self._scale

    def render(self, path: np.ndarray, radius: float, ks):
        """dip, setRadius, paintStroke on the worker (SbrRenderThread.cxx:70-78)."""
        path = np.array(path, dtype=np.float64)
        ks = (np.array(ks[0], dtype=np.float64), np.array(ks[1], dtype=np.float64))

        def job():
            self._brush.dip(ks)
            self._brush.setRadius(radius)
            self._brush.paintStroke(path, self._canvas)

        return self._pool.submit(job)

    def getLinearRgbImage(self):
        """CanvasGpu::getCompositionLinearRgb: a (rows, cols, 3) float64 image."""
        return self._pool.submit(lambda: self._canvas.getComposedGlsl().download())

    def setBrushThicknessScale(self, scale: float) -> None:
        self._scale = float(scale)
        self._pool.submit(self._brush.setThicknessScale, float(scale))

    def enableSmudge(self, enable: bool) -> None:
        if enable:
            raise PaintyError(4, "unsupported: the GL smudge pass is not provided")

    def dryCanvas(self):
        """dryStep(1.0) (SbrRenderThread.cxx:100-104)."""
        return self._pool.submit(self._canvas.dryStep, 1.0)


def mix_single_paint(weights: np.ndarray, palette_K: np.ndarray, palette_S: np.ndarray):
    """PaintMixer::mixSinglePaint (PaintMixer.cxx:327-355): (K, S) of the weighted mix."""
    w = np.ascontiguousarray(weights, dtype=np.float64)
    pk = np.ascontiguousarray(palette_K, dtype=np.float64)
    ps = np.ascontiguousarray(palette_S, dtype=np.float64)
    if pk.shape != (w.size, 3) or ps.shape != (w.size, 3):
        raise ValueError("Palette size does not match underlying size.")
    K = np.zeros(3)
    S = np.zeros(3)
    _check(_lib.painty_mix_paint(_ptr(w), w.size, _ptr(pk), _ptr(ps), _ptr(K), _ptr(S)))
    return K, S


def paint_batch(canvases, brushes, strokes, stream=None) -> int:
    """Paints many canvases in one launch (painty_paint_batch).

    strokes: iterable of (canvas_index, path (n, 2), radius, spacing, K (3), S (3)). For each
    canvas its strokes are applied in order as brush.setRadius, brush.dip, brush.paintStroke.
    Returns the number of stamps.
    """
    strokes = list(strokes)
    desc = np.zeros(len(strokes), dtype=STROKE_DESC)
    paths = []
    offset = 0
    for i, (ci, path, radius, spacing, K, S) in enumerate(strokes):
        p = np.ascontiguousarray(path, dtype=np.float64).reshape(-1, 2)
        desc[i] = (ci, p.shape[0], offset, radius, spacing, K, S)
        paths.append(p)
        offset += p.shape[0]
    pts = np.ascontiguousarray(np.concatenate(paths) if paths else np.zeros((0, 2)))
    carr = (_P * len(canvases))(*[c._h for c in canvases])
    barr = (_P * len(brushes))(*[b._h for b in brushes])
    n = _I64()
    _check(_lib.painty_paint_batch(carr, barr, len(canvases), desc.ctypes.data, len(strokes),
                                   pts.ctypes.data, pts.shape[0], C.byref(n), _stream(stream)))
    return n.value


def batch_last_shape():
    """(CTAs per canvas, clusters, threads per CTA) of the last paint_batch on this thread."""
    cl, n, t = _I32(), _I32(), _I32()
    _check(_lib.painty_batch_last_shape(C.byref(cl), C.byref(n), C.byref(t)))
    return cl.value, n.value, t.value


def batch_last_split():
    """(cluster size, canvases) of the last paint_batch's launch for its heaviest canvases on
    this thread ((0, 0): none)."""
    cl, n = _I32(), _I32()
    _check(_lib.painty_batch_last_split(C.byref(cl), C.byref(n)))
    return cl.value, n.value


class _ServerOptions(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("storage", C.c_int), ("max_active", C.c_int32),
                ("step_stamps", C.c_int64), ("pickup_rate", C.c_double),
                ("deposition_rate", C.c_double), ("footprint", C.c_void_p),
                ("footprint_rows", C.c_int32), ("footprint_cols", C.c_int32)]


class _Request(C.Structure):
    _fields_ = [("canvas_id", C.c_uint64), ("rows", C.c_int32), ("cols", C.c_int32),
                ("r0", C.c_void_p), ("strokes", C.c_void_p), ("nstrokes", C.c_int64),
                ("points", C.c_void_p), ("npoints", C.c_int64), ("out_rgb", C.c_void_p)]


class _Counters(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "cancelled", "steps",
                                          "stamps", "evictions", "restores")] + \
               [("resident_bytes", C.c_uint64), ("peak_resident_bytes", C.c_uint64)] + \
               [(n, C.c_int64) for n in ("active", "pending", "canvases", "worker_busy_us",
                                          "worker_create_us", "worker_launch_us",
                                          "worker_finish_us")] + \
               [("heap_bytes", C.c_uint64), ("heap_fallbacks", C.c_int64)]


_sig("painty_server_create", C.POINTER(_ServerOptions), C.POINTER(_P))
_sig("painty_server_submit", _P, C.POINTER(_Request), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64))
_sig("painty_server_wait", _P, C.c_uint64, _D, C.POINTER(_D), C.POINTER(_I64))
_sig("painty_server_cancel", _P, C.c_uint64)
_sig("painty_server_release", _P, C.c_uint64)
_sig("painty_server_poll", _P, _D, C.POINTER(C.c_uint64))
_sig("painty_server_stats", _P, C.POINTER(_Counters))
_sig("painty_server_destroy", _P)


def _strokes_to_desc(strokes):
    desc = np.zeros(len(strokes), dtype=STROKE_DESC)
    paths, offset = [], 0
    for i, (path, radius, spacing, K, S) in enumerate(strokes):
        p = np.ascontiguousarray(path, dtype=np.float64).reshape(-1, 2)
        desc[i] = (0, p.shape[0], offset, radius, spacing, K, S)
        paths.append(p)
        offset += p.shape[0]
    pts = np.ascontiguousarray(np.concatenate(paths) if paths else np.zeros((0, 2)))
    return desc, pts


class Server:
    """Continuous-batching render server (painty_server_*): requests paint strokes on a new
    canvas or continue one; results are the canvases' KM composites."""

    def __init__(self, budget_bytes: int, footprint: np.ndarray, storage: str = "f16",
                 pickup_rate: float = 0.05, deposition_rate: float = 0.1, max_active: int = 256,
                 step_stamps: int = 16384):
        self._fp = np.ascontiguousarray(footprint, dtype=np.float64)
        o = _ServerOptions(int(budget_bytes), STORAGE[storage], max_active, step_stamps,
                           pickup_rate, deposition_rate, self._fp.ctypes.data,
                           self._fp.shape[0], self._fp.shape[1])
        h = _P()
        _check(_lib.painty_server_create(C.byref(o), C.byref(h)))
        self._h = h.value
        self._dims = {}
        self._live = {}  # request id -> buffers that must outlive the request

    def submit(self, strokes, canvas_id: int = 0, rows: int = 0, cols: int = 0, r0=None,
               want_result: bool = True, out=None):
        """strokes: [(path, radius, spacing, K, S)]; returns (request_id, canvas_id).
        out: the caller's (rows, cols, 3) float32 buffer for the result (pinned host memory
        keeps the server's worker from blocking on the copy); by default a new array."""
        desc, pts = _strokes_to_desc(strokes)
        if canvas_id:
            rows, cols = self._dims.get(canvas_id, (0, 0))
        r0a = None if r0 is None else np.ascontiguousarray(r0, dtype=np.float32)
        if out is not None:
            if (out.dtype != np.float32 or out.shape != (rows, cols, 3)
                    or not out.flags["C_CONTIGUOUS"]):
                raise ValueError("out must be a C-contiguous float32 array of (rows, cols, 3)")
        elif want_result:
            out = np.empty((rows, cols, 3), dtype=np.float32)
        req = _Request(canvas_id, rows, cols, None if r0a is None else r0a.ctypes.data,
                       desc.ctypes.data, len(desc), pts.ctypes.data, pts.shape[0],
                       None if out is None else out.ctypes.data)
        rid, cid = C.c_uint64(), C.c_uint64()
        _check(_lib.painty_server_submit(self._h, C.byref(req), C.byref(rid), C.byref(cid)))
        self._dims.setdefault(cid.value, (rows, cols))
        self._live[rid.value] = (out, r0a)  # a pinned substrate is read when the canvas is made
        return rid.value, cid.value

    def wait(self, request_id: int, timeout: float = -1.0):
        """Blocks until the request finished; returns (result image or None, latency s,
        stamps). Raises on a failed, cancelled or unfinished request."""
        lat, st = _D(), _I64()
        status = _lib.painty_server_wait(self._h, request_id, timeout, C.byref(lat), C.byref(st))
        out = self._live.get(request_id, (None, None))[0]
        if status != 6:  # not a timeout: the request is over
            self._live.pop(request_id, None)
        _check(status)
        return out, lat.value, st.value

    def poll(self, timeout: float = -1.0):
        """The id of the next request to finish (completion order), or None on timeout."""
        rid = C.c_uint64()
        status = _lib.painty_server_poll(self._h, timeout, C.byref(rid))
        if status == 6:
            return None
        _check(status)
        return rid.value

    def cancel(self, request_id: int) -> None:
        _check(_lib.painty_server_cancel(self._h, request_id))

    def release(self, canvas_id: int) -> None:
        """Drops a canvas once the requests queued on it have finished."""
        _check(_lib.painty_server_release(self._h, canvas_id))

    def stats(self) -> dict:
        c = _Counters()
        _check(_lib.painty_server_stats(self._h, C.byref(c)))
        return {n: getattr(c, n) for n, _ in _Counters._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            _check(_lib.painty_server_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
