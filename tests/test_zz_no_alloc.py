"""painty_stamps_f32_noalloc: stamping for callers that cannot allocate device memory (GPU).

Some callers cannot call cudaMalloc -- a plugin whose host application hands out fixed
device buffers, or a real-time loop that must not stall on an allocation. This entry point
takes every buffer from the caller and keeps its only scratch in a fixed array inside the
library. This test calls it through the C ABI on buffers the test allocates itself, twice in a
row, and checks every plane it writes: the canvas and the pickup map against the allocating
entry point (painty_stamps) on the same inputs, and the caller's snapshot planes against the
double oracle's snapshot buffer.

Kept in its own file, collected last, so a run that stops at its first failure has already
run every other test.
"""
import ctypes as C
import math

import numpy as np
import pytest

from painty_gb300 import workloads
from test_gpu_stamps import F32_REL_TOL

pytestmark = pytest.mark.gpu

_FP = C.POINTER(C.c_float)


class StampBuffers(C.Structure):
    _fields_ = [
        ("canvas_K", _FP * 3), ("canvas_S", _FP * 3), ("canvas_V", _FP),
        ("snapshot_K", _FP * 3), ("snapshot_S", _FP * 3), ("snapshot_V", _FP),
        ("pickup_K", _FP * 3), ("pickup_S", _FP * 3), ("pickup_V", _FP),
        ("footprint", _FP), ("stamps", C.POINTER(C.c_double)), ("n", C.c_int64),
        ("rows", C.c_int32), ("cols", C.c_int32), ("pitch", C.c_int64),
        ("footprint_side", C.c_int32), ("map_side", C.c_int32),
        ("radius", C.c_double), ("pickup_rate", C.c_double), ("deposition_rate", C.c_double),
        ("capacity", C.c_double), ("paint_K", C.c_double * 3), ("paint_S", C.c_double * 3),
    ]


def _fp(t):
    return C.cast(C.c_void_p(t.data_ptr()), _FP)


def _records(torch, st):
    rec = np.array([[x, y, math.cos(-t), math.sin(-t)] for x, y, t in st], dtype=np.float64)
    return torch.from_numpy(rec).cuda()


def _rel(got, want):
    """Largest error relative to max(|want|, 1), the stamp tests' FP32 measure."""
    return float((np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1.0)).max())


def _fn(pg):
    fn = pg._lib.painty_stamps_f32_noalloc
    fn.argtypes = [C.POINTER(StampBuffers), C.c_void_p]
    fn.restype = C.c_int
    return fn


# radius 12: a small stamp; radius 90: footprint side 255 and map side 256, the largest the
# fixed scratch array accepts
@pytest.mark.parametrize("radius", [12.0, 90.0])
def test_noalloc_matches_allocating_entry(pg, oracle, radius):
    torch = pytest.importorskip("torch")
    lib = pg._lib
    fn = _fn(pg)

    rows, cols, pitch = 150, 190, 200
    rng = np.random.default_rng(int(radius))
    wet = {"K": rng.uniform(0.01, 5, (rows, cols, 3)), "S": rng.uniform(0.05, 3, (rows, cols, 3)),
           "V": np.where(rng.random((rows, cols)) < 0.5, 0.0, rng.uniform(0, 3, (rows, cols)))}
    wet = {k: v.astype(np.float32) for k, v in wet.items()}
    paint = (rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3))
    fp_img = workloads.footprint_image(seed=7)

    # allocating entry point
    canvas = pg.Canvas(rows, cols, "f32")
    for k, v in wet.items():
        canvas.upload(k, v)
    brush = pg.FootprintBrush(radius, fp_img)
    brush.setPickupRate(0.05)
    brush.setDepositionRate(0.1)
    brush.dip(paint)
    r_eff, F, S = brush.info()
    if radius == 90.0:
        assert (F, S) == (255, 256)
    # the double oracle on the same values, for the snapshot buffer
    oc = oracle.canvas(rows, cols)
    for k, v in wet.items():
        oc.set(k, v.astype(np.float64))
    ob = oracle.brush(radius, fp_img)
    ob.set_rates(0.05, 0.1)
    ob.dip(*paint)

    # caller-owned device buffers for the allocation-free entry point
    def planes(n, h, w):
        return [torch.zeros((h, w), dtype=torch.float32, device="cuda") for _ in range(n)]

    cK, cS, cV = planes(3, rows, pitch), planes(3, rows, pitch), planes(1, rows, pitch)[0]
    for i in range(3):
        cK[i][:, :cols] = torch.from_numpy(np.ascontiguousarray(wet["K"][..., i]))
        cS[i][:, :cols] = torch.from_numpy(np.ascontiguousarray(wet["S"][..., i]))
    cV[:, :cols] = torch.from_numpy(wet["V"])
    sK = [t.clone() for t in cK]  # painty copies the canvas into the snapshot on first use
    sS = [t.clone() for t in cS]
    sV = cV.clone()
    pK, pS, pV = planes(3, S, S), planes(3, S, S), planes(1, S, S)[0]  # dipped: all zero
    footprint = torch.from_numpy(brush.getFootprint().astype(np.float32)).cuda()

    buf = StampBuffers()
    for i in range(3):
        buf.canvas_K[i], buf.canvas_S[i] = _fp(cK[i]), _fp(cS[i])
        buf.snapshot_K[i], buf.snapshot_S[i] = _fp(sK[i]), _fp(sS[i])
        buf.pickup_K[i], buf.pickup_S[i] = _fp(pK[i]), _fp(pS[i])
        buf.paint_K[i], buf.paint_S[i] = float(paint[0][i]), float(paint[1][i])
    buf.canvas_V, buf.snapshot_V, buf.pickup_V = _fp(cV), _fp(sV), _fp(pV)
    buf.footprint = _fp(footprint)
    buf.rows, buf.cols, buf.pitch = rows, cols, pitch
    buf.footprint_side, buf.map_side = F, S
    buf.radius, buf.pickup_rate, buf.deposition_rate, buf.capacity = r_eff, 0.05, 0.1, 1.0

    def host(ts, h, w):
        return np.stack([t[:h, :w].cpu().numpy() for t in ts], axis=-1)

    for call in range(2):  # two calls in a row; state carries over as with painty's brush
        st = np.stack([rng.uniform(-10, cols + 10, 12), rng.uniform(-10, rows + 10, 12),
                       rng.uniform(-3.2, 3.2, 12)], axis=1)
        st[0, :2] = [0.5, 0.25]
        brush.stamps(st, canvas)
        ob.stamps(oc, st)
        rec = _records(torch, st)
        buf.stamps = C.cast(C.c_void_p(rec.data_ptr()), C.POINTER(C.c_double))
        buf.n = len(st)
        status = fn(C.byref(buf), None)
        assert status == 0, lib.painty_last_error().decode()
        torch.cuda.synchronize()
        errs = {
            "canvas K": _rel(host(cK, rows, cols), canvas.download("K")),
            "canvas S": _rel(host(cS, rows, cols), canvas.download("S")),
            "canvas V": _rel(cV[:, :cols].cpu().numpy(), canvas.download("V")),
            "pickup K": _rel(host(pK, S, S), brush.getPickupMap("K")),
            "pickup S": _rel(host(pS, S, S), brush.getPickupMap("S")),
            "pickup V": _rel(pV.cpu().numpy(), brush.getPickupMap("V")),
            "snapshot K": _rel(host(sK, rows, cols), ob.snapshot("K")),
            "snapshot S": _rel(host(sS, rows, cols), ob.snapshot("S")),
            "snapshot V": _rel(sV[:, :cols].cpu().numpy(), ob.snapshot("V")),
        }
        assert max(errs.values()) <= F32_REL_TOL, (call, errs)


def test_noalloc_rejects_bad_sizes_and_values(pg):
    lib = pg._lib
    fn = _fn(pg)

    def call(F, S, radius=10.0, rate=0.05):
        buf = StampBuffers()
        buf.rows, buf.cols, buf.pitch = 10, 10, 10
        buf.footprint_side, buf.map_side = F, S
        buf.radius, buf.pickup_rate, buf.deposition_rate, buf.capacity = radius, rate, 0.1, 1.0
        return fn(C.byref(buf), None), lib.painty_last_error().decode()

    status, msg = call(257, 257)  # the first map side beyond the scratch array
    assert status == 1 and "256" in msg, msg  # PAINTY_ERR_INVALID_ARGUMENT
    assert call(255, 257)[0] == 1
    assert call(31, 32, radius=float("nan"))[0] == 1
    assert call(31, 32, radius=-1.0)[0] == 1
    assert call(31, 32, rate=float("inf"))[0] == 1
