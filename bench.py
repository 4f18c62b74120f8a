"""Benchmark: Kubelka-Munk layer composite (headline) and imprint-brush stamping (secondary).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline workload: the composite stress case -- a 4096 x 4096 canvas, 8 stacked FP32 paint
layers (K ~ U[0.01,5], S ~ U[0.05,3], h ~ U[0,0.5] with 20% h = 0 and 5% h in [1e-7,1e-4]),
substrate R0 ~ U[0.8,0.95], output RGB reflectance. Metric: Mpixel-composites/s, a pixel
counted once it has gone through all 8 layers. One step = one fused composite launch over
resident inputs (4.2 GB per step, above the 129 MB L2, so no L2 flush is needed).

`e2e` is the same metric through the C ABI with host buffers: each step is one
painty_compose_layers_host call that uploads the 8 layers and R0 from pinned host memory,
composites and downloads the RGB result, its transfers pipelined in row bands; the line also
carries this box's measured host-link bandwidth and the step's fraction of that bound.

Secondary (the `stamps` object): the plain imprint-brush case -- a 1024 x 768 FP32 canvas,
200 Catmull-Rom strokes of radius U[8,32] at 0.25 r spacing through the C ABI -- as
stamps/s.

With --impl reference the reference's CPU implementation of the composite (painty's
ComputeReflectance loop, restated in oracle/) is timed on this machine's host cores on a
bounded row sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ROWS, COLS, LAYERS = 4096, 4096, 8
BYTES_PER_PX = 28 * LAYERS + 24  # FP32: 7 planes read per layer, R0 read, RGB written
METRIC = "Mpix KM composites/s"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_from_profile():
    p = ROOT / "profiles" / "km_composite_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_launch")
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
         "utilization.gpu")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.file = None
        self.window = None  # (t0, t1) wall-clock bounds of the timed region

    def wait_ready(self, timeout: float = 5.0) -> None:
        """Blocks until the sampler has written its first line (it takes a moment to start)."""
        t = time.time()
        while self.proc is not None and time.time() - t < timeout:
            if Path(self.file.name).stat().st_size > 0:
                return
            time.sleep(0.05)

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        import datetime

        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                util = float(f[9]) if len(f) > 9 else float("nan")
                rows.append((ts, float(f[1]), float(f[2]), f[5], f[6], f[7], f[8], util))
            except ValueError:
                continue
        os.unlink(self.file.name)
        where = "timed region"
        if self.window is not None:
            t0, t1 = self.window
            inside = [r for r in rows if t0 - 0.05 <= r[0] <= t1 + 0.15]
            if not inside:  # region shorter than the sampling period: nearest samples after it
                inside = [r for r in rows if t1 <= r[0] <= t1 + 0.5][:2]
                where = "first samples after the timed region"
            rows = inside
        rows = [r[1:] for r in rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(r[0] for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[2 + i] == "Active"})
        util = [r[6] for r in rows if r[6] == r[6]]
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "window": where,
                "gpu_util_pct_mean": round(float(np.mean(util)), 1) if util else None}


def _workloads_module():
    """painty_gb300/workloads.py loaded by path: the reference arm must not import the package
    (its __init__ maps the CUDA library)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("painty_workloads_standalone",
                                                  ROOT / "painty_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod  # dataclasses look their module up while being defined
    spec.loader.exec_module(mod)
    return mod


def _headline_config(ws: int) -> dict:
    """The `config` of the headline line, shared by both arms."""
    return {"workload": f"KM composite {ROWS}x{COLS}, {LAYERS} stacked FP32 layers -> RGB",
            "rows": ROWS, "cols": COLS, "layers": LAYERS, "storage": "f32",
            "l2": "inputs 4.2 GB per step > 129 MB L2 (no flush needed)",
            "parallelism": f"replicas{ws}"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def generate_stack_device(torch, seed: int):
    """The composite workload generated on the device (same distributions as
    painty_gb300.workloads.composite_stack), returned as pinned host arrays."""
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    dev = "cuda"
    host = {}

    def uni(shape, lo, hi):
        t = torch.empty(shape, device=dev, dtype=torch.float32)
        t.uniform_(lo, hi, generator=g)
        return t

    K = uni((LAYERS, 3, ROWS, COLS), 0.01, 5.0)
    S = uni((LAYERS, 3, ROWS, COLS), 0.05, 3.0)
    V = uni((LAYERS, ROWS, COLS), 0.0, 0.5)
    sel = uni((LAYERS, ROWS, COLS), 0.0, 1.0)
    small = uni((LAYERS, ROWS, COLS), 1e-7, 1e-4)
    V = torch.where(sel < 0.20, torch.zeros_like(V), V)
    V = torch.where((sel >= 0.20) & (sel < 0.25), small, V)
    R0 = uni((3, ROWS, COLS), 0.8, 0.95)
    for name, t in (("K", K), ("S", S), ("V", V), ("R0", R0)):
        h = torch.empty(t.shape, dtype=torch.float32, pin_memory=True)
        h.copy_(t)
        host[name] = h
    del K, S, V, sel, small, R0
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return host


def run_precision_only(args):
    import torch

    import painty_gb300 as pg

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    host = generate_stack_device(torch, seed=1)
    Kh, Sh, Vh, R0h = (host[k].numpy() for k in ("K", "S", "V", "R0"))
    print(json.dumps(run_precision(pg, torch, (Kh, Sh, Vh, R0h))), flush=True)


def run_batch_only(args):
    import torch

    import painty_gb300 as pg

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    for s_ in ("f32", "f16"):
        print(json.dumps(run_batch(pg, torch, s_, args.batch_canvases, args.batch_max_strokes)),
              flush=True)


def run_serve_only(args):
    import torch

    import painty_gb300 as pg

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if args.serve_sweep:
        print(json.dumps(run_serving(pg, torch, full_rate=args.serve_rate,
                                     full_s=args.serve_seconds)), flush=True)
    else:
        print(json.dumps(run_serve(pg, torch, args.serve_rate, args.serve_seconds)), flush=True)


def run_stamps_only(args):
    """The stamping case alone (profiling runs): prints its stamps object."""
    import torch

    import painty_gb300 as pg

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    out = run_stamps_config0(pg, torch, args.strokes)
    if pg.PHASE_TIMERS:  # PAINTY_PHASE_TIMERS=1: where a stamp's cycles go, per warp
        out["phases"] = pg.take_phase_cycles()
        out["phases"]["note"] = ("phase-timing build: clock cycles per stamp per warp, averaged "
                                 "over warps and over the timed and untimed steps")
    print(json.dumps(out), flush=True)


def run_cluster_sweep(args):
    """Stamps/s by brush radius and cluster size on one 1024x768 FP32 canvas: 12 strokes of 8
    control points per point, one untimed pass first, PAINTY_STAMP_CLUSTER set per point (the
    library reads it at every stroke). One JSON line per radius."""
    import numpy as np
    import torch

    import painty_gb300 as pg
    from painty_gb300 import workloads

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    fp = workloads.footprint_image(seed=7)
    old = os.environ.get("PAINTY_STAMP_CLUSTER")
    try:
        for r in (3.0, 5.0, 7.0, 8.5, 10.0, 13.0, 16.0, 20.0, 24.0, 30.0):
            row = {"r": r}
            for cl in (1, 2, 4, 8, 16):
                os.environ["PAINTY_STAMP_CLUSTER"] = str(cl)
                rng = np.random.default_rng(3)
                c = pg.Canvas(768, 1024, "f32")
                c.upload("R0", np.full((768, 1024, 3), 0.85))
                b = pg.FootprintBrush(r, fp)
                b.setPickupRate(0.05)
                b.setDepositionRate(0.1)
                paths = [np.stack([rng.uniform(100, 924, 8), rng.uniform(100, 668, 8)], axis=1)
                         for _ in range(12)]

                def run():
                    n = 0
                    for p in paths:
                        b.dip((rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)))
                        n += b.paintStroke(p, c, spacing=0.25 * r)
                    return n

                run()
                torch.cuda.synchronize()
                t = time.perf_counter()
                n = run()
                torch.cuda.synchronize()
                row[str(cl)] = round(n / (time.perf_counter() - t))
                row["F"] = b.info()[1]
            print(json.dumps(row), flush=True)
    finally:
        if old is None:
            os.environ.pop("PAINTY_STAMP_CLUSTER", None)
        else:
            os.environ["PAINTY_STAMP_CLUSTER"] = old


def _event_ms(torch, fn, reps: int, warm: int = 3) -> float:
    """Average device time of fn() over `reps` calls (CUDA events on the current stream)."""
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def run_texture_paths(pg, torch, cpu: bool = True):
    """The next rows beside the hot path: the texture brush (TextureBrush + Smudge), the GL
    canvas path (TextureBrushGpu strip raster + imprint, GLSL compose and drying step) and
    the lit render (Renderer::render), each with the oracle's CPU time on a sample."""
    from oracle.oracle import Oracle
    from painty_gb300 import workloads

    peak, peak_kind = _peaks()
    rows, cols = 768, 1024
    tex = workloads.stroke_texture(seed=13)
    strokes = workloads.strokes(cols, rows, 40, seed=3)
    out = {}
    o = Oracle() if cpu else None
    # -- TextureBrush: host-synchronous per stroke (the smudge needs the thickness maximum)
    for storage, smudge in (("f32", True), ("f32", False), ("f64", True)):
        c = pg.Canvas(rows, cols, storage)
        b = pg.TextureBrush(tex)
        b.enableSmudge(smudge)
        todo = strokes if storage == "f32" else strokes[:8]
        for s in todo[:2]:
            b.setRadius(s.radius)
            b.dip((s.K, s.S))
            b.paintStroke(s.path, c)
        torch.cuda.synchronize()
        t = time.perf_counter()
        px = 0
        for s in todo:
            b.setRadius(s.radius)
            b.dip((s.K, s.S))
            px += b.paintStroke(s.path, c)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        key = f"texture_brush_{storage}{'_smudge' if smudge else ''}"
        out[key] = {"metric": "strokes/s", "value": round(len(todo) / dt, 2),
                    "painted_mpix_per_s": round(px / dt / 1e6, 3),
                    "ms_per_stroke": round(dt * 1e3 / len(todo), 3)}
    if o is not None:
        oc = o.canvas(rows, cols)
        ob = o.texture_brush(tex)
        t = time.perf_counter()
        px = 0
        for s in strokes[:4]:
            ob.set_radius(s.radius)
            ob.dip(s.K, s.S)
            px += ob.paint_stroke(oc, s.path)
        dt = time.perf_counter() - t
        out["texture_brush_f32_smudge"]["cpu_baseline"] = {
            "value": round(4 / dt, 3), "unit": "strokes/s", "cores": 1, "kind": "port",
            "sample": "the first 4 strokes, painty's TextureBrush + Smudge restated (double)"}
    # -- TextureBrushGpu on the GL canvas path
    gd = pg.TextureBrushDictionary(1)
    rng = np.random.default_rng(0)
    for rc, nr in ((8, 24), (32, 64)):
        for lc, nc in ((400, 400), (1600, 1600)):
            for k in range(3):
                gd.add(rc, lc, rng.random((nr, nc)))
    gstrokes = workloads.strokes(cols, rows, 200, seed=3)
    c = pg.Canvas(rows, cols, "f32")
    gb = pg.TextureBrushGpu(gd)

    def gl_all():
        for s in gstrokes:
            gb.setRadius(s.radius)
            gb.dip((s.K, s.S))
            gb.paintStroke(s.path, c)

    ms = _event_ms(torch, gl_all, 3, warm=1)
    out["gl_texture_brush_f32"] = {"metric": "strokes/s", "value": round(len(gstrokes) / ms * 1e3, 1),
                                   "ms_per_stroke": round(ms / len(gstrokes), 4)}
    if o is not None:
        od = o.texture_dictionary(1)
        rng = np.random.default_rng(0)
        for rc, nr in ((8, 24), (32, 64)):
            for lc, nc in ((400, 400), (1600, 1600)):
                for k in range(3):
                    od.add(rc, lc, rng.random((nr, nc)))
        ogb = o.gpu_texture_brush()
        K4 = np.zeros((rows, cols, 4), np.float32)
        S4 = np.zeros((rows, cols, 4), np.float32)
        t = time.perf_counter()
        for s in gstrokes[:10]:
            ogb.set_radius(s.radius)
            ogb.dip(s.K, s.S)
            ogb.paint_stroke(od, K4, S4, s.path)
        dt = time.perf_counter() - t
        out["gl_texture_brush_f32"]["cpu_baseline"] = {
            "value": round(10 / dt, 2), "unit": "strokes/s", "cores": 1, "kind": "port",
            "sample": "the first 10 strokes, the GL path's shaders restated in float"}
    # -- lit render and the GLSL passes at 4096^2 (inputs above L2)
    n = 4096
    big = pg.Canvas(n, n, "f32")
    g = np.random.default_rng(1)
    big.upload("K", g.uniform(0.01, 5.0, (n, n, 3)).astype(np.float32))
    big.upload("S", g.uniform(0.05, 3.0, (n, n, 3)).astype(np.float32))
    big.upload("V", g.uniform(0, 1, (n, n)).astype(np.float32))
    img = pg.Image(n, n, "f32")
    r = pg.Renderer()
    for key, fn, nbytes in (
            ("render_f32", lambda: r.render(big, img), 32 + 12 + 12),
            ("glsl_compose_f32", lambda: big.getComposedGlsl(img), 32 + 12 + 12),
            ("dry_step_f32", lambda: big.dryStep(0.0), 32 + 12 + 12 + 32)):
        ms = _event_ms(torch, fn, 20)
        gbs = n * n * nbytes / (ms * 1e-3) / 1e9
        out[key] = {"metric": "Mpix/s", "value": round(n * n / ms / 1e3, 1),
                    "ms_per_launch": round(ms, 4),
                    "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak,
                                 "unit": "GB/s", "frac": round(gbs / peak, 3),
                                 "bytes_per_px": nbytes, "peak_kind": peak_kind}}
    if o is not None:
        sr = 64
        oc = o.canvas(sr, n)
        g = np.random.default_rng(2)
        oc.set("K", g.uniform(0.01, 5.0, (sr, n, 3)))
        oc.set("S", g.uniform(0.05, 3.0, (sr, n, 3)))
        oc.set("V", g.uniform(0, 1, (sr, n)))
        t = time.perf_counter()
        oc.render()
        dt = time.perf_counter() - t
        out["render_f32"]["cpu_baseline"] = {
            "value": round(sr * n / dt / 1e6, 3), "unit": "Mpix/s", "cores": 1, "kind": "port",
            "sample": f"{sr} rows x {n} cols, painty's Renderer::render restated (double)"}
    return out


def run_texture_only(args):
    import torch

    import painty_gb300 as pg

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    print(json.dumps(run_texture_paths(pg, torch, cpu=not args.no_cpu)), flush=True)


def run_ours(args):
    import torch

    import painty_gb300 as pg

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    host = generate_stack_device(torch, seed=1 + rank)
    Kh, Sh, Vh, R0h = (host[k].numpy() for k in ("K", "S", "V", "R0"))
    layers = []
    for l in range(LAYERS):
        ly = pg.PaintLayer(ROWS, COLS, "f32")
        ly.upload("K", Kh[l], planar=True)
        ly.upload("S", Sh[l], planar=True)
        ly.upload("V", Vh[l], planar=True)
        layers.append(ly)
    r0 = pg.Image(ROWS, COLS)
    r0.upload(R0h, planar=True)
    out = pg.Image(ROWS, COLS)
    stream = torch.cuda.Stream()
    npix = ROWS * COLS

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident composite
    clocks = ClockSampler(local).__enter__()
    clocks.wait_ready()
    for _ in range(args.warmup):
        pg.compose_layers(layers, r0, out, stream=stream)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    l0 = pg.kernel_launch_count()
    wall0 = time.time()
    if True:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            starts[i].record(stream)
            pg.compose_layers(layers, r0, out, stream=stream)
            ends[i].record(stream)
        t1.record(stream)
        barrier()
    clocks.window = (wall0, time.time())
    time.sleep(0.2)
    clocks.__exit__(None, None, None)
    launches = pg.kernel_launch_count() - l0
    total_ms = t0.elapsed_time(t1)
    per = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = ws * npix * args.steps / (total_ms / 1e3) / 1e6
    kern_ms = float(np.mean(per))
    peak, peak_kind = _peaks()
    achieved = BYTES_PER_PX * npix / (kern_ms / 1e3) / 1e9

    # ---- unfused per-layer composite (the plain composeOnto drop-in), same inputs
    for _ in range(2):
        pg.compose_layers(layers, r0, out, fused=False, stream=stream)
    torch.cuda.synchronize()
    u0 = torch.cuda.Event(enable_timing=True)
    u1 = torch.cuda.Event(enable_timing=True)
    u0.record(stream)
    for _ in range(args.steps):
        pg.compose_layers(layers, r0, out, fused=False, stream=stream)
    u1.record(stream)
    torch.cuda.synchronize()
    unfused_value = npix * args.steps / (u0.elapsed_time(u1) / 1e3) / 1e6

    # ---- end to end through the C ABI with host buffers: painty_compose_layers_host
    # (pinned host stacks in, pinned host image out, transfers pipelined in row bands)
    out_host = torch.empty((3, ROWS, COLS), dtype=torch.float32, pin_memory=True).numpy()

    def e2e_step():
        pg.compose_layers_host(Kh, Sh, Vh, R0h, out=out_host)

    e2e_step()
    barrier()
    e_steps = max(1, min(args.steps, 10))
    tw = time.perf_counter()
    for _ in range(e_steps):
        e2e_step()
    barrier()
    e2e_s = (time.perf_counter() - tw) / e_steps
    link = host_link(torch)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = npix * (28 * LAYERS + 12)
    d2h = npix * 12

    stamps = None
    cpu = None
    precision = composite_precision(pg, torch, Kh, Sh, Vh, R0h, max(3, min(args.steps, 100)))
    batch = None
    serve = None
    prec = None
    if not args.no_stamps:
        batch = {s_: run_batch(pg, torch, s_, args.batch_canvases, args.batch_max_strokes,
                               rank, ws) for s_ in ("f32", "f16")}
    if rank == 0 and not args.no_stamps:
        stamps = run_stamps_config0(pg, torch, cpu=not args.no_cpu)
        serve = run_serving(pg, torch, full_rate=args.serve_rate, full_s=args.serve_seconds)
        prec = run_precision(pg, torch, (Kh, Sh, Vh, R0h))
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(Kh, Sh, Vh, R0h)
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "Mpix/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, generated on the device)",
            "config": _headline_config(ws),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "peak_kind": peak_kind, "traffic": _traffic_from_profile(),
                         "algorithmic_bytes_per_launch": BYTES_PER_PX * npix,
                         "kernel": "km_composite_kernel<float,float,float>",
                         "kernel_ms": round(kern_ms, 4)},
            "e2e": {"value": round(ws * npix / e2e_s / 1e6, 2), "unit": "Mpix/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": round(e2e_s * 1e3, 2),
                    "call": "painty_compose_layers_host (pinned host buffers)",
                    "host_link": link,
                    "link_bound_ms": round(h2d / (link["h2d_gbs"] * 1e9) * 1e3, 2),
                    "frac_of_link_bound": round(h2d / (link["h2d_gbs"] * 1e9) / e2e_s, 3)},
            "gpu_launches": launches,
            "unfused_value": round(unfused_value, 2),
            "clocks": clocks.summary(),
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        line["composite_half_storage"] = precision
        if stamps is not None:
            line["stamps"] = stamps
        if batch is not None:
            line["stamps_batched"] = batch
        if serve is not None:
            line["serving"] = serve
        if prec is not None:
            line["precision"] = prec
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def host_link(torch, nbytes: int = 1 << 30, reps: int = 5):
    """Measured host <-> device copy bandwidth of this machine: one pinned 1 GiB buffer copied
    each way, best of `reps` (GB/s)."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, fn in (("h2d_gbs", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h_gbs", lambda: h.copy_(d, non_blocking=True))):
        best = 1e30
        for _ in range(reps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t)
        out[name] = round(nbytes / best / 1e9, 1)
    del h, d
    return out


def run_stamps_config0(pg, torch, nstrokes: int = 200, cpu: bool = False):
    """1024x768 FP32 canvas, 200 strokes, r ~ U[8,32], spacing 0.25 r, through the C ABI."""
    from painty_gb300 import workloads

    rows, cols = 768, 1024
    strokes = workloads.strokes(cols, rows, nstrokes, seed=3)
    fp = workloads.footprint_image(seed=7)
    r0 = workloads.substrate(rows, cols, seed=5)
    canvas = pg.Canvas(rows, cols, "f32")
    brush = pg.FootprintBrush(strokes[0].radius, fp)
    brush.setPickupRate(0.05)
    brush.setDepositionRate(0.1)

    def step():
        canvas.setBackground(r0)
        n = workloads.paint_config0(canvas, brush, strokes)
        pg.Renderer().compose(canvas).download()
        return n

    step()
    torch.cuda.synchronize()
    t = time.perf_counter()
    l0 = pg.kernel_launch_count()
    n = step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    out = {"metric": "stamps/s", "value": round(n / dt, 1), "unit": "stamps/s",
           "stamps_per_step": n, "ms_per_step": round(dt * 1e3, 2),
           "config": "1024x768 FP32, 200 strokes, r U[8,32], spacing 0.25 r, snapshot on, "
                     "deposit 0.1, pickup 0.05, final composite; through the C ABI",
           "gpu_launches": pg.kernel_launch_count() - l0,
           "roofline": stamp_roofline([(s.radius, pg_stroke_stamps(s.path, s.spacing))
                                       for s in strokes], n, dt, "f32")}
    if cpu:
        # painty's imprint loop restated (double, one core) on the first strokes
        from oracle.oracle import Oracle
        o = Oracle()
        oc = o.canvas(rows, cols)
        oc.set("R0", r0)
        ob = o.brush(strokes[0].radius, fp)
        ob.set_rates(0.05, 0.1)
        t = time.perf_counter()
        ns = 0
        used = 0
        for s in strokes:
            ob.set_radius(s.radius)
            ob.dip(s.K, s.S)
            ns += ob.paint_stroke(oc, s.path, s.spacing)
            used += 1
            if time.perf_counter() - t > 10.0:
                break
        cdt = time.perf_counter() - t
        out["cpu_baseline"] = {"value": round(ns / cdt, 1), "unit": "stamps/s", "cores": 1,
                               "kind": "port",
                               "sample": f"the first {used} strokes ({ns} stamps), painty's "
                                         "FootprintBrush imprint loop restated (double)"}
    return out


def run_batch(pg, torch, storage: str, ncanvas: int, max_strokes, rank: int = 0,
              world: int = 1):
    """The batching workload (config-2 distributions) in one painty_paint_batch launch per GPU;
    with several ranks each paints its share of the canvases (longest-processing-time split
    by estimated work), and the job's rate is all stamps over the slowest rank's time."""
    from painty_gb300 import sharding, workloads

    if ncanvas == 512 and max_strokes is None:
        specs, strokes = config2_workload()
    else:
        specs, strokes = workloads.batch_canvases(ncanvas, seed=2, max_strokes=max_strokes)
    if world > 1:
        work = np.zeros(len(specs))
        for c, path, r, sp, _, _ in strokes:
            work[c] += sharding.stroke_work(path, r, sp)
        mine = sharding.canvas_shard(work, rank, world)
        index = {c: i for i, c in enumerate(mine)}
        specs = [specs[c] for c in mine]
        strokes = [(index[s[0]],) + tuple(s[1:]) for s in strokes if s[0] in index]
    fp = workloads.footprint_image(seed=7)
    canvases, brushes = [], []
    for rows, cols, r0 in specs:
        c = pg.Canvas(rows, cols, storage)
        c.upload("R0", r0)
        b = pg.FootprintBrush(8.0, fp)
        b.setPickupRate(0.05)
        b.setDepositionRate(0.1)
        canvases.append(c)
        brushes.append(b)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    l0 = pg.kernel_launch_count()
    t = time.perf_counter()
    n = pg.paint_batch(canvases, brushes, strokes) if strokes else 0
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    if world > 1:
        import torch.distributed as dist
        v = torch.tensor([dt, float(n)], device="cuda", dtype=torch.float64)
        t_ = v[:1].clone()
        dist.all_reduce(t_, op=dist.ReduceOp.MAX)
        n_ = v[1:].clone()
        dist.all_reduce(n_, op=dist.ReduceOp.SUM)
        dt, n = float(t_.item()), int(n_.item())
    px = sum(r * c for r, c, _ in specs)
    cl, nclusters, cta_threads = pg.batch_last_shape()
    split_cl, split_canvases = pg.batch_last_split()
    per_stroke = [pg_stroke_stamps(np.asarray(s[1]), s[3]) for s in strokes]
    per_canvas = np.zeros(len(specs))
    for s_, k_ in zip(strokes, per_stroke):
        per_canvas[s_[0]] += k_
    roof = stamp_roofline([(s[2], k_) for s, k_ in zip(strokes, per_stroke)], n, dt, storage)
    heavy = int(np.argmax(per_canvas)) if len(per_canvas) else -1
    bound = _dependency_bound(specs, strokes, heavy) if heavy >= 0 else None
    if roof:
        roof["note"] = ("canvases run concurrently, each canvas's stamps in order; the "
                        "heaviest canvas's chain of stamps bounds the launch")
    return {"metric": "stamps/s", "value": round(n / dt, 1), "unit": "stamps/s", "stamps": n,
            "s": round(dt, 3), "storage": storage, "gpu_launches": pg.kernel_launch_count() - l0,
            "roofline": roof,
            "ctas_per_canvas": cl, "clusters": nclusters, "cta_threads": cta_threads,
            "heaviest_canvases_launch": {"ctas_per_canvas": split_cl, "canvases": split_canvases},
            "makespan_s": round(dt, 3),
            "heaviest_canvas_stamps": int(per_canvas.max()) if len(per_canvas) else 0,
            "heaviest_canvas_stamps_per_s": round(float(per_canvas.max()) / dt, 1) if n else 0.0,
            "mean_canvas_stamps": round(float(per_canvas.mean()), 1) if len(per_canvas) else 0.0,
            "heaviest_canvas_dependency_bound": bound,
            "config": f"{ncanvas} canvases (side logU[256,2048], aspect U[0.5,2], "
                      f"{pg_canvas_px(px)}), {len(strokes)} strokes (logU[50,2000] per canvas"
                      f"{'' if max_strokes is None else f', at most {max_strokes}'}), "
                      "r logU[4,64], spacing 0.25 r; one persistent launch"}


def serve_plan(rate: float, seconds: float, seed: int = 4):
    """The serving workload: Poisson arrivals at `rate` req/s for `seconds`; each request a
    canvas of side log-uniform in [512, 4096] (aspect 1) with 1-500 strokes (geometric, mean 60)
    from the plain case's generators (r U[8,32], spacing 0.25 r, Dirichlet(0.3) paints); 30%
    continue a canvas an earlier request created. Returns [(t, continue_index or -1, rows,
    cols, strokes)]."""
    from painty_gb300 import workloads

    rng = np.random.default_rng(seed)
    PK, PS = workloads.pigments()
    n = max(1, int(rng.poisson(rate * seconds)))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    plan = []
    for i in range(n):
        cont = -1
        if i > 0 and rng.random() < 0.30:
            cont = int(rng.integers(0, i))
            while plan[cont][1] >= 0:  # continue the canvas an earlier request created
                cont = plan[cont][1]
            rows, cols = plan[cont][2], plan[cont][3]
        else:
            rows = cols = int(np.exp(rng.uniform(np.log(512), np.log(4096))))
        ns = min(500, int(rng.geometric(1.0 / 60.0)))
        paths = np.stack([rng.uniform(0, cols, (ns, 8)), rng.uniform(0, rows, (ns, 8))], axis=2)
        radii = rng.uniform(8, 32, ns)
        w = rng.dirichlet(np.full(len(PK), 0.3), ns)
        K, S = w @ PK, w @ PS
        strokes = [(paths[j], float(radii[j]), 0.25 * float(radii[j]), K[j], S[j])
                   for j in range(ns)]
        plan.append((float(arrivals[i]), cont, rows, cols, strokes))
    return plan


class _PinnedPool:
    """Pinned host buffers for request results, reused by size class, at most `cap` bytes
    (beyond it a request gets pageable memory)."""

    def __init__(self, torch, cap: int):
        self.torch, self.cap, self.total = torch, cap, 0
        self.free = {}
        import threading
        self.lock = threading.Lock()

    @staticmethod
    def size_class(rows: int, cols: int) -> int:
        step = 1 << 22  # floats: classes of 16 MB
        return (rows * cols * 3 + step - 1) // step * step

    def prewarm(self, plan, rate: float, seconds: float = 2.0):
        """Allocates, before the timed run, the buffers `seconds` of arrivals would hold."""
        counts = {}
        for _, _, rows, cols, _ in plan:
            c = self.size_class(rows, cols)
            counts[c] = counts.get(c, 0) + 1
        n = len(plan)
        for cls, k in sorted(counts.items()):
            want = int(np.ceil(k / n * rate * seconds)) + 1
            have = len(self.free.get(cls, []))
            for _ in range(max(0, want - have)):
                if self.total + 4 * cls > self.cap:
                    return
                self.free.setdefault(cls, []).append(
                    self.torch.empty(cls, dtype=self.torch.float32, pin_memory=True))
                self.total += 4 * cls

    def take(self, rows: int, cols: int):
        n = rows * cols * 3
        cls = self.size_class(rows, cols)
        with self.lock:
            lst = self.free.get(cls)
            if lst:
                t = lst.pop()
            elif self.total + 4 * cls <= self.cap:
                t = self.torch.empty(cls, dtype=self.torch.float32, pin_memory=True)
                self.total += 4 * cls
            else:
                return None, np.empty((rows, cols, 3), dtype=np.float32)
        return (cls, t), t[:n].numpy().reshape(rows, cols, 3)

    def substrate(self, seed: int):
        """One pinned buffer of 4096 x 4096 x 3 substrate values U[0.8, 0.95]."""
        if getattr(self, "_sub", None) is None:
            g = np.random.default_rng(seed)
            t = self.torch.empty(4096 * 4096 * 3, dtype=self.torch.float32, pin_memory=True)
            t.numpy()[:] = g.uniform(0.8, 0.95, 4096 * 4096 * 3).astype(np.float32)
            self._sub = t
        return self._sub.numpy()

    def give(self, key):
        if key is not None:
            with self.lock:
                self.free.setdefault(key[0], []).append(key[1])


_BOUND = {}


def _dependency_bound(specs, strokes, c: int):
    """The heaviest canvas's serial work over its critical path when strokes may overlap in
    time wherever their grown boxes share no 32-pixel tile (painty_gb300.schedule): the most a
    stroke-level scheduler could shorten that canvas's chain."""
    from painty_gb300 import schedule
    key = (id(strokes), c)
    if key not in _BOUND:
        mine = [(x[1], x[2], x[3]) for x in strokes if x[0] == c]
        n, W, C = schedule.canvas_dependency_bound(specs[c][0], specs[c][1], mine, tile=32)
        _BOUND[key] = {"canvas": c, "stamps": n, "tile": 32,
                       "serial_work_over_critical_path": round(W / C, 3) if C else None}
    return _BOUND[key]


def run_serve(pg, torch, rate: float, seconds: float, seed: int = 4, budget_gb: float = 120.0,
              storage: str = "f16", drain_s: float = 60.0, plan=None, pool=None,
              max_outstanding: int = 512):
    """Serving at `rate` req/s for `seconds` (serve_plan): a client thread submits each
    request at its arrival time into a result buffer (pinned, from a bounded pool) and releases
    each canvas after its last request; a consumer thread takes results in completion order and
    returns their buffers. A request arriving while `max_outstanding` are unfinished is shed
    (not submitted; counted), which bounds the host memory of an overloaded run. Requests still
    unfinished `drain_s` after the last arrival are cancelled and counted as unfinished.
    Latency = submit to result in the caller's buffer. New canvases take their substrate from
    one pinned U[0.8, 0.95] buffer (a contiguous prefix per canvas), read in place."""
    import threading

    from painty_gb300 import workloads

    plan = plan if plan is not None else serve_plan(rate, seconds, seed)
    n = len(plan)
    index = {}
    last = {}
    for i, (_, cont, *_r) in enumerate(plan):
        last[cont if cont >= 0 else i] = i
    fp = workloads.footprint_image(seed=7)
    pool = pool if pool is not None else _PinnedPool(torch, 32 << 30)
    substrate = pool.substrate(seed)
    pool.prewarm(plan, rate)
    srv = pg.Server(int(budget_gb * (1 << 30)), fp, storage=storage, step_stamps=65536)
    rids = [None] * n
    cids = [None] * n
    keys = [None] * n
    lat = np.full(n, np.nan)
    stamps_done = [0]
    t0 = time.perf_counter()
    deadline = t0 + seconds + drain_s

    outstanding = [0]
    shed = [0]
    lock = threading.Lock()

    def client():
        for i, (t, cont, rows, cols, strokes) in enumerate(plan):
            dt = t - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            root = cont if cont >= 0 else i
            if (outstanding[0] >= max_outstanding or (cont >= 0 and cids[cont] is None)):
                shed[0] += 1  # over the limit (or its canvas's first request was shed)
                if last[root] == i and cids[root] is not None:
                    srv.release(cids[root])
                continue
            keys[i], out = pool.take(rows, cols)
            with lock:
                outstanding[0] += 1
            if cont >= 0:
                rids[i], cids[i] = srv.submit(strokes, canvas_id=cids[cont], out=out)
            else:
                r0 = substrate[:rows * cols * 3].reshape(rows, cols, 3)
                rids[i], cids[i] = srv.submit(strokes, rows=rows, cols=cols, r0=r0, out=out)
            index[rids[i]] = i
            if last[root] == i:
                srv.release(cids[i])

    def consumer():  # results in completion order: buffers go back as soon as they are filled
        got = 0
        while got < n - shed[0] or th.is_alive():
            left = deadline - time.perf_counter()
            rid = srv.poll(max(0.0, left)) if left > 0 else None
            if rid is None:
                break
            got += 1
            while rid not in index:  # the client records the id right after submit returns
                time.sleep(0.0001)
            i = index[rid]
            try:
                _, l, st = srv.wait(rid, 0.0)
                lat[i] = l
                stamps_done[0] += st
            except pg.PaintyError:
                pass
            pool.give(keys[i])
            with lock:
                outstanding[0] -= 1

    th = threading.Thread(target=client)
    tc = threading.Thread(target=consumer)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))).__enter__()
    w0 = time.time()
    th.start()
    tc.start()
    th.join()
    tc.join()
    wall = time.perf_counter() - t0
    sampler.window = (w0, time.time())
    sampler.__exit__(None, None, None)
    device = sampler.summary()
    unfinished = int(sum(1 for i in range(n) if rids[i] is not None and np.isnan(lat[i])))
    for i in range(n):
        if rids[i] is not None and np.isnan(lat[i]):
            srv.cancel(rids[i])
    stats = srv.stats()
    srv.close()
    done = lat[~np.isnan(lat)]
    offered = sum(
        int(sum(pg_stroke_stamps(p, sp) for p, _, sp, _, _ in strokes)) for *_, strokes in plan)
    out = {"metric": "request latency", "arrival_rate": rate, "arrival_window_s": seconds,
           "requests": n, "completed": int(done.size), "unfinished": unfinished,
           "shed": shed[0], "max_outstanding": max_outstanding,
           "p50_s": round(float(np.percentile(done, 50)), 4) if done.size else None,
           "p99_s": round(float(np.percentile(done, 99)), 4) if done.size else None,
           "throughput_req_s": round(done.size / wall, 2),
           "stamps_per_s": round(stamps_done[0] / wall, 1),
           "offered_stamps_per_s": round(offered / seconds, 1),
           "wall_s": round(wall, 2), "storage": storage, "budget_gb": budget_gb,
           "evictions": stats["evictions"], "restores": stats["restores"],
           "launches": stats["steps"],
           "server_worker_busy_frac": round(stats["worker_busy_us"] / 1e6 / wall, 3),
           "server_worker_ms_per": {
               "new_canvas": round(stats["worker_create_us"] / 1e3 / max(1, stats["submitted"]), 3),
               "stamp_launch": round(stats["worker_launch_us"] / 1e3 / max(1, stats["steps"]), 3),
               "finish_launch": round(stats["worker_finish_us"] / 1e3 / max(1, stats["completed"]), 3)},
           "gpu_util_pct_mean": device.get("gpu_util_pct_mean"),
           "clocks": {k: device.get(k) for k in ("sm_mhz", "sm_max_mhz", "reasons")},
           "peak_resident_gb": round(stats["peak_resident_bytes"] / 2**30, 2),
           "config": "Poisson arrivals; canvas side logU[512,4096]; 1-500 strokes (geometric, "
                     "mean 60), r U[8,32], spacing 0.25 r; 30% continue an earlier canvas; "
                     "composite returned per request into a pinned buffer; canvases released "
                     "after their last request"}
    # sustained: nothing left unfinished and completions kept pace with arrivals
    out["sustained"] = bool(unfinished == 0 and shed[0] == 0 and done.size and
                            out["p99_s"] is not None and out["p99_s"] < 10.0)
    return out


def run_serving(pg, torch, rates=(20.0, 50.0, 100.0, 150.0), sweep_s: float = 10.0,
                full_rate: float = 200.0, full_s: float = 60.0):
    """The stated serving run (full_rate req/s for full_s) and a sweep of lower rates over
    shorter windows; reports the highest sustained rate."""
    pool = _PinnedPool(torch, 32 << 30)
    sweep = [run_serve(pg, torch, r, sweep_s, pool=pool, drain_s=30.0) for r in rates]
    full = run_serve(pg, torch, full_rate, full_s, pool=pool)
    ok = [x["arrival_rate"] for x in sweep + [full] if x["sustained"]]
    full["sweep"] = [{k: x[k] for k in ("arrival_rate", "arrival_window_s", "requests",
                                        "completed", "unfinished", "shed", "p50_s", "p99_s",
                                        "throughput_req_s", "stamps_per_s", "sustained")}
                     for x in sweep]
    full["highest_sustained_rate"] = max(ok) if ok else None
    return full


def pg_stroke_stamps(path, spacing):
    d = np.linalg.norm(np.diff(path, axis=0), axis=1)
    return int(np.sum(np.floor(d / spacing)))


def stamp_roofline(pairs, n_stamps: int, seconds: float, storage: str):
    """Algorithmic bytes of stamping against HBM: a stamp of footprint side s reads and
    writes the K, S, V of s^2 canvas pixels (7 values each way: 56 B per pixel in FP32, 28 B
    in 16-bit storage; the snapshot and pickup map add traffic that stays on chip).
    `pairs` = (radius, approximate stamp count) per stroke, to weight the mean footprint;
    n_stamps is the exact total."""
    import math
    w = sum(c for _, c in pairs)
    if w <= 0 or seconds <= 0:
        return None
    mean_px = sum(c * math.ceil(math.sqrt(2.0) * (2 * math.ceil(r) + 1)) ** 2
                  for r, c in pairs) / w
    per_px = 28 if storage in ("f16", "bf16") else 56
    gbs = n_stamps * mean_px * per_px / seconds / 1e9
    peak, kind = _peaks()
    return {"bound": "latency", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
            "frac": round(gbs / peak, 4), "bytes_per_stamp": round(mean_px * per_px),
            "peak_kind": kind,
            "note": "stamps of a canvas run strictly in order on one CTA cluster; the canvas "
                    "and snapshot stay in L2, so the per-stamp chain, not HBM, bounds it"}


def pg_canvas_px(px):
    return f"{px / 1e6:.0f} Mpx"


def composite_precision(pg, torch, Kh, Sh, Vh, R0h, steps: int):
    """Fused composite with FP16 / BF16 layer storage on the same workload: Mpix/s."""
    out = {}
    npix = ROWS * COLS
    for storage in ("f16", "bf16"):
        layers = []
        for l in range(LAYERS):
            ly = pg.PaintLayer(ROWS, COLS, storage)
            ly.upload("K", Kh[l], planar=True)
            ly.upload("S", Sh[l], planar=True)
            ly.upload("V", Vh[l], planar=True)
            layers.append(ly)
        r0 = pg.Image(ROWS, COLS)
        r0.upload(R0h, planar=True)
        img = pg.Image(ROWS, COLS)
        stream = torch.cuda.Stream()
        for _ in range(3):
            pg.compose_layers(layers, r0, img, stream=stream)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            pg.compose_layers(layers, r0, img, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        bytes_px = 14 * LAYERS + 24
        peak, _ = _peaks()
        gbs = bytes_px * npix / (ms / 1e3) / 1e9
        out[storage] = {"value": round(npix / (ms / 1e3) / 1e6, 2), "unit": "Mpix/s",
                        "kernel_ms": round(ms, 4), "achieved_gbs": round(gbs, 1),
                        "frac": round(gbs / peak, 4), "bytes_per_px": bytes_px}
        del layers
    return out


_CONFIG2 = {}


def config2_workload():
    """The batching workload at its stated size (512 canvases, seed 2), generated once."""
    if "w" not in _CONFIG2:
        from painty_gb300 import workloads
        _CONFIG2["w"] = workloads.batch_canvases(512, seed=2)
    return _CONFIG2["w"]


def _precision_canvases(n: int = 8):
    """The n canvases of the batching workload with at least 1500 strokes and the fewest
    stamps (long stroke chains, radii up to 64), in that order."""
    specs, strokes = config2_workload()
    ns = np.zeros(len(specs), int)
    st = np.zeros(len(specs))
    for c, path, r, sp, _, _ in strokes:
        ns[c] += 1
        st[c] += pg_stroke_stamps(np.asarray(path), sp)
    cand = [c for c in np.argsort(st, kind="stable") if ns[c] >= 1500][:n]
    return [int(c) for c in cand], ns, st


def run_precision(pg, torch, host=None):
    """Reduced-precision storage against the double oracle (painty's CPU path restated, pinned
    bit for bit to painty's own code): CIEDE2000 max / mean and max |dR| of the composed
    reflectance, per storage (FP32, FP16, BF16; all arithmetic FP32).

    composite: the composite-stress workload at its full 4096 x 4096 x 8, against the oracle's
               double composite of the same FP32 inputs (all host threads).
    stamps:    the plain workload in full (1024 x 768, 200 strokes) against the oracle.
    batched:   8 canvases of the batching workload (512-canvas generator) with 1500+ strokes,
               the 8 with the fewest stamps, radii up to 64, one paint_batch per storage; against
               the GPU's F64 mode for all 8 (painty's double arithmetic, bit-exact with the
               oracle in the tests) and against the oracle itself for the 2 smallest -- where the
               F64 mode's equality with the oracle is checked too."""
    import concurrent.futures as cf

    from oracle.oracle import Oracle
    from painty_gb300 import workloads

    o = Oracle()
    cores = os.cpu_count() or 1

    def stats(ref, got):
        de_max, de_mean = o.delta_e(got, ref, threads=cores)
        return {"de_max": round(float(de_max), 4), "de_mean": round(float(de_mean), 5),
                "dr_max": float(f"{np.abs(got - ref).max():.3g}")}

    out = {"reference": "the double oracle (painty's CPU path restated; pinned to painty's own "
                        "code bit for bit)", "target": "max dE2000 < 0.5 (16-bit storage)"}
    fp = workloads.footprint_image(seed=7)
    pool = cf.ThreadPoolExecutor(max_workers=4)

    # -- oracle work on host threads, beside the GPU runs below
    rows0, cols0 = 768, 1024
    strokes0 = workloads.strokes(cols0, rows0, 200, seed=3)
    r0h = workloads.substrate(rows0, cols0, seed=5)

    def oracle_config0():
        oc = o.canvas(rows0, cols0)
        oc.set("R0", r0h)
        ob = o.brush(strokes0[0].radius, fp)
        ob.set_rates(0.05, 0.1)
        for s_ in strokes0:
            ob.set_radius(s_.radius)
            ob.dip(s_.K, s_.S)
            ob.paint_stroke(oc, s_.path, s_.spacing)
        return oc.compose(), {p_: oc.get(p_) for p_ in ("K", "S", "V")}

    specs, strokes = config2_workload()
    pick, ns, st = _precision_canvases(8)
    sub_specs = [specs[c] for c in pick]
    index = {c: i for i, c in enumerate(pick)}
    sub_strokes = [(index[x[0]],) + tuple(x[1:]) for x in strokes if x[0] in index]

    def oracle_canvas(i):
        rows, cols, r0 = sub_specs[i]
        oc = o.canvas(rows, cols)
        oc.set("R0", r0.astype(np.float64))
        ob = o.brush(8.0, fp)
        ob.set_rates(0.05, 0.1)
        for ci, path, r, sp, K, S in sub_strokes:
            if ci == i:
                ob.set_radius(r)
                ob.dip(K, S)
                ob.paint_stroke(oc, path, sp)
        return oc.compose(), {p_: oc.get(p_) for p_ in ("K", "S", "V")}

    t_or = time.perf_counter()
    fut0 = pool.submit(oracle_config0)
    fut_c = [pool.submit(oracle_canvas, i) for i in (0, 1)]

    # -- plain painting, full config 0, on the GPU
    imgs0 = {}
    for stg in ("f32", "f16", "bf16"):
        cv = pg.Canvas(rows0, cols0, stg)
        cv.setBackground(r0h)
        br = pg.FootprintBrush(strokes0[0].radius, fp)
        br.setPickupRate(0.05)
        br.setDepositionRate(0.1)
        workloads.paint_config0(cv, br, strokes0)
        imgs0[stg] = (pg.Renderer().compose(cv).download(),
                      {p_: cv.download(p_) for p_ in ("K", "S", "V")})
        del cv, br

    # -- batched painting of the 8 canvases, every storage
    res = {}
    for stg in ("f64", "f32", "f16", "bf16"):
        cvs, brs = [], []
        for rr, cc, r0 in sub_specs:
            cv = pg.Canvas(rr, cc, stg)
            cv.upload("R0", r0)
            b = pg.FootprintBrush(8.0, fp)
            b.setPickupRate(0.05)
            b.setDepositionRate(0.1)
            cvs.append(cv)
            brs.append(b)
        t = time.perf_counter()
        pg.paint_batch(cvs, brs, sub_strokes)
        torch.cuda.synchronize()
        res[stg] = ([pg.Renderer().compose(cv).download() for cv in cvs],
                    [{p_: cv.download(p_) for p_ in ("K", "S", "V")} for cv in (cvs[:2] if stg == "f64" else [])],
                    time.perf_counter() - t)
        del cvs, brs

    # -- composite: full composite-stress workload, GPU storages vs the oracle
    comp = {}
    if host is not None:
        Kh, Sh, Vh, R0h = host
        R, Cc = R0h.shape[1:]
        ref = o.compose_layers_f32_planar_f64(Kh, Sh, Vh, R0h, threads=cores)
        for stg in ("f32", "f16", "bf16"):
            layers = []
            for l in range(Vh.shape[0]):
                ly = pg.PaintLayer(R, Cc, stg)
                ly.upload("K", Kh[l], planar=True)
                ly.upload("S", Sh[l], planar=True)
                ly.upload("V", Vh[l], planar=True)
                layers.append(ly)
            r0 = pg.Image(R, Cc)
            r0.upload(R0h, planar=True)
            img = pg.Image(R, Cc)
            pg.compose_layers(layers, r0, img)
            comp[stg] = stats(ref, img.download())
            del layers, r0, img
        del ref
        comp["workload"] = (f"{R}x{Cc}, {Vh.shape[0]} layers (composite-stress distributions); "
                            "oracle: painty's ComputeReflectance loop in double, every pixel")
    out["composite"] = comp

    ref0, planes0 = fut0.result()
    out["stamps"] = {stg: stats(ref0, imgs0[stg][0]) for stg in ("f32", "f16", "bf16")}
    rel = max(float((np.abs(imgs0["f32"][1][p_] - planes0[p_]) /
                     np.maximum(np.abs(planes0[p_]), 1.0)).max()) for p_ in ("K", "S", "V"))
    out["stamps"]["f32"]["rel_max_KSV"] = float(f"{rel:.3g}")
    out["stamps"]["workload"] = "1024x768, 200 strokes r U[8,32] (the plain workload, full); oracle: the whole canvas"
    ocs = [f.result() for f in fut_c]
    oracle_s = time.perf_counter() - t_or
    bat = {"canvases": pick, "strokes": [int(ns[c]) for c in pick],
           "stamps": [int(st[c]) for c in pick], "rmax": 64}
    bat["vs_gpu_f64"] = {}
    for stg in ("f32", "f16", "bf16"):
        per = [stats(a, b) for a, b in zip(res["f64"][0], res[stg][0])]
        bat["vs_gpu_f64"][stg] = {"de_max": max(q["de_max"] for q in per),
                                  "de_mean": round(float(np.mean([q["de_mean"] for q in per])), 5),
                                  "dr_max": max(q["dr_max"] for q in per)}
    bat["vs_oracle"] = {"canvases": pick[:2]}
    for stg in ("f32", "f16", "bf16"):
        per = [stats(ocs[i][0], res[stg][0][i]) for i in range(2)]
        bat["vs_oracle"][stg] = {"de_max": max(q["de_max"] for q in per),
                                 "de_mean": round(float(np.mean([q["de_mean"] for q in per])), 5),
                                 "dr_max": max(q["dr_max"] for q in per)}
    bat["vs_oracle"]["gpu_f64_equals_oracle"] = bool(all(
        np.array_equal(res["f64"][1][i][p_], ocs[i][1][p_]) for i in range(2) for p_ in ("K", "S", "V")))
    bat["gpu_s"] = {stg: round(res[stg][2], 2) for stg in res}
    bat["oracle_s"] = round(oracle_s, 1)
    out["batched"] = bat
    pool.shutdown()
    torch.cuda.synchronize()
    return out


def cpu_baseline(Kh, Sh, Vh, R0h, target_s: float = 8.0):
    """painty's composite restated (oracle/), one thread, on a row sample of the workload."""
    from oracle.oracle import Oracle

    o = Oracle()

    def sample(rows):
        K = np.ascontiguousarray(Kh[:, :, :rows])
        S = np.ascontiguousarray(Sh[:, :, :rows])
        V = np.ascontiguousarray(Vh[:, :rows])
        R = np.ascontiguousarray(R0h[:, :rows])
        return K, S, V, R

    K, S, V, R = sample(8)
    t = time.perf_counter()
    o.compose_layers_f32_planar(K, S, V, R, threads=1)
    per_row = (time.perf_counter() - t) / 8
    rows = int(max(8, min(ROWS, target_s / max(per_row, 1e-9))))
    K, S, V, R = sample(rows)
    t = time.perf_counter()
    o.compose_layers_f32_planar(K, S, V, R, threads=1)
    dt = time.perf_counter() - t
    return {"value": round(rows * COLS / dt / 1e6, 4), "unit": "Mpix/s", "cores": 1,
            "kind": "port",
            "sample": f"first {rows} of {ROWS} rows ({rows * COLS} px x {LAYERS} layers), "
                      f"double-precision ComputeReflectance loop, {dt:.1f} s"}


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return
    from oracle.oracle import Oracle

    workloads = _workloads_module()
    o = Oracle()
    cores = os.cpu_count() or 1
    rows = 256  # per step: 256 rows x 4096 cols through all 8 layers
    K, S, V, R0 = workloads.composite_stack(rows, COLS, layers=LAYERS, seed=1)
    for _ in range(args.warmup):
        o.compose_layers_f32_planar(K, S, V, R0, threads=cores)
    t = time.perf_counter()
    for _ in range(args.steps):
        o.compose_layers_f32_planar(K, S, V, R0, threads=cores)
    dt = (time.perf_counter() - t) / args.steps
    value = rows * COLS / dt / 1e6
    sample = (f"{rows} rows x {COLS} cols x {LAYERS} layers per step of the 4096x4096 "
              f"workload, painty's ComputeReflectance loop (double) restated, {cores} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mpix/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": _headline_config(ws),
        "cpu_baseline": {"value": round(value, 3), "unit": "Mpix/s", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--rows", type=int, default=ROWS, help="composite rows (profiling cases)")
    ap.add_argument("--cols", type=int, default=COLS, help="composite cols (profiling cases)")
    ap.add_argument("--no-stamps", action="store_true")
    ap.add_argument("--stamps-only", action="store_true", help="only the stamping case")
    ap.add_argument("--batch-canvases", type=int, default=512,
                    help="canvases in the batched stamping case (the stated workload: 512)")
    ap.add_argument("--batch-max-strokes", type=int, default=None,
                    help="cap on strokes per canvas in the batched stamping case (none: as stated)")
    ap.add_argument("--strokes", type=int, default=200, help="strokes in the stamping case")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cluster-sweep", action="store_true",
                    help="stamps/s by brush radius and stamp cluster size")
    ap.add_argument("--serve-only", action="store_true", help="only the serving case")
    ap.add_argument("--precision-only", action="store_true", help="only the precision case")
    ap.add_argument("--batch-only", action="store_true", help="only the batched stamping case")
    ap.add_argument("--texture-only", action="store_true",
                    help="only the texture brushes, GL canvas path and lit render")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serving arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serving arrival window")
    ap.add_argument("--serve-sweep", action="store_true",
                    help="with --serve-only: the rate sweep before the stated run")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    globals()["ROWS"], globals()["COLS"] = args.rows, args.cols
    if args.impl == "reference":
        run_reference(args)
    elif args.cluster_sweep:
        run_cluster_sweep(args)
    elif args.stamps_only:
        run_stamps_only(args)
    elif args.serve_only:
        run_serve_only(args)
    elif args.precision_only:
        run_precision_only(args)
    elif args.batch_only:
        run_batch_only(args)
    elif args.texture_only:
        run_texture_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
