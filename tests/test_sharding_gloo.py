"""Multi-rank placement (painty_gb300.sharding) exercised by world-size-2 gloo process groups
on the CPU: every canvas and row lands on exactly one rank, the ranks agree on the split, the
slowest rank's time is what a max all-reduce reports, and sharded work gathered from the ranks
equals the unsharded result bit for bit (each rank computing its share through the oracle)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from painty_gb300 import sharding


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, work, rows, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = sharding.canvas_shard(work, rank, world)
    lo, hi = sharding.row_shard(rows, rank, world)
    # gather every rank's canvases and row band
    got = [None] * world
    dist.all_gather_object(got, (mine, lo, hi, float(np.sum(np.asarray(work)[mine]))))
    t = torch.tensor([1.0 + rank])  # stand-in per-rank time: the slowest rank is reported
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((got, float(t.item())))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_canvas_and_row_shards_gloo(world):
    rng = np.random.default_rng(3)
    work = list(np.exp(rng.uniform(0, 5, 37)))
    rows = 4097
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, work, rows, q)) for r in range(world)]
    for p in procs:
        p.start()
    got, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    canvases = sorted(i for m, _, _, _ in got for i in m)
    assert canvases == list(range(len(work)))  # each canvas exactly once
    bands = sorted((lo, hi) for _, lo, hi, _ in got)
    assert bands[0][0] == 0 and bands[-1][1] == rows
    assert all(bands[i][1] == bands[i + 1][0] for i in range(len(bands) - 1))
    loads = [w for *_, w in got]
    assert max(loads) <= sum(work) / world + max(work) + 1e-9  # LPT bound
    assert tmax == float(world)


def test_shard_arguments():
    with pytest.raises(ValueError):
        sharding.canvas_shard([1.0], 2, 2)
    with pytest.raises(ValueError):
        sharding.row_shard(10, -1, 2)
    assert sharding.canvas_shard([], 0, 3) == []
    assert sharding.row_shard(10, 0, 1) == (0, 10)


def _shard_inputs():
    from painty_gb300 import workloads
    K, S, V, R0 = workloads.composite_stack(37, 29, layers=4, seed=9)
    specs, strokes = workloads.batch_canvases(5, seed=4, smin=40, smax=90, strokes_min=2,
                                              strokes_max=5, rmin=2.0, rmax=9.0)
    return (K, S, V, R0), specs, strokes


def _paint_canvas(o, spec, strokes, ci):
    from painty_gb300 import workloads
    rows, cols, r0 = spec
    oc = o.canvas(rows, cols)
    oc.set("R0", r0.astype(np.float64))
    ob = o.brush(8.0, workloads.footprint_image(seed=7))
    ob.set_rates(0.05, 0.1)
    for c, path, r, sp, K, S in strokes:
        if c == ci:
            ob.set_radius(r)
            ob.dip(K, S)
            ob.paint_stroke(oc, path, sp)
    return oc.compose()


def _compute_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import Oracle
    o = Oracle()
    (K, S, V, R0), specs, strokes = _shard_inputs()
    # composite: this rank's row band
    lo, hi = sharding.row_shard(R0.shape[1], rank, world)
    band = o.compose_layers_f32_planar_f64(K[:, :, lo:hi], S[:, :, lo:hi], V[:, lo:hi],
                                           R0[:, lo:hi])
    # painting: this rank's canvases (work estimated per stroke, split by LPT)
    work = np.zeros(len(specs))
    for c, path, r, sp, _, _ in strokes:
        work[c] += sharding.stroke_work(path, r, sp)
    mine = sharding.canvas_shard(work, rank, world)
    painted = {ci: _paint_canvas(o, specs[ci], strokes, ci) for ci in mine}
    got = [None] * world
    dist.all_gather_object(got, ((lo, hi, band), painted))
    if rank == 0:
        out.put(got)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_work_equals_unsharded_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_compute_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    from oracle.oracle import Oracle
    o = Oracle()
    (K, S, V, R0), specs, strokes = _shard_inputs()
    whole = o.compose_layers_f32_planar_f64(K, S, V, R0)
    bands = sorted((lo, hi, band) for (lo, hi, band), _ in got)
    assert all(b[2].shape[0] == b[1] - b[0] for b in bands)
    assert np.array_equal(np.concatenate([b[2] for b in bands]), whole)
    painted = {}
    for _, part in got:
        assert not set(part) & set(painted)  # each canvas on one rank
        painted.update(part)
    assert sorted(painted) == list(range(len(specs)))
    for ci in range(len(specs)):
        assert np.array_equal(painted[ci], _paint_canvas(o, specs[ci], strokes, ci)), ci
