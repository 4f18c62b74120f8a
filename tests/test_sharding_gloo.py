"""Multi-rank placement (painty_gb300.sharding) exercised by world-size-2 gloo process groups
on the CPU: every canvas and row lands on exactly one rank, the ranks agree on the split, and
the slowest rank's time is what a max all-reduce reports."""
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
