"""Continuous-batching server (painty_server_*) on the GPU."""
import threading
import time

import numpy as np
import pytest

from painty_gb300 import workloads

pytestmark = pytest.mark.gpu


def _strokes(rng, rows, cols, n, rmin=2.0, rmax=12.0):
    out = []
    for _ in range(n):
        path = np.stack([rng.uniform(0, cols, 6), rng.uniform(0, rows, 6)], axis=1)
        r = float(np.exp(rng.uniform(np.log(rmin), np.log(rmax))))
        out.append((path, r, 0.25 * r, rng.uniform(0.01, 5, 3), rng.uniform(0.05, 3, 3)))
    return out


def _request_set(seed, n):
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(n):
        rows, cols = int(rng.integers(40, 200)), int(rng.integers(40, 200))
        reqs.append((rows, cols, rng.uniform(0.8, 0.95, (rows, cols, 3)).astype(np.float32),
                     _strokes(rng, rows, cols, int(rng.integers(1, 12)))))
    return reqs


@pytest.mark.parametrize("storage", ["f16", "f32"])
def test_result_same_alone_and_in_the_mix(pg, storage):
    fp = workloads.footprint_image(seed=7)
    reqs = _request_set(3, 24)
    target = 5
    rows, cols, r0, strokes = reqs[target]
    alone = pg.Server(8 << 30, fp, storage=storage, step_stamps=2000)
    rid, _ = alone.submit(strokes, rows=rows, cols=cols, r0=r0)
    a_img, _, a_st = alone.wait(rid, 60)
    alone.close()
    # the same request among others, submitted from two client threads while others run
    mix = pg.Server(8 << 30, fp, storage=storage, step_stamps=2000)
    ids = {}

    def client(idx):
        for i in idx:
            rr, cc, r0_, st_ = reqs[i]
            ids[i] = mix.submit(st_, rows=rr, cols=cc, r0=r0_)[0]
            time.sleep(0.002)

    t1 = threading.Thread(target=client, args=(range(0, 24, 2),))
    t2 = threading.Thread(target=client, args=(range(1, 24, 2),))
    t1.start(); t2.start(); t1.join(); t2.join()
    results = {i: mix.wait(ids[i], 120) for i in ids}
    s = mix.stats()
    mix.close()
    m_img, _, m_st = results[target]
    assert m_st == a_st
    assert np.array_equal(a_img, m_img)
    assert s["completed"] == 24 and s["failed"] == 0
    assert s["steps"] >= 24  # every request launched at least one chunk of strokes
    # everything came from the server's device reservation
    assert s["heap_bytes"] >= 8 << 30 and s["heap_fallbacks"] == 0


def test_heap_reuses_released_memory(pg):
    """Canvases of mixed sizes created and released one after another, many times over a
    small budget: the reservation's freed ranges are merged and reused, never exceeded, and
    each result equals the same request on a fresh server."""
    fp = workloads.footprint_image(seed=7)
    rng = np.random.default_rng(11)
    srv = pg.Server(96 << 20, fp, storage="f16", step_stamps=4000)
    first = None
    for i in range(40):
        side = int(rng.choice([96, 160, 300, 480]))
        st = _strokes(np.random.default_rng(100 + i), side, side, 2)
        rid, cid = srv.submit(st, rows=side, cols=side)
        img, _, _ = srv.wait(rid, 60)
        srv.release(cid)
        if i == 0:
            first = (side, st, img)
    s = srv.stats()
    srv.close()
    assert s["completed"] == 40 and s["failed"] == 0 and s["heap_fallbacks"] == 0
    side, st, img = first
    fresh = pg.Server(96 << 20, fp, storage="f16", step_stamps=4000)
    again, _, _ = fresh.wait(fresh.submit(st, rows=side, cols=side)[0], 60)
    fresh.close()
    assert np.array_equal(img, again)


def test_continuation_matches_batch_painting(pg):
    fp = workloads.footprint_image(seed=7)
    rng = np.random.default_rng(8)
    rows, cols = 90, 130
    r0 = rng.uniform(0.8, 0.95, (rows, cols, 3)).astype(np.float32)
    parts = [_strokes(rng, rows, cols, 4), _strokes(rng, rows, cols, 3), _strokes(rng, rows, cols, 5)]
    srv = pg.Server(4 << 30, fp, storage="f64", step_stamps=1500)
    rid, cid = srv.submit(parts[0], rows=rows, cols=cols, r0=r0)
    rids = [rid] + [srv.submit(p, canvas_id=cid)[0] for p in parts[1:]]  # queued behind it
    imgs = [srv.wait(r, 60)[0] for r in rids]
    srv.close()
    # the same strokes through painty_paint_batch on one canvas
    c = pg.Canvas(rows, cols, "f64")
    c.upload("R0", r0.astype(np.float64))
    b = pg.FootprintBrush(8.0, fp)
    b.setPickupRate(0.05)
    b.setDepositionRate(0.1)
    for p in parts:
        pg.paint_batch([c], [b], [(0,) + s for s in p])
    want = pg.Renderer().compose(c).download(dtype=np.float32)
    assert np.array_equal(imgs[-1], want)


def test_eviction_victim_is_not_admitted_in_the_same_round(pg):
    """Three canvases over a budget that holds two, their continuations queued behind each
    other: admitting a new canvas evicts an idle one whose next request is also waiting. That
    request must wait for a later round (and a restore), not paint the canvas being evicted.
    Results equal those of a server that never evicts."""
    fp = workloads.footprint_image(seed=7)
    rng = np.random.default_rng(31)
    side = 300
    rounds = [[_strokes(rng, side, side, 3) for _ in range(3)] for _ in range(4)]
    r0 = rng.uniform(0.8, 0.95, (side, side, 3)).astype(np.float32)

    def run(budget):
        srv = pg.Server(budget, fp, storage="f16", step_stamps=20000)
        cids, rids = [None] * 3, []
        for rnd in rounds:
            for k in range(3):
                if cids[k] is None:
                    rid, cids[k] = srv.submit(rnd[k], rows=side, cols=side, r0=r0)
                else:
                    rid, _ = srv.submit(rnd[k], canvas_id=cids[k])
                rids.append(rid)
        imgs = [srv.wait(r, 120)[0] for r in rids]
        st = srv.stats()
        srv.close()
        return imgs, st

    tight, st = run(20 << 20)  # two of these canvases fit
    roomy, _ = run(4 << 30)
    assert st["evictions"] > 0 and st["restores"] > 0 and st["failed"] == 0, st
    for a, b in zip(tight, roomy):
        assert np.array_equal(a, b)


def test_eviction_and_restore_keep_results(pg):
    fp = workloads.footprint_image(seed=7)
    reqs = _request_set(11, 10)
    base = pg.Server(8 << 30, fp, storage="f16", step_stamps=4000)
    cids, rids = [], []
    for rows, cols, r0, st in reqs:
        r, c = base.submit(st, rows=rows, cols=cols, r0=r0)
        rids.append(r)
        cids.append(c)
    first = [base.wait(r, 60)[0] for r in rids]
    more = [_strokes(np.random.default_rng(99 + i), reqs[i][0], reqs[i][1], 3) for i in range(10)]
    again = [base.wait(base.submit(more[i], canvas_id=cids[i])[0], 60)[0] for i in range(10)]
    base.close()
    # a budget for about three canvases: continuing the others needs evictions and restores
    per = max(rr * cc for rr, cc, _, _ in reqs) * 60 + (4 << 20)
    tight = pg.Server(3 * per, fp, storage="f16", step_stamps=4000, max_active=3)
    cids2, rids2 = [], []
    for rows, cols, r0, st in reqs:
        r, c = tight.submit(st, rows=rows, cols=cols, r0=r0)
        rids2.append(r)
        cids2.append(c)
    first2 = [tight.wait(r, 60)[0] for r in rids2]
    again2 = [tight.wait(tight.submit(more[i], canvas_id=cids2[i])[0], 60)[0] for i in range(10)]
    s = tight.stats()
    tight.close()
    assert s["evictions"] > 0 and s["restores"] > 0
    assert s["peak_resident_bytes"] <= 3 * per
    for a, b in zip(first + again, first2 + again2):
        assert np.array_equal(a, b)


def test_rejections_and_cancellation(pg):
    fp = workloads.footprint_image(seed=7)
    srv = pg.Server(64 << 20, fp, storage="f32", step_stamps=500, max_active=1)
    rng = np.random.default_rng(2)
    big, _ = srv.submit(_strokes(rng, 3000, 3000, 1), rows=3000, cols=3000)
    with pytest.raises(RuntimeError, match="budget"):
        srv.wait(big, 30)
    with pytest.raises(ValueError):
        srv.submit([], canvas_id=12345)
    slow, cid = srv.submit(_strokes(rng, 150, 150, 40, 8, 20), rows=150, cols=150)
    queued, _ = srv.submit(_strokes(rng, 150, 150, 2), canvas_id=cid)
    srv.cancel(queued)
    with pytest.raises(RuntimeError, match="cancel"):
        srv.wait(queued, 60)
    srv.wait(slow, 120)
    s = srv.stats()
    assert s["failed"] == 1 and s["cancelled"] == 1 and s["completed"] == 1
    srv.submit(_strokes(rng, 150, 150, 200, 8, 20), canvas_id=cid)
    srv.close()  # the unfinished request ends cancelled; close returns


def test_release_frees_canvases_and_pinned_results(pg):
    """painty_server_release drops a canvas after its queued requests; results land in the
    caller's pinned buffers and equal those of pageable ones."""
    torch = pytest.importorskip("torch")
    fp = workloads.footprint_image(seed=7)
    reqs = _request_set(21, 3)
    srv = pg.Server(8 << 30, fp, storage="f16", step_stamps=3000)
    outs, rids, cids = [], [], []
    for rows, cols, r0, st in reqs:
        out = torch.empty((rows, cols, 3), dtype=torch.float32, pin_memory=True).numpy()
        r, c = srv.submit(st, rows=rows, cols=cols, r0=r0, out=out)
        outs.append(out)
        rids.append(r)
        cids.append(c)
    extra, _ = srv.submit(_strokes(np.random.default_rng(5), reqs[0][0], reqs[0][1], 3),
                          canvas_id=cids[0])
    srv.release(cids[0])  # after its two queued requests
    srv.release(cids[1])
    for r in rids + [extra]:
        srv.wait(r, 60)
    for _ in range(200):  # the worker frees released canvases on its next round
        s = srv.stats()
        if s["canvases"] == 1 and s["resident_bytes"] < s["peak_resident_bytes"]:
            break
        time.sleep(0.01)
    assert s["canvases"] == 1 and s["completed"] == 4
    with pytest.raises(ValueError):
        srv.submit(_strokes(np.random.default_rng(6), 20, 20, 1), canvas_id=cids[1])
    srv.close()
    # the same first requests with pageable results
    ref = pg.Server(8 << 30, fp, storage="f16", step_stamps=3000)
    for (rows, cols, r0, st), out in zip(reqs, outs):
        img, _, _ = ref.wait(ref.submit(st, rows=rows, cols=cols, r0=r0)[0], 60)
        assert np.array_equal(img, out)
    ref.close()


def test_poll_returns_each_request_once_in_completion_order(pg):
    fp = workloads.footprint_image(seed=7)
    reqs = _request_set(31, 6)
    srv = pg.Server(8 << 30, fp, storage="f32", step_stamps=5000)
    ids = [srv.submit(st, rows=rr, cols=cc, r0=r0)[0] for rr, cc, r0, st in reqs]
    seen = [srv.poll(60.0) for _ in ids]
    assert sorted(seen) == sorted(ids)
    assert srv.poll(0.05) is None
    for rid in ids:  # finished: waiting returns at once
        srv.wait(rid, 0.0)
    srv.close()
