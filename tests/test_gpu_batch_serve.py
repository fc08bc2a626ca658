"""Batched and served runs: each run's stats in the mix are identical to
the same run alone (and to the oracle)."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from oracle import pp_oracle as orc
from common import params, rows_array, first_diff

pytestmark = pytest.mark.gpu


def _mix(n):
    runs = []
    sides = [20, 33, 50, 64, 100]
    for i in range(n):
        p = params(sides[i % len(sides)], 1 + (i % 2), iters=60 + 17 * (i % 5))
        runs.append((p, 100 + i))
    return runs


def test_batch_equals_alone_and_oracle():
    runs = _mix(12)
    out = pp.batch_run(runs, pool_factor=40)
    for (p, seed), rows in zip(runs, out):
        alone = rows_array(pp.run(p, seed))
        got = rows_array(rows)
        assert first_diff(got, alone) is None, (p.grid_x, seed)
        assert first_diff(got, orc.run(p, seed)) is None


@pytest.mark.parametrize("tile", [1024, 4096])
def test_batch_tile_sizes(tile):
    runs = _mix(6)
    out = pp.batch_run(runs, pool_factor=40, tile_cells=tile, use_graph=False)
    for (p, seed), rows in zip(runs, out):
        assert first_diff(rows_array(rows), orc.run(p, seed)) is None


def test_batch_64_mixed_sizes_short():
    runs = []
    for i in range(64):
        side, v = [(200, 1), (800, 2), (1600, 1), (3200, 2)][i * 4 // 64]
        runs.append((params(side, v, iters=5), 100 + i))
    out = pp.batch_run(runs, pool_factor=40)
    for k in (0, 31, 32, 47, 48, 63):
        p, seed = runs[k]
        assert first_diff(rows_array(out[k]), rows_array(pp.run(p, seed))) is None


def test_serve_alone_equals_mix():
    srv = pp.Server(mem_budget_bytes=2 << 30, max_runs=8, stats_chunk=16)
    reqs = _mix(10)
    ids = []
    # staggered arrivals: submit a few, advance, submit more
    for i, (p, seed) in enumerate(reqs):
        ids.append(srv.submit(p, seed))
        if i % 3 == 2:
            srv.poll(7)
    for _ in range(200):
        q, r = srv.load()
        if q == 0 and r == 0:
            break
        srv.poll(16)
    assert sorted(srv.finished()) == sorted(ids) and srv.finished() == []
    for rid, (p, seed) in zip(ids, reqs):
        ev = srv.status(rid)
        assert ev.done == 1 and ev.status == 0
        rows = rows_array(srv.read(rid))
        assert len(rows) == p.iters + 1
        assert first_diff(rows, orc.run(p, seed)) is None, rid
        srv.release(rid)
    srv.close()


def test_serve_admission_waits_for_memory_and_slots():
    srv = pp.Server(mem_budget_bytes=256 << 20, max_runs=2, stats_chunk=8)
    reqs = [(params(60, 1, iters=40), 7 + i) for i in range(5)]
    ids = [srv.submit(p, s) for p, s in reqs]
    srv.poll(8)
    q, r = srv.load()
    assert r <= 2 and q >= 3
    for _ in range(100):
        q, r = srv.load()
        if q == 0 and r == 0:
            break
        srv.poll(8)
    for rid, (p, s) in zip(ids, reqs):
        assert srv.status(rid).done == 1
        assert first_diff(rows_array(srv.read(rid)), orc.run(p, s)) is None
    srv.close()


def test_serve_cancel():
    srv = pp.Server(mem_budget_bytes=512 << 20, max_runs=4, stats_chunk=8)
    a = srv.submit(params(40, 1, iters=100), 1)
    b = srv.submit(params(40, 2, iters=50), 2)
    srv.poll(8)
    srv.cancel(a)
    ev = srv.status(a)
    assert ev.done == 1 and ev.status == pp.PP_ERR_CANCELLED
    for _ in range(20):
        srv.poll(8)
    assert srv.status(b).done == 1
    assert first_diff(rows_array(srv.read(b)), orc.run(params(40, 2, iters=50), 2)) is None
    srv.close()


def test_serve_rejects_oversized():
    srv = pp.Server(mem_budget_bytes=64 << 20, max_runs=2)
    with pytest.raises(pp.PPError) as e:
        srv.submit(params(3200, 2, iters=10), 1)
    assert e.value.code == pp.PP_OUT_OF_RESOURCES
    srv.close()


@pytest.mark.parametrize("tile", [512, 2048])
def test_serve_tile_sizes(tile):
    """The server's tile size option gives the same results as the oracle."""
    srv = pp.Server(mem_budget_bytes=1 << 30, max_runs=4, stats_chunk=16,
                    tile_cells=tile)
    reqs = [(params(s, v, iters=60), 70 + i)
            for i, (s, v) in enumerate([(90, 2), (41, 1), (300, 1)])]
    ids = [srv.submit(p, seed) for p, seed in reqs]
    for _ in range(100):
        q, r = srv.load()
        if q == 0 and r == 0:
            break
        srv.poll(16)
    for rid, (p, seed) in zip(ids, reqs):
        assert srv.status(rid).done == 1
        assert first_diff(rows_array(srv.read(rid)), orc.run(p, seed)) is None
    srv.close()
    with pytest.raises(pp.PPError):
        pp.Server(tile_cells=4096)
