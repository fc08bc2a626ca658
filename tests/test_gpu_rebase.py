"""Runs past the grass re-base. A cell's grass is stored as the 16-bit
iteration at which it is alive again, and every 8192 world iterations a
sweep moves the regrowth iteration of every alive cell up to the current
iteration so that the 16-bit differences never wrap. The reference keeps a
plain countdown (opencl/pp/pp_gpu.cl:448-476), so this sweep is new; these
tests run plain, served and restored worlds across it and compare every
stats row with the oracle."""
import pytest

import pphpc_gb300 as pp
from oracle import pp_oracle as orc
from common import params, rows_array, first_diff

pytestmark = pytest.mark.gpu

REBASE = 8192   # world iterations between re-basing sweeps


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
@pytest.mark.parametrize("side,version,seed", [
    (40, 1, 0),     # both species alive throughout
    (50, 2, 2),     # the wolves die out near iteration 1600
    (40, 2, 1),     # extinct by iteration 270: every cell alive for 8000+
])
def test_plain_run_crosses_rebase(sort_pipeline, side, version, seed):
    p = params(side, version, iters=REBASE + 300)
    want = orc.run(p, seed)
    got = rows_array(pp.run(p, seed, sort_pipeline=sort_pipeline, max_agents=1 << 17))
    assert first_diff(got, want) is None


def test_graph_and_chunks_across_rebase():
    """Stepping in uneven chunks that straddle the re-base, with and without
    CUDA graphs, gives the oracle's rows."""
    p = params(40, 1, iters=REBASE + 200)
    want = orc.run(p, 3)
    for use_graph in (True, False):
        with pp.Simulation(p, 3, max_agents=1 << 17, use_graph=use_graph) as sim:
            rows = [sim.stats0()]
            for n in (4000, 4100, 91, 2, 1, 6, 192):     # 8392 in all
                rows += sim.step(n)
        assert first_diff(rows_array(rows), want) is None, use_graph


def test_served_runs_cross_rebase_mid_flight():
    """A served world runs for more than 8192 iterations while runs come and
    go: one run spans the whole stream, one is admitted near world iteration
    5000 and crosses the re-base at its own iteration ~3200, one is admitted
    after the re-base."""
    srv = pp.Server(mem_budget_bytes=1 << 30, max_runs=4, stats_chunk=64)
    reqs = {}
    a = params(40, 1, iters=REBASE + 700)
    reqs[srv.submit(a, 11)] = (a, 11)
    done = 0
    late = [(5000, params(50, 2, iters=4000), 12), (REBASE + 100, params(30, 1, iters=400), 13)]
    while True:
        while late and done >= late[0][0]:
            _, p, s = late.pop(0)
            reqs[srv.submit(p, s)] = (p, s)
        q, r = srv.load()
        if q == 0 and r == 0 and not late:
            break
        srv.poll(250)
        done += 250
    assert done > REBASE + 400
    for rid, (p, s) in reqs.items():
        ev = srv.status(rid)
        assert ev.done == 1 and ev.status == 0, rid
        got = rows_array(srv.read(rid))
        assert first_diff(got, orc.run(p, s)) is None, (rid, p.grid_x)
    srv.close()


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
@pytest.mark.parametrize("before", [REBASE - 150, REBASE + 60])
def test_snapshot_across_rebase(tmp_path, sort_pipeline, before):
    """Saved just before (or just after) the first re-base and restored into
    a new world, the run continues with the oracle's rows."""
    p = params(40, 1, iters=REBASE + 400)
    want = orc.run(p, 21)
    path = str(tmp_path / "snap.bin")
    kw = dict(max_agents=1 << 17, sort_pipeline=sort_pipeline)
    with pp.Simulation(p, 21, **kw) as sim:
        first = rows_array([sim.stats0()] + sim.step(before))
        sim.save(path)
    assert first_diff(first, want[:before + 1]) is None
    with pp.Simulation.restore(path, p, **kw) as sim:
        assert sim.info()[0] == before
        resumed = rows_array([sim.stats0()] + sim.step(p.iters - before))
    assert first_diff(resumed, want[before:]) is None
