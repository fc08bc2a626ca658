"""Focal measures computed on the GPU as the iterations run (pp_sim_focal,
pp_serve_focal) equal those computed on the host from the stats rows
(tests/focal.py): extrema and their iterations exactly, steady-state mean
and standard deviation to 1e-9 relative."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params, rows_array
from focal import focal_measures

pytestmark = pytest.mark.gpu


def _check(got, rows, cells, ss_from):
    want = focal_measures(rows, cells, ss_from)
    assert np.array_equal(got[:, :4], want[:, :4]), (got[:, :4], want[:, :4])
    np.testing.assert_allclose(got[:, 4:], want[:, 4:], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
@pytest.mark.parametrize("side,version,seed,iters,ss_from", [
    (100, 1, 0, 600, 200), (64, 2, 3, 300, 100)])
def test_sim_focal_measures(sort_pipeline, side, version, seed, iters, ss_from):
    p = params(side, version)
    with pp.Simulation(p, seed, sort_pipeline=sort_pipeline, ss_from=ss_from) as sim:
        rows = rows_array([sim.stats0()] + sim.step(iters))
        got = sim.focal().as_array()
        assert sim.focal().ss_n == iters - ss_from
    _check(got, rows, p.grid_x * p.grid_y, ss_from)


def test_serve_focal_measures():
    srv = pp.Server(mem_budget_bytes=2 << 30, max_runs=4, stats_chunk=32, ss_from=50)
    reqs = [(params(40, 1, iters=150), 5), (params(60, 2, iters=120), 6),
            (params(30, 1, iters=90), 7)]
    ids = [srv.submit(p, s) for p, s in reqs]
    for _ in range(100):
        srv.poll(16)
        if all(srv.status(i).done for i in ids):
            break
    for rid, (p, s) in zip(ids, reqs):
        assert srv.status(rid).status == 0
        rows = rows_array(srv.read(rid))
        _check(srv.focal(rid).as_array(), rows, p.grid_x * p.grid_y, 50)
    srv.close()
