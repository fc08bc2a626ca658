"""Full-size runs against oracle fixtures made on the CPU
(tests/golden/make_golden.py large): the 12800x12800 v1 workload through its
population peak (rows 0..300 and the state after them) and for all 4000
iterations, in both pipelines, and every class of the 64-run batched mix for
all 4000 iterations, plain, batched in the real mix, and served."""
import hashlib
import os

import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params, rows_array, first_diff

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ["init_sheep", "sheep_gain_from_food", "sheep_reproduce_threshold",
          "sheep_reproduce_prob", "init_wolves", "wolves_gain_from_food",
          "wolves_reproduce_threshold", "wolves_reproduce_prob", "grass_restart",
          "grid_x", "grid_y", "iters"]
MIX_FIXTURES = {100: "mix_200v1_s100", 132: "mix_800v2_s132",
                148: "mix_1600v1_s148", 156: "mix_3200v2_s156"}
POOL_FACTOR = 40   # v2 populations peak near 36x their initial agents


def _fixture(name):
    path = os.path.join(GOLDEN, "stats_%s.npz" % name)
    if not os.path.exists(path):
        pytest.fail("missing fixture %s (tests/golden/make_golden.py large)" % path)
    g = np.load(path)
    p = pp.make_params(**dict(zip(FIELDS, (int(x) for x in g["params"]))))
    return g, p, int(g["seed"][0])


def _digest(cell, en, grass):
    h = hashlib.sha256()
    for a in (cell, en, grass):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
def test_12800_through_population_peak(sort_pipeline):
    g, p, seed = _fixture("12800v1_s2_r300")
    want = g["rows"]
    iters = len(want) - 1
    pool = int(g["pool"][0])
    with pp.Simulation(p, seed, max_agents=pool, sort_pipeline=sort_pipeline) as sim:
        got = rows_array([sim.stats0()] + sim.step(iters))
        assert first_diff(got, want) is None
        cell, en, grass = sim.state()
    assert _digest(cell, en, grass) == str(g["state_sha256"])


def _mix(iters=4000):
    runs, seed = [], 100
    for side, v, n in [(200, 1, 32), (800, 2, 16), (1600, 1, 8), (3200, 2, 8)]:
        for _ in range(n):
            runs.append((params(side, v, iters=iters), seed))
            seed += 1
    return runs


def test_mix_classes_alone_full_length():
    for seed, name in MIX_FIXTURES.items():
        g, p, s = _fixture(name)
        assert s == seed
        n0 = p.init_sheep + p.init_wolves
        got = rows_array(pp.run(p, s, max_agents=POOL_FACTOR * n0))
        assert first_diff(got, g["rows"]) is None, name


def test_real_64_run_mix_against_oracle():
    """The 64-run mix of 4000 iterations in one batched world: the first run
    of each class equals the oracle's rows."""
    runs = _mix()
    out = pp.batch_run(runs, pool_factor=POOL_FACTOR)
    for k, (p, seed) in enumerate(runs):
        if seed in MIX_FIXTURES:
            g, pf, s = _fixture(MIX_FIXTURES[seed])
            assert (pf.grid_x, pf.sheep_gain_from_food) == (p.grid_x, p.sheep_gain_from_food)
            assert first_diff(rows_array(out[k]), g["rows"]) is None, MIX_FIXTURES[seed]


def test_served_world_holds_mix_classes():
    """One served world holds the four classes and a few other runs arriving
    later; each class's rows equal the oracle's."""
    srv = pp.Server(mem_budget_bytes=48 << 30, max_runs=16, pool_factor=POOL_FACTOR,
                    stats_chunk=64)
    ids = {}
    for seed, name in MIX_FIXTURES.items():
        g, p, s = _fixture(name)
        ids[srv.submit(p, s)] = g["rows"]
    extra = []
    for _ in range(200):
        q, r = srv.load()
        if q == 0 and r == 0:
            break
        srv.poll(64)
        if len(extra) < 4:
            p = params(300 + 100 * len(extra), 1 + len(extra) % 2, iters=500)
            extra.append(srv.submit(p, 900 + len(extra)))
    for rid, want in ids.items():
        ev = srv.status(rid)
        assert ev.done == 1 and ev.status == 0
        assert first_diff(rows_array(srv.read(rid)), want) is None, rid
    srv.close()


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
def test_12800_full_run_rows(sort_pipeline):
    """The 12800x12800 v1 workload (seed 2, pool 5x) against every row the
    oracle's full-length fixture holds (all 4000 iterations, or the first
    rows of an interrupted generation), in both iteration pipelines."""
    path = os.path.join(GOLDEN, "stats_12800v1_s2_full.npz")
    if not os.path.exists(path):
        pytest.skip("full-length fixture not generated (make_golden.py large)")
    g, p, seed = _fixture("12800v1_s2_full")
    want = g["rows"]
    k = int(g["iters_done"][0])
    assert len(want) == k + 1 and k >= 500
    got = rows_array(pp.run(p, seed, k, max_agents=int(g["pool"][0]),
                            sort_pipeline=sort_pipeline))
    assert first_diff(got, want) is None
