"""Autotuner: it returns one of the candidate geometries, caches it, and a
tuned simulation or batch gives the same stats as the oracle (the geometry
never changes results)."""
import pytest

import pphpc_gb300 as pp
from oracle import pp_oracle as orc
from common import params, rows_array, first_diff

pytestmark = pytest.mark.gpu


def test_autotune_returns_a_candidate_and_caches():
    p = params(300, 2, iters=200)
    t1 = pp.autotune(p, 5)
    assert t1["tile_cells"] in (512, 1024, 2048, 4096, 8192)
    assert t1["tile_cells"] >= 1024 or t1["sort_pipeline"] == 0
    assert t1["ns_per_agent_step"] > 0
    t2 = pp.autotune(p, 5)
    assert t2 == t1


def test_tuned_simulation_is_bit_exact():
    p = params(120, 1, iters=150)
    got = rows_array(pp.run(p, 9, autotune=True))
    assert first_diff(got, orc.run(p, 9)) is None


def test_tuned_batch_is_bit_exact():
    runs = [(params(s, v, iters=80), 40 + i)
            for i, (s, v) in enumerate([(40, 1), (64, 2), (100, 1), (33, 2)])]
    out = pp.batch_run(runs, pool_factor=40, autotune=True)
    for (p, seed), rows in zip(runs, out):
        assert first_diff(rows_array(rows), orc.run(p, seed)) is None
