"""The reference's own CPU kernels (opencl/pp/pp_cpu.cl, compiled unmodified
by oracle/ref/build_ref.py and driven by a restatement of the reference
host's launch loop): invariants of its runs, independence from the host
thread count, and the work sizes of pp_cpu.c:232-325."""
import numpy as np
import pytest

from common import params
from oracle import pp_ref

pytestmark = pytest.mark.skipif(not pp_ref.available(),
                                reason="reference kernels unavailable")


def test_worksizes_follow_the_reference_host():
    # max gws = rows / 3; rows per work item rows / gws, plus one when the
    # remainder allows it (pp_cpu.c:245-322)
    for rows in (3, 4, 10, 100, 101, 400, 12800):
        gws, rpw = pp_ref.worksizes(rows)
        assert gws == rows // 3
        r = rows // gws
        if rows % gws and (gws - 1) * (r + 1) < rows - 3:
            r += 1
        assert rpw == r
        # every row is covered by exactly one (work item, turn) pair
        covered = set()
        for g in range(gws):
            for t in range(rpw):
                y = t + g * rpw
                if y < rows:
                    last = g == gws - 1 and t == rpw - 1
                    covered.update(range(y, rows) if last else [y])
        assert covered == set(range(rows)), rows
    with pytest.raises(ValueError):
        pp_ref.worksizes(2)


@pytest.mark.parametrize("side,version,seed", [(100, 1, 0), (60, 2, 4)])
def test_thread_count_does_not_change_the_run(side, version, seed):
    p = params(side, version, iters=400)
    a = pp_ref.run_raw(p, seed, threads=1)
    b = pp_ref.run_raw(p, seed, threads=4)
    c = pp_ref.run_raw(p, seed, threads=0)
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_row0_and_bookkeeping():
    p = params(100, 1, iters=300)
    r = pp_ref.run_raw(p, 3)
    assert r[0, 0] == p.init_sheep and r[0, 1] == p.init_wolves
    cells = p.grid_x * p.grid_y
    assert np.all(r[:, 2] <= cells)
    # mean initial energy: uniform in [1, 2 gain]
    assert abs(r[0, 3] / r[0, 0] - (1 + 2 * 4) / 2) < 0.5
    assert abs(r[0, 4] / r[0, 1] - (1 + 2 * 20) / 2) < 2.5
    # countdowns are at most the restart value
    assert np.all(r[:, 5] <= 10 * (cells - r[:, 2]))
    assert not r[:, 6].any()
    # different seeds give different runs
    assert not np.array_equal(r, pp_ref.run_raw(p, 4))


def test_too_many_initial_agents_is_refused():
    p = params(50, 1, iters=5)
    with pytest.raises(RuntimeError):
        pp_ref.run_raw(p, 0, max_agents=p.init_sheep + p.init_wolves - 1)


def test_sim_steps_equal_a_whole_run():
    p = params(80, 2, iters=120)
    whole = pp_ref.run_raw(p, 9)
    s = pp_ref.Sim(p, 9, 120)
    rows = [s.row(0)] + list(s.step(50)) + list(s.step(70))
    s.close()
    assert np.array_equal(np.array(rows), whole)
