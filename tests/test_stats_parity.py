"""Statistical parity of the oracle's rules (which the CUDA path reproduces
bit for bit) with the CPU restatement of the reference's pp_cpu algorithm
(shuffled, sequential in-cell actions, its own RNG): 30 replications each,
PPHPC focal measures, alpha = 0.05 family-wise (Holm)."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np

from common import params
from focal import compare, focal_measures, format_table
from oracle import cpu_port
from oracle import pp_oracle as orc

REPS = 30
SS_FROM = 1000


def _pool():
    return ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))


def _port_fms(p, seeds):
    with _pool() as ex:
        runs = list(ex.map(lambda s: cpu_port.run(p, s, nthreads=1), seeds))
    return np.array([focal_measures(r, p.grid_x * p.grid_y, SS_FROM) for r in runs])


def _oracle_fms(p, seeds):
    with _pool() as ex:
        runs = list(ex.map(lambda s: orc.run(p, s), seeds))
    return np.array([focal_measures(r, p.grid_x * p.grid_y, SS_FROM) for r in runs])


def test_oracle_vs_cpu_algorithm_100v1():
    p = params(100, 1, iters=4000)
    a = _oracle_fms(p, range(REPS))
    b = _port_fms(p, range(5000, 5000 + REPS))
    ok, table = compare(a, b)
    print("\n" + format_table(table))
    assert ok, format_table(table)


def test_comparison_detects_a_changed_parameter():
    """Power check: the same comparison tells v1 from v1 with a sheep gain
    of 5 instead of 4."""
    p = params(100, 1, iters=2000)
    q = params(100, 1, iters=2000)
    q.sheep_gain_from_food = 5
    a = _port_fms(p, range(REPS))
    b = _port_fms(q, range(100, 100 + REPS))
    ok, table = compare(a, b)
    assert not ok
    assert sum(t[4] < 0.05 for t in table) >= 6
