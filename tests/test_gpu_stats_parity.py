"""Statistical parity of the CUDA path with the CPU restatement of the
reference's pp_cpu algorithm: 30 GPU replications (one batched world)
against 30 CPU replications, PPHPC focal measures, alpha = 0.05
family-wise (Holm)."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params
from focal import compare, focal_measures, format_table
from oracle import cpu_port

pytestmark = pytest.mark.gpu

REPS = 30
SS_FROM = 1000


def _gpu_fms(p, seeds, pool_factor):
    out = pp.batch_run([(p, s) for s in seeds], pool_factor=pool_factor)
    return np.array([focal_measures(np.array([r.as_tuple() for r in rows], np.uint64),
                                    p.grid_x * p.grid_y, SS_FROM) for rows in out])


def _port_fms(p, seeds):
    with ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))) as ex:
        runs = list(ex.map(lambda s: cpu_port.run(p, s, nthreads=1), seeds))
    return np.array([focal_measures(r, p.grid_x * p.grid_y, SS_FROM) for r in runs])


@pytest.mark.parametrize("side,version,pool_factor", [(100, 1, 8), (200, 2, 40), (400, 2, 40)])
def test_gpu_vs_cpu_algorithm(side, version, pool_factor):
    p = params(side, version, iters=4000)
    a = _gpu_fms(p, range(REPS), pool_factor)
    b = _port_fms(p, range(7000, 7000 + REPS))
    ok, table = compare(a, b)
    print("\n%dx%d v%d\n" % (side, side, version) + format_table(table))
    assert ok, format_table(table)
