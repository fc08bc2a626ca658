"""Statistical parity of the CUDA path with the reference's own CPU
algorithm (opencl/pp/pp_cpu.cl compiled unmodified, on all host threads;
only its RNG is a stand-in): 30 GPU replications (one batched world) against
30 CPU replications, PPHPC focal measures of the six outputs, alpha = 0.05
family-wise (Holm), with the count of uncorrected p < 0.05 reported."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params
from focal import compare, focal_measures, format_table, raw_below
from oracle import pp_ref

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not pp_ref.available(),
                                 reason="reference kernels unavailable")]

REPS = 30
SS_FROM = 1000


def _gpu_fms(p, seeds, pool_factor):
    out = pp.batch_run([(p, s) for s in seeds], pool_factor=pool_factor)
    return np.array([focal_measures(np.array([r.as_tuple() for r in rows], np.uint64),
                                    p.grid_x * p.grid_y, SS_FROM) for rows in out])


def _ref_fms(p, seeds):
    return np.array([focal_measures(pp_ref.run(p, s), p.grid_x * p.grid_y, SS_FROM)
                     for s in seeds])


@pytest.mark.parametrize("side,version,pool_factor", [
    (100, 1, 8), (200, 2, 40), (400, 2, 40), (800, 1, 8)])
def test_gpu_vs_reference_cpu(side, version, pool_factor):
    p = params(side, version, iters=4000)
    a = _gpu_fms(p, range(REPS), pool_factor)
    b = _ref_fms(p, range(7000, 7000 + REPS))
    ok, table = compare(a, b)
    print("\n%dx%d v%d\n" % (side, side, version) + format_table(table))
    assert ok, format_table(table)
    assert raw_below(table) <= 8, format_table(table)
