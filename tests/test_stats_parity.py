"""Statistical parity of the oracle's rules (which the CUDA path reproduces
bit for bit) with the reference's own CPU algorithm (opencl/pp/pp_cpu.cl,
compiled unmodified; only its RNG is a stand-in): 30 replications each,
PPHPC focal measures, alpha = 0.05 family-wise (Holm), and power checks
that the same comparison tells a changed sheep or wolf parameter apart."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np
import pytest

from common import params
from focal import compare, focal_measures, format_table, raw_below
from oracle import pp_oracle as orc
from oracle import pp_ref

pytestmark = pytest.mark.skipif(not pp_ref.available(),
                                reason="reference kernels unavailable")

REPS = 30
SS_FROM = 1000


def _ref_fms(p, seeds):
    return np.array([focal_measures(pp_ref.run(p, s), p.grid_x * p.grid_y, SS_FROM)
                     for s in seeds])


def _oracle_fms(p, seeds):
    with ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))) as ex:
        runs = list(ex.map(lambda s: orc.run(p, s), seeds))
    return np.array([focal_measures(r, p.grid_x * p.grid_y, SS_FROM) for r in runs])


def test_oracle_vs_reference_cpu_100v1():
    p = params(100, 1, iters=4000)
    a = _oracle_fms(p, range(REPS))
    b = _ref_fms(p, range(5000, 5000 + REPS))
    ok, table = compare(a, b)
    print("\n" + format_table(table))
    assert ok, format_table(table)
    assert raw_below(table) <= 8, format_table(table)


@pytest.mark.parametrize("field,value", [("sheep_gain_from_food", 5),
                                         ("wolves_reproduce_prob", 6)])
def test_comparison_detects_a_changed_parameter(field, value):
    """Power checks: the same comparison tells v1 from v1 with a sheep gain
    of 5 instead of 4, or a wolf reproduction probability of 6% instead of
    5%."""
    p = params(100, 1, iters=2000)
    q = params(100, 1, iters=2000)
    setattr(q, field, value)
    a = _ref_fms(p, range(REPS))
    b = _ref_fms(q, range(100, 100 + REPS))
    ok, table = compare(a, b)
    print("\n%s = %d\n" % (field, value) + format_table(table))
    assert not ok
    assert raw_below(table) >= 6
