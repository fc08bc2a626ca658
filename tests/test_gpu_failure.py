"""Failure detection without a GPU fault: a device-side wait whose flag
nothing sets gives up after a bounded number of polls, the host reads
PP_ERR_TIMEOUT, and the device stays usable for the next launches."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from common import first_diff, params, rows_array
from oracle import pp_oracle as orc

pytestmark = pytest.mark.gpu


def test_lookback_prefixes():
    n = 300
    got = pp.lookback_selftest(n)
    k = np.arange(n, dtype=np.uint64)
    assert np.array_equal(got.astype(np.uint64), k * (k + 1) // 2)


@pytest.mark.parametrize("stall", [0, 37, 298])
def test_stalled_wait_times_out_and_device_stays_usable(stall):
    """Chunk `stall` never publishes; the chunk after it waits on a flag
    nothing sets."""
    with pytest.raises(pp.PPError) as ei:
        pp.lookback_selftest(300, stall_chunk=stall)
    assert ei.value.code == pp.PP_ERR_TIMEOUT
    # the context is intact: the self-test and a simulation run again
    got = pp.lookback_selftest(64)
    assert int(got[-1]) == 63 * 64 // 2
    p = params(50, 1, iters=40)
    assert first_diff(rows_array(pp.run(p, 3)), orc.run(p, 3)) is None
