"""Snapshot and resume: a simulation saved after some iterations and
restored from the file continues with exactly the stats and state of the
uninterrupted simulation (every draw is keyed by cell, iteration and rank,
none by memory layout), in both iteration pipelines."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params, rows_array

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
@pytest.mark.parametrize("side,version,seed,before,after", [
    (50, 1, 4, 70, 80), (64, 2, 9, 40, 60), (120, 1, 2, 33, 50)])
def test_restore_continues_bit_exact(tmp_path, sort_pipeline, side, version, seed,
                                     before, after):
    p = params(side, version)
    kw = dict(max_agents=1 << 20, sort_pipeline=sort_pipeline)
    with pp.Simulation(p, seed, **kw) as sim:
        straight = rows_array([sim.stats0()] + sim.step(before + after))
        cell_s, en_s, grass_s = sim.state()
    path = str(tmp_path / "snap.bin")
    with pp.Simulation(p, seed, **kw) as sim:
        sim.step(before)
        sim.save(path)
    with pp.Simulation.restore(path, p, **kw) as sim:
        assert sim.info()[0] == before
        resumed = rows_array([sim.stats0()] + sim.step(after))
        assert sim.info()[0] == before + after
        cell_r, en_r, grass_r = sim.state()
    assert np.array_equal(resumed, straight[before:])
    assert np.array_equal(cell_r, cell_s) and np.array_equal(en_r, en_s)
    assert np.array_equal(grass_r, grass_s)


def test_restore_rejects_other_files(tmp_path):
    bad = tmp_path / "not_a_snapshot.bin"
    bad.write_bytes(b"hello world" * 10)
    with pytest.raises(pp.PPError) as ei:
        pp.Simulation.restore(str(bad), params(20, 1))
    assert ei.value.code == pp.PP_INVALID_PARAMS_FILE
