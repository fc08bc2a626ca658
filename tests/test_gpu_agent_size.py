"""The reference's -a/--agent-size mode (pp_gpu.c:334, 1632-1634; packed
agents pp_gpu.cl:150-316) on the GPU: the energy field is 16 bits wide for
64-bit agents and 11 bits for 32-bit ones, gains and the move's decrement
are modulo that width, and an agent dies when the decrement leaves 0.
Parameters with gains near the field width make energies wrap (an agent
can reach energy 0 and come back at the field maximum after its next
move); stats and final state must equal the oracle's at the same width, in
both iteration pipelines, batched, served, through a snapshot and through
the command line."""
import os
import subprocess

import numpy as np
import pytest

import pphpc_gb300 as pp
from common import first_diff, rows_array
from oracle import pp_oracle as orc

pytestmark = pytest.mark.gpu

# gains and thresholds close to the field maxima (2047 and 65535)
WRAP11 = dict(sheep_gain_from_food=700, sheep_reproduce_threshold=1500,
              sheep_reproduce_prob=20, wolves_gain_from_food=1500,
              wolves_reproduce_threshold=1800, wolves_reproduce_prob=10,
              grass_restart=10)
WRAP16 = dict(sheep_gain_from_food=20000, sheep_reproduce_threshold=50000,
              sheep_reproduce_prob=20, wolves_gain_from_food=45000,
              wolves_reproduce_threshold=60000, wolves_reproduce_prob=10,
              grass_restart=10)
BITS = {32: 11, 64: 16}


def wrap_params(gains, side=64, iters=150, gy=None):
    gy = side if gy is None else gy
    return pp.make_params(init_sheep=side * gy // 6, init_wolves=side * gy // 12,
                          grid_x=side, grid_y=gy, iters=iters, **gains)


def _oracle_state(p, seed, bits, iters):
    st = orc.State(p, seed, energy_bits=bits)
    for _ in range(iters):
        st.step()
    cell, en = st.agents()
    grass = st.grass()
    st.close()
    return cell, en, grass


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
@pytest.mark.parametrize("agent_size,gains", [(32, WRAP11), (64, WRAP16)],
                         ids=["a32", "a64"])
def test_modular_energy_matches_oracle(sort_pipeline, agent_size, gains):
    p = wrap_params(gains)
    bits = BITS[agent_size]
    want = orc.run(p, 5, energy_bits=bits)
    # the width matters for these parameters
    assert first_diff(want, orc.run(p, 5)) is not None
    with pp.Simulation(p, 5, agent_size=agent_size, sort_pipeline=sort_pipeline,
                       max_agents=1 << 18) as sim:
        got = rows_array([sim.stats0()] + sim.step(p.iters))
        cell, en, grass = sim.state()
    assert first_diff(got, want) is None
    c, e, g = _oracle_state(p, 5, bits, p.iters)
    assert np.array_equal(cell, c) and np.array_equal(en, e)
    assert np.array_equal(grass, g)


@pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])
def test_largest_grid_of_32_bit_agents(sort_pipeline):
    """1024 x 1024, the largest grid 10-bit coordinates hold."""
    p = wrap_params(WRAP11, side=1024, iters=12)
    with pp.Simulation(p, 8, agent_size=32, sort_pipeline=sort_pipeline) as sim:
        got = rows_array([sim.stats0()] + sim.step(p.iters))
    assert first_diff(got, orc.run(p, 8, energy_bits=11)) is None


def test_agent_size_batched_and_served():
    runs = [(wrap_params(WRAP11, side=s, gy=gy, iters=it), seed)
            for s, gy, it, seed in [(64, 64, 120, 1), (200, 90, 80, 2),
                                    (33, 47, 150, 3), (512, 512, 20, 4)]]
    out = pp.batch_run(runs, pool_factor=8, agent_size=32)
    for (p, seed), rows in zip(runs, out):
        assert first_diff(rows_array(rows), orc.run(p, seed, energy_bits=11)) is None
    srv = pp.Server(mem_budget_bytes=1 << 30, max_runs=4, stats_chunk=16,
                    agent_size=32)
    ids = [srv.submit(p, seed) for p, seed in runs]
    for _ in range(400):
        q, r = srv.load()
        if q == 0 and r == 0:
            break
        srv.poll(16)
    for rid, (p, seed) in zip(ids, runs):
        ev = srv.status(rid)
        assert ev.done == 1 and ev.status == 0
        assert first_diff(rows_array(srv.read(rid)),
                          orc.run(p, seed, energy_bits=11)) is None
        srv.release(rid)
    srv.close()


def test_snapshot_keeps_agent_size(tmp_path):
    """The snapshot records the agent size: a restore without it continues
    with the saved width."""
    p = wrap_params(WRAP11, iters=120)
    path = str(tmp_path / "a32.snap")
    with pp.Simulation(p, 6, agent_size=32, max_agents=1 << 18) as sim:
        sim.step(50)
        sim.save(path)
    with pp.Simulation.restore(path, p, max_agents=1 << 18) as sim:
        resumed = rows_array([sim.stats0()] + sim.step(70))
    assert first_diff(resumed, orc.run(p, 6, energy_bits=11)[50:]) is None


def test_cli_agent_size_32(tmp_path):
    p = wrap_params(WRAP11, iters=100)
    cfg = tmp_path / "wrap.txt"
    cfg.write_text("".join("%s = %d\n" % kv for kv in [
        ("INIT_SHEEP", p.init_sheep),
        ("SHEEP_GAIN_FROM_FOOD", p.sheep_gain_from_food),
        ("SHEEP_REPRODUCE_THRESHOLD", p.sheep_reproduce_threshold),
        ("SHEEP_REPRODUCE_PROB", p.sheep_reproduce_prob),
        ("INIT_WOLVES", p.init_wolves),
        ("WOLVES_GAIN_FROM_FOOD", p.wolves_gain_from_food),
        ("WOLVES_REPRODUCE_THRESHOLD", p.wolves_reproduce_threshold),
        ("WOLVES_REPRODUCE_PROB", p.wolves_reproduce_prob),
        ("GRASS_RESTART", p.grass_restart),
        ("GRID_X", p.grid_x), ("GRID_Y", p.grid_y), ("ITERS", p.iters)]))
    want = orc.run(p, 3, energy_bits=11)
    for args, rows in [(["-a", "32"], want), ([], orc.run(p, 3, energy_bits=16))]:
        out = tmp_path / "stats.txt"
        r = subprocess.run([pp.CLI_PATH, "-p", str(cfg), "-s", str(out), "-r", "3"]
                           + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                           text=True)
        assert r.returncode == 0, r.stderr
        lines = out.read_text().splitlines()
        assert len(lines) == p.iters + 1
        for i in range(0, p.iters + 1, 7):
            w = rows[i]
            s = pp.PPStatistics(int(w[0]), int(w[1]), int(w[2]), int(w[3]),
                                int(w[4]), int(w[5]))
            assert lines[i] == pp.format_row(s, p), (args, i)
    assert first_diff(want, orc.run(p, 3, energy_bits=16)) is not None
