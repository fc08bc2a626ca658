"""The -a/--agent-size mode without a GPU: the oracle's modular energy
arithmetic (pp_gpu.cl:150-316, move pp_gpu.cl:805-810) and the argument
checks of the library and the command line, which return before any device
work."""
import os
import subprocess

import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params
from oracle import pp_oracle as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

WRAP11 = dict(sheep_gain_from_food=700, sheep_reproduce_threshold=1500,
              sheep_reproduce_prob=20, wolves_gain_from_food=1500,
              wolves_reproduce_threshold=1800, wolves_reproduce_prob=10,
              grass_restart=10)


def test_oracle_move_is_modular():
    """Energy 1 dies; energy 0 (a wrapped gain) survives with the field
    maximum, as PPG_AG_ENERGY_SUB then the zero test do."""
    p = params(16, 1)
    cell = np.array([5, 5, 9, 100], np.uint32)
    en = np.array([0, 1, 2, 2047 | 0x80000000], np.uint32)
    co, eo = orc.move(p, 7, 1, cell, en, energy_bits=11)
    dead = p.grid_x * p.grid_y
    assert co[1] == dead and all(co[i] != dead for i in (0, 2, 3))
    assert list(eo & 0x7fffffff)[0::2] == [2047, 1] and eo[3] == (2046 | 0x80000000)
    co, eo = orc.move(p, 7, 1, cell, en, energy_bits=16)
    assert eo[0] == 65535 and co[1] == dead
    # the wide field: energy 0 cannot arise, the rule is unchanged at >= 1
    co, eo = orc.move(p, 7, 1, cell[1:], en[1:])
    assert co[0] == dead and list(eo[1:] & 0x7fffffff) == [1, 2046]


def test_oracle_gains_wrap_and_zero_energy_agents_live():
    p = pp.make_params(init_sheep=680, init_wolves=340, grid_x=64, grid_y=64,
                       iters=150, **WRAP11)
    st = orc.State(p, 3, energy_bits=11)
    zeros = 0
    for _ in range(150):
        st.step()
        _, en = st.agents()
        e = en & 0x7fffffff
        assert e.max(initial=0) <= 2047
        zeros += int((e == 0).sum())
    st.close()
    assert zeros > 0


def test_library_rejects_agent_sizes():
    p = params(16, 1)
    for bad in (1, 16, 48, 128):
        with pytest.raises(pp.PPError) as ei:
            pp.Simulation(p, 1, agent_size=bad)
        assert ei.value.code == pp.PP_INVALID_ARGS
        with pytest.raises(pp.PPError) as ei:
            pp.batch_run([(p, 1)], agent_size=bad)
        assert ei.value.code == pp.PP_INVALID_ARGS
        with pytest.raises(pp.PPError) as ei:
            pp.Server(agent_size=bad)
        assert ei.value.code == pp.PP_INVALID_ARGS
    # 32-bit agents hold 10-bit coordinates
    for gx, gy in [(1025, 8), (8, 1025)]:
        with pytest.raises(pp.PPError) as ei:
            pp.Simulation(params(0, 1, gx=gx, gy=gy), 1, agent_size=32)
        assert ei.value.code == pp.PP_INVALID_ARGS


def _cli(*args):
    return subprocess.run([pp.CLI_PATH] + list(args), stdout=subprocess.PIPE,
                          stderr=subprocess.PIPE, text=True)


def test_cli_agent_size_argument(tmp_path):
    r = _cli("-a", "48", "-p", os.path.join(GOLDEN, "config100v1.txt"))
    assert r.returncode == pp.PP_INVALID_ARGS & 0xff
    assert "must be either 32 or 64" in r.stderr
    txt = open(os.path.join(GOLDEN, "config100v1.txt")).read().replace(
        "GRID_X = 100", "GRID_X = 2000")
    f = tmp_path / "wide.txt"
    f.write_text(txt)
    r = _cli("--agent-size", "32", "-p", str(f), "-s", str(tmp_path / "s.txt"))
    assert r.returncode == pp.PP_INVALID_ARGS & 0xff
    assert "-a 64" in r.stderr


def test_cli_accepts_the_references_opencl_options():
    """OpenCL tuning options of the reference parse (with a note) and have no
    effect: the run goes on to the agent-size check."""
    r = _cli("--a-sort", "s-bitonic", "--a-sort-opts", "lws=64", "--a-rng", "lcg",
             "--l-def", "64", "--vw-grass", "4", "-c", "-cl-fast-relaxed-math",
             "-a", "48", "-p", os.path.join(GOLDEN, "config100v1.txt"))
    assert r.returncode == pp.PP_INVALID_ARGS & 0xff
    assert "--a-sort has no effect" in r.stderr and "-c/--compiler" in r.stderr
