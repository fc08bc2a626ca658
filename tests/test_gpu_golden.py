"""Full-length runs of the benchmark configurations on the GPU against the
committed golden fixtures (oracle output), the command-line drop-in, and
the 12800x12800 configuration against the oracle and size-independent
properties."""
import os
import subprocess

import numpy as np
import pytest

import pphpc_gb300 as pp
from oracle import pp_oracle as orc
from common import rows_array, first_diff

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ["init_sheep", "sheep_gain_from_food", "sheep_reproduce_threshold",
          "sheep_reproduce_prob", "init_wolves", "wolves_gain_from_food",
          "wolves_reproduce_threshold", "wolves_reproduce_prob", "grass_restart",
          "grid_x", "grid_y", "iters"]


@pytest.mark.parametrize("cfg,seed,fixture", [("config100v1", 0, "stats_100v1_s0"),
                                              ("config400v2", 1, "stats_400v2_s1")])
def test_config_full_length(cfg, seed, fixture):
    p = pp.load_params(os.path.join(GOLDEN, cfg + ".txt"))
    want = np.load(os.path.join(GOLDEN, fixture + ".npz"))["rows"]
    got = rows_array(pp.run(p, seed))
    d = first_diff(got, want)
    assert d is None, d


def test_small_fixtures():
    g = np.load(os.path.join(GOLDEN, "stats_small.npz"))
    for n in [k for k in g.files if not k.endswith(("_params", "_seed"))]:
        d = dict(zip(FIELDS, (int(x) for x in g[n + "_params"])))
        p = pp.make_params(**d)
        got = rows_array(pp.run(p, int(g[n + "_seed"][0]), len(g[n]) - 1))
        assert first_diff(got, g[n]) is None, n


def test_cli_stats_file(tmp_path):
    out = tmp_path / "stats.txt"
    r = subprocess.run([pp.CLI_PATH, "-p", os.path.join(GOLDEN, "config100v1.txt"),
                        "-s", str(out), "-r", "0"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    want = np.load(os.path.join(GOLDEN, "stats_100v1_s0.npz"))["rows"]
    lines = out.read_text().splitlines()
    assert len(lines) == 4001
    for i in range(0, 4001, 50):
        r_ = want[i]
        s = pp.PPStatistics(int(r_[0]), int(r_[1]), int(r_[2]), int(r_[3]),
                            int(r_[4]), int(r_[5]))
        assert lines[i] == pp.format_row(s, p), i


def test_cli_iters_and_pool_limit(tmp_path):
    out = tmp_path / "s.txt"
    cfg = os.path.join(GOLDEN, "config400v2.txt")
    r = subprocess.run([pp.CLI_PATH, "-p", cfg, "-s", str(out), "-r", "1",
                        "--iters", "300", "-m", "2000"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == pp.PP_OUT_OF_RESOURCES & 0xff
    r = subprocess.run([pp.CLI_PATH, "-p", cfg, "-s", str(out), "-r", "1",
                        "--iters", "300"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0
    assert len(out.read_text().splitlines()) == 301


def test_12800_first_iterations_bit_exact():
    p = pp.load_params(os.path.join(GOLDEN, "config12800v1.txt"))
    cap = 5 * (p.init_sheep + p.init_wolves)  # v1 transient peaks at 4.25x
    st = orc.State(p, 2, capacity=cap)
    want = [st.stats()] + [st.step() for _ in range(2)]
    st.close()
    got = rows_array(pp.run(p, 2, 2, max_agents=cap))
    assert first_diff(got, np.array(want, np.uint64)) is None


def test_12800_properties_long():
    """Size-independent checks at full size: determinism across runs and
    graph/no-graph launch modes, population bookkeeping, grass bounds."""
    p = pp.load_params(os.path.join(GOLDEN, "config12800v1.txt"))
    cap = 5 * (p.init_sheep + p.init_wolves)  # v1 transient peaks at 4.25x
    a = rows_array(pp.run(p, 2, 200, max_agents=cap))
    b = rows_array(pp.run(p, 2, 200, max_agents=cap, use_graph=False))
    assert np.array_equal(a, b)
    cells = p.grid_x * p.grid_y
    assert np.all(a[:, 2] <= cells) and np.all(a[:, 5] <= 10 * cells)
    assert np.all(a[:, 3] >= a[:, 0]) and np.all(a[:, 4] >= a[:, 1])
    assert a[-1][0] > 0 and a[-1][1] > 0
