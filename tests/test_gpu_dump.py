"""The debugging dump in the formats of the reference's PPG_DUMP mode
(opencl/pp/pp_gpu.c:415-555): the agent lines reproduce the oracle's state
after every iteration, and the cell lines agree with the agent indices and
the grass countdowns."""
import re
import subprocess

import numpy as np
import pytest

import pphpc_gb300 as pp
from common import params
from oracle import pp_oracle as orc

pytestmark = pytest.mark.gpu

AGENT = re.compile(r"^\[\s*(\d+)\] ([0-9a-f]{16}): \(\s*(\d+),\s*(\d+)\) type=(\d+) energy=(\d+)$")
CELL = re.compile(r"^\((\d+), (\d+)\) -> \((\d+), (\d+)\) (.*)\[Grass: (\d+)\]$")
CELL0 = re.compile(r"^\((\d+), (\d+)\) -> \(-, -\) \[Grass: (\d+)\]$")


def _blocks(path, header):
    blocks, cur = [], None
    for line in open(path).read().split("\n"):
        if line.startswith(header):
            cur = [line]
            blocks.append(cur)
        elif cur is not None and line:
            cur.append(line)
    return blocks


def test_dump_matches_oracle_state(tmp_path):
    p = params(30, 1)
    seed, iters = 11, 6
    fa, fc = str(tmp_path / "dump_agents.txt"), str(tmp_path / "dump_cells.txt")
    o = orc.State(p, seed, capacity=1 << 16)
    want = []
    with pp.Simulation(p, seed, max_agents=1 << 16) as sim:
        for it in range(iters + 1):
            if it:
                sim.step(1)
                o.step()
            sim.dump(fa, fc, 0x00)
            cell, en = o.agents()
            want.append((cell.copy(), en.copy(), o.grass().copy()))
    ab = _blocks(fa, "Iter ")
    cb = _blocks(fc, "Iteration ")
    assert len(ab) == len(cb) == iters + 1
    for it, (cell, en, grass) in enumerate(want):
        label = -1 if it == 0 else it
        assert ab[it][0].startswith("Iter %d," % label)
        assert cb[it][0] == "Iteration %d" % label
        rows = [AGENT.match(l).groups() for l in ab[it][1:]]
        assert len(rows) == len(cell)
        for k, (idx, hexv, x, y, t, e) in enumerate(rows):
            x, y, t, e = int(x), int(y), int(t), int(e)
            assert int(idx) == k
            assert y * p.grid_x + x == cell[k]
            assert t == en[k] >> 31 and e == en[k] & 0x7fffffff
            assert int(hexv, 16) == (x << 48) | (y << 32) | (t << 16) | (e & 0xffff)
        lines = cb[it][1:]
        assert len(lines) == p.grid_x * p.grid_y
        for c, line in enumerate(lines):
            if label == -1:
                x, y, g = map(int, CELL0.match(line).groups())
            else:
                m = CELL.match(line).groups()
                x, y, f, l, g = int(m[0]), int(m[1]), int(m[2]), int(m[3]), int(m[5])
                ks = np.nonzero(cell == c)[0]
                if len(ks):
                    assert (f, l) == (ks[0], ks[-1])
                    assert ("More than 1" in m[4]) == (len(ks) > 1)
                else:
                    assert f == l == (1 << 16)
            assert (x, y) == (c % p.grid_x, c // p.grid_x)
            assert g == grass[c]


def test_cli_dump_only_occupied_cells(tmp_path):
    cfg = tmp_path / "config.txt"
    cfg.write_text("INIT_SHEEP = 40\nSHEEP_GAIN_FROM_FOOD = 4\nSHEEP_REPRODUCE_THRESHOLD = 2\n"
                   "SHEEP_REPRODUCE_PROB = 4\nINIT_WOLVES = 20\nWOLVES_GAIN_FROM_FOOD = 20\n"
                   "WOLVES_REPRODUCE_THRESHOLD = 2\nWOLVES_REPRODUCE_PROB = 5\n"
                   "GRASS_RESTART = 10\nGRID_X = 25\nGRID_Y = 25\nITERS = 4\n")
    r = subprocess.run([pp.CLI_PATH, "-p", str(cfg), "-s", str(tmp_path / "stats.txt"),
                        "-r", "3", "--dump", "0x11"], cwd=str(tmp_path),
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    stats = [l.split("\t") for l in (tmp_path / "stats.txt").read_text().splitlines()]
    ab = _blocks(str(tmp_path / "dump_agents.txt"), "Iter ")
    cb = _blocks(str(tmp_path / "dump_cells.txt"), "Iteration ")
    assert len(ab) == len(cb) == 5
    for it in range(5):
        assert len(ab[it]) - 1 == int(stats[it][0]) + int(stats[it][1])
    # 0x10: only cells holding agents after the first iteration, none at -1
    assert len(cb[0]) == 1
    for it in range(1, 5):
        for line in cb[it][1:]:
            m = CELL.match(line).groups()
            assert int(m[2]) <= int(m[3]) < 1 << 24
