"""The CUDA path evaluates a cell's actions in closed form, one thread per
agent (act_agent in pphpc_gb300/csrc/pp_act.cuh: the k-th wolf eats the k-th
sheep; a sheep acts iff the wolves before it are no more than the sheep
before it; the first acting sheep takes live grass). The oracle runs the
reference's literal sequential scan of the cell's list instead
(opencl/pp/pp_cpu.cl:690-848: each wolf walks the list for the first sheep
still in it and removes it; an eaten sheep is skipped at its turn). This
test compiles the closed form for the host and checks that both agree on
random cells of 0 to 12 agents, with priority ties, energy wrap and every
mix of types. No GPU is used."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle import pp_oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "helpers", "act_closed_form.cu")
LIB = os.path.join(ROOT, "tests", "helpers", "_build", "libact_closed_form.so")
CSRC = os.path.join(ROOT, "pphpc_gb300", "csrc")

TYPE_BIT = 0x80000000
EATEN_BIT = 0x40000000
KID_BIT = 0x40000000
_u32p = C.POINTER(C.c_uint32)


def _lib():
    from pphpc_gb300 import build as b
    deps = [SRC, os.path.join(CSRC, "pp_act.cuh"), os.path.join(CSRC, "pp_device.cuh")]
    if (not os.path.exists(LIB) or not b.native_ok(LIB)
            or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps)):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        subprocess.run([b.NVCC, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC",
                        "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                        SRC, "-o", LIB], check=True)
    L = C.CDLL(LIB)
    L.act_cells_closed_form.argtypes = [_u32p, C.c_uint32] + [_u32p] * 8
    return L


def _p(a):
    return a.ctypes.data_as(_u32p)


@pytest.mark.parametrize("seed,energy_bits,prio_range", [
    (1, 0, 1 << 32), (2, 0, 4), (3, 16, 3), (4, 11, 1 << 32), (5, 5, 2)])
def test_closed_form_equals_literal_scan(seed, energy_bits, prio_range):
    rng = np.random.default_rng(seed)
    ncells = 20000                      # 5 cases x 20000 = 100000 cells
    m = rng.integers(0, 13, ncells)
    off = np.zeros(ncells + 1, np.uint32)
    off[1:] = np.cumsum(m)
    n = int(off[-1])
    mask = (1 << (energy_bits or 30)) - 1
    wolf_share = rng.random(ncells)     # per cell: all sheep .. all wolves
    wolf = rng.random(n) < np.repeat(wolf_share, m)
    energy = rng.integers(1, min(mask, 80) + 1, n)
    en = (energy | np.where(wolf, TYPE_BIT, 0)).astype(np.uint32)
    prio = rng.integers(0, prio_range, n, dtype=np.uint64).astype(np.uint32)
    dice = rng.integers(0, 100, n).astype(np.uint32)
    g0 = np.where(rng.random(ncells) < 0.5, 0, rng.integers(1, 10, ncells)).astype(np.uint32)
    prm = dict(sheep_gain_from_food=int(rng.integers(0, 40)),
               sheep_reproduce_threshold=int(rng.integers(0, 6)),
               sheep_reproduce_prob=int(rng.integers(0, 101)),
               wolves_gain_from_food=int(rng.integers(0, 40)),
               wolves_reproduce_threshold=int(rng.integers(0, 6)),
               wolves_reproduce_prob=int(rng.integers(0, 101)),
               grass_restart=int(rng.integers(1, 20)),
               init_sheep=0, init_wolves=0, grid_x=1, grid_y=1, iters=1)
    o = orc.oparams(prm, energy_bits)
    params = np.array([o.sheep_gain, o.sheep_thr, o.sheep_prob, o.wolves_gain,
                       o.wolves_thr, o.wolves_prob, o.grass_restart, mask], np.uint32)
    val = np.zeros(max(n, 1), np.uint32)
    kid = np.zeros(max(n, 1), np.uint32)
    eaters = np.zeros(ncells, np.uint32)
    _lib().act_cells_closed_form(_p(params), ncells, _p(off), _p(en), _p(prio), _p(dice),
                                 _p(g0), _p(val), _p(kid), _p(eaters))
    # the oracle's literal scan, cell by cell
    L = orc.lib()
    fin = np.zeros(13, np.uint32)
    okid = np.zeros(13, np.uint32)
    has = np.zeros(13, np.uint8)
    eat = np.zeros(13, np.uint8)
    u8p = C.POINTER(C.c_uint8)
    g = C.c_uint32()
    for c in range(ncells):
        a, b = int(off[c]), int(off[c + 1])
        g.value = int(g0[c])
        L.ppo_act_cell(C.byref(o), b - a, _p(en[a:b]), _p(prio[a:b]), _p(dice[a:b]),
                       C.byref(g), _p(fin), _p(okid), has.ctypes.data_as(u8p),
                       eat.ctypes.data_as(u8p))
        k = b - a
        v, kd = val[a:b], kid[a:b]
        assert np.array_equal((v & EATEN_BIT) != 0, eat[:k] != 0), c
        live = eat[:k] == 0
        assert np.array_equal(v[live] & 0x3fffffff, fin[:k][live]), c
        assert np.array_equal(v & TYPE_BIT, en[a:b] & TYPE_BIT), c
        assert np.array_equal((kd & KID_BIT) != 0, has[:k] != 0), c
        assert np.array_equal(kd[has[:k] != 0] & (KID_BIT - 1), okid[:k][has[:k] != 0]), c
        ate = g0[c] == 0 and g.value != 0
        assert eaters[c] == (1 if ate else 0), c
        assert g.value == (o.grass_restart if ate else g0[c]), c
