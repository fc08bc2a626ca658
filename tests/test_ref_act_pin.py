"""Pins the oracle's in-cell actions to the reference's own code, bit for
bit. The reference's step2 kernel (opencl/pp/pp_cpu.cl:596-866, compiled
unmodified, with its in-cell shuffle switched off by its own MAX_AGENT_SHUF
option) runs over cells whose agent lists are given in a chosen order; with
reproduction probabilities of 0 or 100 every draw's outcome is fixed. The
oracle's literal scan (ppo_act_cell), given the same order as priorities
and 16-bit energies (the reference's ushort field), must produce the same
survivors with the same energies, the same newborns, the same grass and the
same stats row, on random cells of 0 to 12 agents with energies that wrap."""
import ctypes as C

import numpy as np
import pytest

from oracle import pp_oracle as orc
from oracle import pp_ref

pytestmark = pytest.mark.skipif(not pp_ref.available(),
                                reason="reference kernels unavailable")


def _case(rng, grid_x):
    ncell = 3 * grid_x
    prm = dict(sheep_gain_from_food=int(rng.integers(0, 3000)),
               sheep_reproduce_threshold=int(rng.integers(1, 7)),
               sheep_reproduce_prob=int(rng.choice([0, 100])),
               wolves_gain_from_food=int(rng.integers(0, 60000)),
               wolves_reproduce_threshold=int(rng.integers(1, 7)),
               wolves_reproduce_prob=int(rng.choice([0, 100])),
               grass_restart=int(rng.integers(1, 20)),
               init_sheep=0, init_wolves=0, grid_x=grid_x, grid_y=3, iters=1)
    m = rng.integers(0, 13, ncell)
    m[rng.random(ncell) < 0.3] = 0
    cell_of = np.repeat(np.arange(ncell, dtype=np.uint32), m)
    n = len(cell_of)
    wolf_share = np.repeat(rng.random(ncell), m)
    typ = (rng.random(n) < wolf_share).astype(np.uint8)
    energy = rng.integers(1, 65536, n)
    small = rng.random(n) < 0.5
    energy[small] = rng.integers(1, 40, small.sum())
    # a sheep left at energy 0 by a wrapping gain reads as a free slot in the
    # reference (its record is all zeros); keep sheep gains from landing there
    sheep = typ == 0
    bad = sheep & (energy + prm["sheep_gain_from_food"] == 65536)
    energy[bad] -= 1
    grass = np.where(rng.random(ncell) < 0.5, 0,
                     rng.integers(1, prm["grass_restart"] + 1, ncell)).astype(np.uint32)
    return prm, m, cell_of, energy.astype(np.uint16), typ, grass


@pytest.mark.parametrize("seed", range(6))
def test_oracle_actions_equal_reference_step2(seed):
    rng = np.random.default_rng(seed)
    grid_x = 1500
    prm, m, cell_of, energy, typ, grass = _case(rng, grid_x)
    lists, gout, st = pp_ref.step2_cells(prm, cell_of, energy, typ, grass)
    o = orc.oparams(prm, 16)
    L = orc.lib()
    u32p, u8p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint8)
    en = (energy.astype(np.uint32) | (typ.astype(np.uint32) << 31)).astype(np.uint32)
    fin = np.zeros(13, np.uint32)
    kid = np.zeros(13, np.uint32)
    has = np.zeros(13, np.uint8)
    eat = np.zeros(13, np.uint8)
    g = C.c_uint32()
    off = np.concatenate([[0], np.cumsum(m)])
    sums = np.zeros(6, np.uint64)
    for c in range(3 * grid_x):
        a, b = int(off[c]), int(off[c + 1])
        k = b - a
        prio = np.arange(k, dtype=np.uint32)          # list order = acting order
        dice = np.zeros(k, np.uint32)                  # < prob iff prob is 100
        g.value = int(grass[c])
        L.ppo_act_cell(C.byref(o), k, en[a:b].ctypes.data_as(u32p),
                       prio.ctypes.data_as(u32p), dice.ctypes.data_as(u32p), C.byref(g),
                       fin.ctypes.data_as(u32p), kid.ctypes.data_as(u32p),
                       has.ctypes.data_as(u8p), eat.ctypes.data_as(u8p))
        # the reference prepends the cell's newborns, newest first, to the
        # surviving agents in their list order
        t = typ[a:b]
        want = [(int(kid[j]), int(t[j])) for j in range(k) if has[j]][::-1]
        want += [(int(fin[j]), int(t[j])) for j in range(k) if not eat[j]]
        assert lists[c] == want, (c, lists[c], want)
        assert gout[c] == g.value, c
        for e_, t_ in want:
            sums[t_] += 1
            sums[3 + t_] += e_
        sums[2] += g.value == 0
        sums[5] += g.value
    # the stats row: counts and 32-bit sums, as the reference accumulates them
    assert st[0] == sums[0] and st[1] == sums[1] and st[2] == sums[2]
    assert st[3] == int(sums[3]) % (1 << 32) and st[4] == int(sums[4]) % (1 << 32)
    assert st[5] == int(sums[5]) % (1 << 32) and st[6] == 0
