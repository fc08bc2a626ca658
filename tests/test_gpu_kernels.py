"""Kernel-level parity on the GPU: each kernel alone, through the C ABI,
against the oracle (or a numpy restatement for the sort and offsets)."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from oracle import pp_oracle as orc
from common import params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ctr,key", [((0, 0, 0, 0), (0, 0)),
                                     ((123, 7, 2, 0), (0xdeadbeef, 0x1234)),
                                     ((0xfffffff0, 0xffffffff, 3, 0xffffffff),
                                      (0xffffffff, 0xffffffff))])
def test_philox_matches_oracle(ctr, key):
    n = 1 << 16
    got = pp.philox_fill(ctr, key, n)
    want = orc.philox_fill(ctr, key, n)
    assert np.array_equal(got, want)


def test_philox_million_counters():
    n = 1_000_000
    got = pp.philox_fill((0, 5, 2, 0), (42, 0), n)
    want = orc.philox_fill((0, 5, 2, 0), (42, 0), n)
    assert np.array_equal(got, want)


def _agents(rng, p, n):
    # cell-sorted, as the move's input always is (ranks within cells key the draws)
    cell = np.sort(rng.integers(0, p.grid_x * p.grid_y, n, dtype=np.uint32))
    e = rng.integers(0, 60, n, dtype=np.uint32)
    t = rng.integers(0, 2, n, dtype=np.uint32) << np.uint32(31)
    return cell, e | t


@pytest.mark.parametrize("gx,gy", [(100, 100), (1, 1), (1, 7), (9, 1), (257, 3),
                                   (12800, 12800), (65535, 2)])
def test_move_matches_oracle(gx, gy):
    rng = np.random.default_rng(gx * 7 + gy)
    p = params(10, gx=gx, gy=gy, sheep=10, wolves=10)
    cell, en = _agents(rng, p, 50_000)
    # put agents on all four borders and corners
    cell[:4] = [0, gx - 1, (gy - 1) * gx, gx * gy - 1]
    en[:4] = 10
    order = np.argsort(cell, kind="stable")
    cell, en = cell[order], en[order]
    for it in (1, 2, 4000):
        gc, ge = pp.move(p, 99, it, cell, en)
        oc, oe = orc.move(p, 99, it, cell, en)
        assert np.array_equal(gc, oc), it
        assert np.array_equal(ge, oe), it


def test_move_energy_death():
    """Energy 1 dies in the move; energy 0 (only reachable by a gain that
    wraps the energy field) wraps to the field maximum and lives, as the
    reference's modular decrement does (pp_gpu.cl:805-810)."""
    p = params(20)
    cell = np.arange(6, dtype=np.uint32)
    en = np.array([0, 1, 2, 0x80000000, 0x80000001, 0x80000002], np.uint32)
    gc, ge = pp.move(p, 1, 1, cell, en)
    dead = p.grid_x * p.grid_y
    assert list(gc[[1, 4]]) == [dead] * 2
    assert ge[2] == 1 and ge[5] == 0x80000001
    assert ge[0] == 0x3fffffff and ge[3] == 0x80000000 | 0x3fffffff
    assert all(gc[[0, 2, 3, 5]] < dead)
    oc, oe = orc.move(p, 1, 1, cell, en)
    assert np.array_equal(gc, oc) and np.array_equal(ge, oe)


def _stable(keys, vals):
    o = np.argsort(keys, kind="stable")
    return keys[o], vals[o]


@pytest.mark.parametrize("n", [0, 1, 2, 31, 4095, 4096, 4097, 100_000, 1_234_567])
@pytest.mark.parametrize("key_bits", [14, 28])
def test_radix_sort_random(n, key_bits):
    rng = np.random.default_rng(n + key_bits)
    keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = pp.radix_sort(keys, vals, key_bits)
    wk, wv = _stable(keys, vals)
    assert np.array_equal(gk, wk)
    assert np.array_equal(gv, wv)


@pytest.mark.parametrize("digit_bits", [5, 6, 7, 8])
def test_radix_sort_digit_widths(digit_bits):
    rng = np.random.default_rng(digit_bits)
    n = 300_000
    keys = rng.integers(0, 1 << 27, n, dtype=np.uint32)
    vals = rng.integers(0, 1 << 32, n, dtype=np.uint32)
    gk, gv = pp.radix_sort(keys, vals, 27, digit_bits)
    wk, wv = _stable(keys, vals)
    assert np.array_equal(gk, wk) and np.array_equal(gv, wv)


@pytest.mark.parametrize("kind", ["equal", "reverse", "dead_heavy", "sorted", "few"])
def test_radix_sort_adversarial(kind):
    n = 500_000
    rng = np.random.default_rng(5)
    dead = 1 << 24
    if kind == "equal":
        keys = np.full(n, 12345, np.uint32)
    elif kind == "reverse":
        keys = np.arange(n, 0, -1, dtype=np.uint32)
    elif kind == "dead_heavy":
        keys = np.where(rng.random(n) < 0.9, dead,
                        rng.integers(0, dead, n)).astype(np.uint32)
    elif kind == "sorted":
        keys = np.sort(rng.integers(0, dead, n)).astype(np.uint32)
    else:
        keys = rng.integers(0, 3, n).astype(np.uint32) * 1000
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = pp.radix_sort(keys, vals, 25)
    wk, wv = _stable(keys, vals)
    assert np.array_equal(gk, wk) and np.array_equal(gv, wv)


@pytest.mark.parametrize("n,cells", [(0, 10), (1, 1), (1000, 10_000), (50_000, 1000),
                                     (100_000, 1_000_000)])
def test_cell_offsets(n, cells):
    rng = np.random.default_rng(n)
    keys = np.sort(rng.integers(0, cells + 1, n)).astype(np.uint32)  # cells = dead
    off = pp.cell_offsets(keys, cells)
    want = np.searchsorted(keys, np.arange(cells + 1), side="left")
    assert np.array_equal(off, want.astype(np.uint32))
