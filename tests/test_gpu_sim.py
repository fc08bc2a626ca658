"""Whole-step parity on the GPU: every stats row and the full agent/grass
state, bit-exact against the oracle, for small grids and edge cases."""
import numpy as np
import pytest

import pphpc_gb300 as pp
from oracle import pp_oracle as orc
from common import params, rows_array, first_diff

pytestmark = pytest.mark.gpu

# both iteration pipelines: fused act+move (default) and the sort pipeline
PIPES = pytest.mark.parametrize("sort_pipeline", [False, True], ids=["fused", "sort"])


def _check_run(p, seed, iters, **kw):
    got = rows_array(pp.run(p, seed, iters, **kw))
    want = orc.run(p, seed, iters)
    d = first_diff(got, want)
    assert d is None, d
    return got


@pytest.mark.parametrize("side,version,seed,iters", [
    (25, 1, 0, 400), (25, 2, 1, 300), (50, 1, 2, 500), (50, 2, 3, 300),
    (100, 1, 0, 1000), (64, 2, 9, 200), (33, 1, 17, 300)])
@PIPES
def test_stats_bit_exact(side, version, seed, iters, sort_pipeline):
    _check_run(params(side, version), seed, iters, sort_pipeline=sort_pipeline)


@PIPES
@pytest.mark.parametrize("tile", [1024, 2048, 4096, 8192])
def test_tile_sizes_agree(tile, sort_pipeline):
    _check_run(params(70, 2), 5, 150, tile_cells=tile, sort_pipeline=sort_pipeline)


@pytest.mark.parametrize("side,version,pool", [(70, 2, 0), (200, 2, 40), (150, 1, 0)])
def test_512_cell_tiles(side, version, pool):
    """The fused pipeline's 512-cell tiles (128-thread CTAs, crowded tiles
    at v2 densities); the sort pipeline refuses them."""
    p = params(side, version)
    cap = pool * (p.init_sheep + p.init_wolves) if pool else 0
    _check_run(p, 6, 120, tile_cells=512, max_agents=cap)
    with pytest.raises(pp.PPError) as ei:
        pp.Simulation(p, 6, tile_cells=512, sort_pipeline=True)
    assert ei.value.code == pp.PP_INVALID_ARGS


@pytest.mark.parametrize("digit_bits", [5, 6, 8])
def test_digit_widths_agree(digit_bits):
    _check_run(params(60, 1), 4, 150, digit_bits=digit_bits, sort_pipeline=True)


def test_wide_grid_many_tiles():
    # rows longer than a tile: moves across tile edges in x and y, with the
    # per-row wrap landing in far tiles
    _check_run(params(0, 1, gx=9000, gy=7, sheep=2500, wolves=1200), 13, 120,
               tile_cells=1024)


def test_without_graph():
    _check_run(params(40, 1), 11, 100, use_graph=False)


@pytest.mark.parametrize("gx,gy,s,w", [(1, 1, 5, 3), (1, 50, 20, 10), (50, 1, 20, 10),
                                       (7, 13, 40, 20), (300, 2, 30, 30),
                                       (65535, 2, 3000, 1500), (2, 65535, 3000, 1500)])
@PIPES
def test_degenerate_grids(gx, gy, s, w, sort_pipeline):
    _check_run(params(0, 1, gx=gx, gy=gy, sheep=s, wolves=w), 3, 120,
               sort_pipeline=sort_pipeline)


@pytest.mark.parametrize("s,w", [(0, 0), (50, 0), (0, 50)])
def test_single_species_and_empty(s, w):
    _check_run(params(30, 1, sheep=s, wolves=w), 8, 150)


@PIPES
def test_crowded_cells(sort_pipeline):
    # many agents per cell: exercises long in-cell orderings and the
    # shared-memory overflow path of the act kernel
    _check_run(params(0, 2, gx=20, gy=20, sheep=3000, wolves=1500), 12, 60,
               max_agents=400_000, sort_pipeline=sort_pipeline)


def test_dense_tiles_record_cache_paths():
    """512-cell tiles of a dense world (act_cap 2 T, so the move phase's
    record cache is spread over the dead counter, grass and permutation
    words), every acting agent reproducing: tiles pass from the spread cache
    (outputs that fit) through the uncached record writes (about twice as
    many outputs as agents, more than the spread words hold) to the crowded
    path as the population doubles."""
    p = params(0, 2, gx=64, gy=64, sheep=3000, wolves=1500, iters=8)
    p.sheep_reproduce_threshold = 0
    p.sheep_reproduce_prob = 100
    p.wolves_reproduce_threshold = 0
    p.wolves_reproduce_prob = 100
    pool = 2_000_000
    # agents a tile at the acts of iterations 1, 2, 3: about 560 (outputs
    # ~970, cached), 970 (outputs ~1650, uncached), 1650 (crowded)
    st = orc.State(p, 7, capacity=pool)
    want = np.array([st.stats()] + [st.step() for _ in range(p.iters)], np.uint64)
    st.close()
    got = rows_array(pp.run(p, 7, tile_cells=512, max_agents=pool))
    assert first_diff(got, want) is None


def test_pool_overflow_at_scale_is_refused():
    """A pool far below the population: 3200^2 v2 grows to about 27 times
    its initial agents while the pool holds 5 times, and on 512-cell tiles most
    tiles outgrow both their shared memory and the global scratch, for
    hundreds of iterations. The run is refused with PP_OUT_OF_RESOURCES
    (pp_gpu.c:847-852), and the device stays usable."""
    p = params(3200, 2, iters=300)
    n0 = p.init_sheep + p.init_wolves
    with pytest.raises(pp.PPError) as ei:
        pp.run(p, 2, max_agents=5 * n0, tile_cells=512)
    assert ei.value.code == pp.PP_OUT_OF_RESOURCES
    _check_run(params(40, 1), 3, 60)


@PIPES
def test_state_bit_exact_after_steps(sort_pipeline):
    p = params(40, 2)
    seed = 21
    o = orc.State(p, seed, capacity=1 << 20)
    with pp.Simulation(p, seed, max_agents=1 << 20, sort_pipeline=sort_pipeline) as sim:
        cell, en, grass = sim.state()
        ocell, oen = o.agents()
        assert np.array_equal(cell, ocell) and np.array_equal(en, oen)
        assert np.array_equal(grass, o.grass())
        for k in range(1, 40):
            sim.step(1)
            o.step()
            cell, en, grass = sim.state()
            ocell, oen = o.agents()
            assert np.array_equal(cell, ocell), k
            assert np.array_equal(en, oen), k
            assert np.array_equal(grass, o.grass()), k


def test_chunked_steps_equal_single_call():
    p = params(30, 1)
    a = rows_array(pp.run(p, 6, 300))
    with pp.Simulation(p, 6) as sim:
        rows = [sim.stats0()]
        for n in (1, 7, 50, 100, 142):
            rows += sim.step(n)
    assert np.array_equal(a, rows_array(rows))


@PIPES
def test_pool_overflow_reports_error(sort_pipeline):
    p = params(50, 2)
    with pytest.raises(pp.PPError) as ei:
        pp.run(p, 1, 200, max_agents=1500, sort_pipeline=sort_pipeline)
    assert ei.value.code == pp.PP_OUT_OF_RESOURCES


def test_invariants_long_run():
    p = params(100, 1)
    rows = rows_array(pp.run(p, 0, 2000))
    restart = p.grass_restart
    cells = p.grid_x * p.grid_y
    assert np.all(rows[:, 2] <= cells)
    assert np.all(rows[:, 5] <= cells * restart)
    assert np.all((rows[:, 0] == 0) | (rows[:, 3] >= rows[:, 0]))


@pytest.mark.parametrize("tile", [1024, 2048, 4096])
@pytest.mark.parametrize("side,version,seed,iters,pool", [
    (200, 1, 3, 300, 12000), (256, 1, 8, 200, 20000), (160, 2, 5, 30, 16000)])
def test_sparse_tiles_bit_exact(side, version, seed, iters, pool, tile):
    # a pool of well under one agent per cell: the act runs 128-thread CTAs
    # (sparse tiles) instead of the 256-thread ones the other tests get
    _check_run(params(side, version), seed, iters, max_agents=pool, tile_cells=tile)


def test_cached_device_buffers_reused_and_released():
    """A destroyed world's buffers stay in the process cache; the next
    world of the same shape reuses them, stale contents and all, with the
    same results; releasing the cache frees them."""
    pp.release_cached_memory()
    p = params(200, 2, iters=60)
    want = orc.run(p, 3)
    first = rows_array(pp.run(p, 3))
    cached = pp.release_cached_memory(0)
    assert cached > 0 and pp.release_cached_memory(0) == 0
    pp.run(p, 3)
    again = rows_array(pp.run(p, 3))
    assert first_diff(first, want) is None and first_diff(again, want) is None
    assert pp.release_cached_memory() >= cached


@PIPES
def test_threshold_zero_newborns_of_energy_zero(sort_pipeline):
    """Under a reproduction threshold of 0 a parent of energy 1 has a child
    of energy 0, which exists (pp_gpu.cl:948-960) and, by the modular
    decrement, leaves its first move with the field's maximum energy."""
    p = params(60, 1, iters=40)
    p.sheep_reproduce_threshold = 0
    p.wolves_reproduce_threshold = 0
    cap = 40 * (p.init_sheep + p.init_wolves)
    _check_run(p, 4, 40, sort_pipeline=sort_pipeline, max_agents=cap)
    st = orc.State(p, 4, capacity=cap)
    for _ in range(40):
        st.step()
    _, en = st.agents()
    st.close()
    assert ((en & 0x3fffffff) == 0x3fffffff).any()
