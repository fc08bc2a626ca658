"""ctypes wrapper of the CPU oracle (oracle/pp_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import this.
It is pinned to the reference's own CPU kernels (its actions bit for bit
where the draws' outcomes can be fixed, its dynamics statistically); see
pp_oracle.h.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libpp_oracle.so")

_u32p = C.POINTER(C.c_uint32)


class OParams(C.Structure):
    _fields_ = [(f, C.c_uint32) for f in (
        "init_sheep", "sheep_gain", "sheep_thr", "sheep_prob", "init_wolves",
        "wolves_gain", "wolves_thr", "wolves_prob", "grass_restart", "grid_x",
        "grid_y", "grid_xy", "iters", "energy_bits")]


class OStats(C.Structure):
    _fields_ = [("sheep", C.c_uint32), ("wolves", C.c_uint32),
                ("grass", C.c_uint32), ("errors", C.c_uint32),
                ("sheep_en", C.c_uint64), ("wolves_en", C.c_uint64),
                ("grass_en", C.c_uint64)]

    def as_tuple(self):
        return (self.sheep, self.wolves, self.grass, self.sheep_en,
                self.wolves_en, self.grass_en)


_lib = None


def use_threads():
    """Load the oracle built with its independent loops on OpenMP threads
    (identical results; for generating long fixtures). Call before any
    other use of this module."""
    global _lib, LIB_PATH
    if _lib is not None:
        raise RuntimeError("oracle library already loaded")
    from pphpc_gb300 import build as _b
    LIB_PATH = _b.build_oracle(omp=True)


def lib():
    global _lib
    if _lib is None:
        from pphpc_gb300 import build as _b  # builds oracle/_build too
        if not os.path.exists(LIB_PATH) or not _b.native_ok(LIB_PATH):
            _b.build_oracle()
        L = C.CDLL(LIB_PATH)
        L.ppo_philox.argtypes = [_u32p, _u32p, _u32p]
        L.ppo_philox_fill.argtypes = [C.c_uint32] * 7 + [_u32p]
        L.ppo_draw.restype = C.c_uint32
        L.ppo_draw.argtypes = [C.c_uint32, C.c_uint32]
        L.ppo_create.restype = C.c_void_p
        L.ppo_create.argtypes = [C.POINTER(OParams), C.c_uint64, C.c_uint32]
        L.ppo_destroy.argtypes = [C.c_void_p]
        L.ppo_stats_now.argtypes = [C.c_void_p, C.POINTER(OStats)]
        L.ppo_step.restype = C.c_int
        L.ppo_step.argtypes = [C.c_void_p, C.POINTER(OStats)]
        L.ppo_run.restype = C.c_int
        L.ppo_run.argtypes = [C.POINTER(OParams), C.c_uint64, C.c_uint32, C.POINTER(OStats)]
        L.ppo_num_agents.restype = C.c_uint32
        L.ppo_num_agents.argtypes = [C.c_void_p]
        L.ppo_iter.restype = C.c_uint32
        L.ppo_iter.argtypes = [C.c_void_p]
        L.ppo_get_agents.argtypes = [C.c_void_p, _u32p, _u32p]
        L.ppo_get_grass.argtypes = [C.c_void_p, C.POINTER(C.c_uint16)]
        L.ppo_move.argtypes = [C.POINTER(OParams), C.c_uint64, C.c_uint32, C.c_uint32,
                               _u32p, _u32p, _u32p, _u32p]
        L.ppo_sort.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _u32p, C.c_uint32]
        L.ppo_grass.argtypes = [C.c_uint32, C.POINTER(C.c_uint16)]
        L.ppo_act.restype = C.c_int64
        L.ppo_act.argtypes = [C.POINTER(OParams), C.c_uint64, C.c_uint32, C.c_uint32,
                              _u32p, _u32p, C.POINTER(C.c_uint16), _u32p, _u32p,
                              C.c_uint32]
        _u8p = C.POINTER(C.c_uint8)
        L.ppo_act_cell.argtypes = [C.POINTER(OParams), C.c_uint32, _u32p, _u32p, _u32p,
                                   _u32p, _u32p, _u32p, _u8p, _u8p]
        _lib = L
    return _lib


def oparams(p, energy_bits=0):
    """Convert a PPParameters (or any object/dict with the reference field
    names) to the oracle's struct; energy_bits = width of the energy field
    (11 and 16 as the reference's 32- and 64-bit agents; 0 = 30)."""
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    o = OParams()
    o.init_sheep = get("init_sheep")
    o.sheep_gain = get("sheep_gain_from_food")
    o.sheep_thr = get("sheep_reproduce_threshold")
    o.sheep_prob = get("sheep_reproduce_prob")
    o.init_wolves = get("init_wolves")
    o.wolves_gain = get("wolves_gain_from_food")
    o.wolves_thr = get("wolves_reproduce_threshold")
    o.wolves_prob = get("wolves_reproduce_prob")
    o.grass_restart = get("grass_restart")
    o.grid_x = get("grid_x")
    o.grid_y = get("grid_y")
    o.grid_xy = o.grid_x * o.grid_y
    o.iters = get("iters")
    o.energy_bits = energy_bits
    return o


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    out = (C.c_uint32 * 4)()
    lib().ppo_philox(c, k, out)
    return tuple(out)


def philox_fill(ctr, key, n):
    out = np.zeros(4 * n, np.uint32)
    lib().ppo_philox_fill(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], n,
                          out.ctypes.data_as(_u32p))
    return out.reshape(n, 4)


def draw(w, n):
    return lib().ppo_draw(w, n)


def run(p, seed, iters=None, energy_bits=0):
    """Stats rows (iters+1) as an (iters+1, 6) uint64 array:
    sheep, wolves, grass, sheep_en, wolves_en, grass_en."""
    o = oparams(p, energy_bits)
    iters = o.iters if iters is None else iters
    rows = (OStats * (iters + 1))()
    rc = lib().ppo_run(C.byref(o), seed, iters, rows)
    if rc != 0:
        raise RuntimeError("oracle run failed (%d)" % rc)
    return np.array([r.as_tuple() for r in rows], dtype=np.uint64)


class State:
    """Step-by-step oracle state (for state-level comparisons)."""

    def __init__(self, p, seed, capacity=0, energy_bits=0):
        self.o = oparams(p, energy_bits)
        self._h = lib().ppo_create(C.byref(self.o), seed, capacity)
        if not self._h:
            raise MemoryError("oracle allocation failed")

    def stats(self):
        s = OStats()
        lib().ppo_stats_now(self._h, C.byref(s))
        return s.as_tuple()

    def step(self):
        s = OStats()
        rc = lib().ppo_step(self._h, C.byref(s))
        if rc != 0:
            raise RuntimeError("oracle step failed (%d)" % rc)
        return s.as_tuple()

    def agents(self):
        n = lib().ppo_num_agents(self._h)
        cell = np.zeros(max(n, 1), np.uint32)
        en = np.zeros(max(n, 1), np.uint32)
        lib().ppo_get_agents(self._h, cell.ctypes.data_as(_u32p), en.ctypes.data_as(_u32p))
        return cell[:n], en[:n]

    def grass(self):
        g = np.zeros(self.o.grid_xy, np.uint16)
        lib().ppo_get_grass(self._h, g.ctypes.data_as(C.POINTER(C.c_uint16)))
        return g

    def close(self):
        if self._h:
            lib().ppo_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def move(p, seed, it, cell, en, energy_bits=0):
    o = oparams(p, energy_bits)
    cell = np.ascontiguousarray(cell, np.uint32)
    en = np.ascontiguousarray(en, np.uint32)
    co = np.zeros_like(cell)
    eo = np.zeros_like(en)
    lib().ppo_move(C.byref(o), seed, it, len(cell), cell.ctypes.data_as(_u32p),
                   en.ctypes.data_as(_u32p), co.ctypes.data_as(_u32p),
                   eo.ctypes.data_as(_u32p))
    return co, eo


def act(p, seed, it, cell, en, grass, cap, energy_bits=0):
    o = oparams(p, energy_bits)
    cell = np.ascontiguousarray(cell, np.uint32)
    en = np.ascontiguousarray(en, np.uint32)
    g = np.array(grass, np.uint16)
    co = np.zeros(cap, np.uint32)
    eo = np.zeros(cap, np.uint32)
    m = lib().ppo_act(C.byref(o), seed, it, len(cell), cell.ctypes.data_as(_u32p),
                      en.ctypes.data_as(_u32p), g.ctypes.data_as(C.POINTER(C.c_uint16)),
                      co.ctypes.data_as(_u32p), eo.ctypes.data_as(_u32p), cap)
    if m < 0:
        raise RuntimeError("oracle act overflow")
    return co[:m], eo[:m], g
