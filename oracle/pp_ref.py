"""ctypes wrapper of oracle/_ref/libpp_cpu_ref.so: the reference's own CPU
kernels (opencl/pp/pp_cpu.cl, compiled unmodified by oracle/ref/build_ref.py)
driven by the reference host's work sizes and launch loop on host threads.

TEST AND BASELINE INFRASTRUCTURE ONLY: the statistical target of the parity
tests and the CPU baseline of bench.py. Only its RNG is not the reference's
(cl_ops is absent; see oracle/ref/ocl_compat.hpp), so a seed gives a
different trajectory than the reference's binary would, drawn by the same
algorithm.
"""
import ctypes as C
import time

import numpy as np

FIELDS = ["init_sheep", "sheep_gain_from_food", "sheep_reproduce_threshold",
          "sheep_reproduce_prob", "init_wolves", "wolves_gain_from_food",
          "wolves_reproduce_threshold", "wolves_reproduce_prob", "grass_restart",
          "grid_x", "grid_y", "grid_xy", "iters"]
DEFAULT_MAX_AGENTS = 16777216    # the reference's -m default (pp_cpu.c:30-36)

_u32p = C.POINTER(C.c_uint32)
_lib = None


class Unavailable(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        from oracle.ref import build_ref
        path = build_ref.build()
        if path is None:
            raise Unavailable("the reference tree and its preprocessed kernels "
                              "are both absent")
        L = C.CDLL(path)
        L.ppr_create.restype = C.c_void_p
        L.ppr_create.argtypes = [_u32p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int,
                                 C.POINTER(C.c_int)]
        L.ppr_destroy.argtypes = [C.c_void_p]
        L.ppr_step.restype = C.c_int
        L.ppr_step.argtypes = [C.c_void_p, C.c_uint32, _u32p]
        L.ppr_row.argtypes = [C.c_void_p, C.c_uint32, _u32p]
        L.ppr_threads.restype = C.c_int
        L.ppr_threads.argtypes = [C.c_void_p]
        L.ppr_run.restype = C.c_int
        L.ppr_run.argtypes = [_u32p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, _u32p]
        L.ppr_worksizes.restype = C.c_int
        L.ppr_worksizes.argtypes = [C.c_uint32, C.POINTER(C.c_ulong), C.POINTER(C.c_ulong)]
        _lib = L
    return _lib


def available():
    try:
        lib()
        return True
    except (Unavailable, RuntimeError, OSError):
        return False


def _params(p):
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    vals = []
    for f in FIELDS:
        if f == "grid_xy":
            vals.append(get("grid_x") * get("grid_y"))
        else:
            vals.append(get(f))
    return (C.c_uint32 * 13)(*vals)


def worksizes(rows):
    g, r = C.c_ulong(), C.c_ulong()
    if lib().ppr_worksizes(rows, C.byref(g), C.byref(r)) != 0:
        raise ValueError("fewer than three rows")
    return g.value, r.value


def run(p, seed, iters=None, max_agents=0, threads=0):
    """Stats rows 0..iters as an (iters+1, 6) uint64 array (sheep, wolves,
    grass, sheep_en, wolves_en, grass_en; the reference's 32-bit sums), and
    raises if the run recorded allocation errors."""
    rows = run_raw(p, seed, iters, max_agents, threads)
    if rows[:, 6].any():
        raise RuntimeError("reference run had %d allocation errors" % int(rows[:, 6].sum()))
    return rows[:, :6].astype(np.uint64)


def run_raw(p, seed, iters=None, max_agents=0, threads=0):
    """(iters+1, 7) uint32 rows including the errors column."""
    prm = _params(p)
    n = prm[12] if iters is None else iters
    out = np.zeros((n + 1, 7), np.uint32)
    rc = lib().ppr_run(prm, seed, n, max_agents, threads, out.ctypes.data_as(_u32p))
    if rc != 0:
        raise RuntimeError("reference run failed (%d)" % rc)
    return out


class Sim:
    """Step-by-step reference simulation (one at a time per process)."""

    def __init__(self, p, seed, max_iters, max_agents=0, threads=0):
        rc = C.c_int()
        self._h = lib().ppr_create(_params(p), seed, max_iters, max_agents, threads,
                                   C.byref(rc))
        if not self._h:
            raise RuntimeError("reference create failed (%d)" % rc.value)

    def threads(self):
        return lib().ppr_threads(self._h)

    def step(self, n):
        out = np.zeros((n, 7), np.uint32)
        rc = lib().ppr_step(self._h, n, out.ctypes.data_as(_u32p))
        if rc != 0:
            raise RuntimeError("reference step failed (%d)" % rc)
        return out

    def row(self, it):
        out = np.zeros(7, np.uint32)
        lib().ppr_row(self._h, it, out.ctypes.data_as(_u32p))
        return out

    def close(self):
        if self._h:
            lib().ppr_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def timed_steps(p, seed, steps, warmup, max_agents=0, threads=0):
    """warmup untimed iterations, then `steps` iterations timed one by one
    on the host clock; agent-steps/s over the timed ones (agents at the
    start of each iteration, as the GPU bench counts them)."""
    t0 = time.perf_counter()
    s = Sim(p, seed, warmup + steps, max_agents, threads)
    t_init = time.perf_counter() - t0
    prev = s.row(0)
    if warmup:
        prev = s.step(warmup)[-1]
    times, agent_steps = [], 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        r = s.step(1)[0]
        times.append(time.perf_counter() - t0)
        agent_steps += float(prev[0]) + float(prev[1])
        prev = r
    threads_used = s.threads()
    s.close()
    total = sum(times)
    return {"value": agent_steps / total, "ms_per_step": 1e3 * total / steps,
            "agent_steps": agent_steps, "seconds": total, "cores": threads_used,
            "setup_s": t_init}


_lib_noshuf = None


def lib_noshuf():
    """The reference's kernels with the in-cell shuffle compiled out."""
    global _lib_noshuf
    if _lib_noshuf is None:
        from oracle.ref import build_ref
        path = build_ref.build(noshuf=True)
        if path is None:
            raise Unavailable("the reference tree and its preprocessed kernels "
                              "are both absent")
        L = C.CDLL(path)
        u16p, u8p = C.POINTER(C.c_uint16), C.POINTER(C.c_uint8)
        L.ppr_step2_cells.restype = C.c_int
        L.ppr_step2_cells.argtypes = [_u32p, C.c_uint32, _u32p, u16p, u8p, _u32p,
                                      C.c_uint32, u16p, u8p, _u32p, _u32p, _u32p]
        _lib_noshuf = L
    return _lib_noshuf


def step2_cells(p, cell_of, energy, typ, grass):
    """One run of the reference's step2 kernel (shuffle compiled out) over a
    grid_x x 3 grid: agent i in cell cell_of[i] (list order = array order)
    with energy[i] (u16) and type typ[i]; grass: 3 grid_x countdowns.
    Returns (per-cell lists of (energy, type) after the step, grass after,
    the stats row of 7 uint32)."""
    prm = _params(p)
    cell_of = np.ascontiguousarray(cell_of, np.uint32)
    energy = np.ascontiguousarray(energy, np.uint16)
    typ = np.ascontiguousarray(typ, np.uint8)
    grass = np.ascontiguousarray(grass, np.uint32)
    ncell = len(grass)
    cap = 3 * len(cell_of) + 16
    oe = np.zeros(cap, np.uint16)
    ot = np.zeros(cap, np.uint8)
    cnt = np.zeros(ncell, np.uint32)
    gout = np.zeros(ncell, np.uint32)
    st = np.zeros(7, np.uint32)
    u16p, u8p = C.POINTER(C.c_uint16), C.POINTER(C.c_uint8)
    rc = lib_noshuf().ppr_step2_cells(
        prm, len(cell_of), cell_of.ctypes.data_as(_u32p), energy.ctypes.data_as(u16p),
        typ.ctypes.data_as(u8p), grass.ctypes.data_as(_u32p), cap,
        oe.ctypes.data_as(u16p), ot.ctypes.data_as(u8p), cnt.ctypes.data_as(_u32p),
        gout.ctypes.data_as(_u32p), st.ctypes.data_as(_u32p))
    if rc != 0:
        raise RuntimeError("reference step2 harness failed (%d)" % rc)
    lists, o = [], 0
    for c in range(ncell):
        k = int(cnt[c])
        lists.append(list(zip(oe[o:o + k].tolist(), ot[o:o + k].tolist())))
        o += k
    return lists, gout, st
