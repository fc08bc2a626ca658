"""ctypes wrapper of oracle/pp_cpu_port.c, the OpenMP restatement of the
reference's CPU algorithm (pp_cpu). CPU baseline and reference-semantics
side of the statistical comparison; TEST AND BASELINE INFRASTRUCTURE ONLY.
"""
import ctypes as C
import os
import subprocess
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(_HERE, "pp_cpu_port.c")
LIB_PATH = os.path.join(_HERE, "_build", "libpp_cpu_port.so")


class PParams(C.Structure):
    _fields_ = [(f, C.c_uint32) for f in (
        "init_sheep", "sheep_gain", "sheep_thr", "sheep_prob", "init_wolves",
        "wolves_gain", "wolves_thr", "wolves_prob", "grass_restart", "grid_x",
        "grid_y", "grid_xy", "iters")]


class PStats(C.Structure):
    _fields_ = [("sheep", C.c_uint32), ("wolves", C.c_uint32),
                ("grass", C.c_uint32), ("errors", C.c_uint32),
                ("sheep_en", C.c_uint64), ("wolves_en", C.c_uint64),
                ("grass_en", C.c_uint64)]

    def as_tuple(self):
        return (self.sheep, self.wolves, self.grass, self.sheep_en,
                self.wolves_en, self.grass_en)


def build():
    from pphpc_gb300.build import native_ok
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if (not os.path.exists(LIB_PATH) or not native_ok(LIB_PATH)
            or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC)):
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-fPIC", "-shared",
                        "-Wall", "-o", LIB_PATH, SRC], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.pcp_create.restype = C.c_void_p
        L.pcp_create.argtypes = [C.POINTER(PParams), C.c_uint64, C.c_uint32, C.c_int]
        L.pcp_destroy.argtypes = [C.c_void_p]
        L.pcp_step.restype = C.c_int
        L.pcp_step.argtypes = [C.c_void_p, C.POINTER(PStats)]
        L.pcp_stats_now.argtypes = [C.c_void_p, C.POINTER(PStats)]
        L.pcp_run.restype = C.c_int
        L.pcp_run.argtypes = [C.POINTER(PParams), C.c_uint64, C.c_uint32, C.c_uint32,
                              C.c_int, C.POINTER(PStats)]
        L.pcp_max_threads.restype = C.c_int
        _lib = L
    return _lib


def pparams(p):
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    o = PParams()
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
    return o


def threads():
    return lib().pcp_max_threads()


def run(p, seed, iters=None, max_agents=0, nthreads=0):
    """(iters+1, 6) uint64 stats of one run of the reference CPU algorithm."""
    o = pparams(p)
    iters = o.iters if iters is None else iters
    if not max_agents:
        max_agents = max(4 * (o.init_sheep + o.init_wolves), 3 * o.grid_x * o.grid_y) + 1024
    rows = (PStats * (iters + 1))()
    rc = lib().pcp_run(C.byref(o), seed, iters, max_agents, nthreads or threads(), rows)
    if rc not in (0, -8):
        raise RuntimeError("cpu port failed (%d)" % rc)
    return np.array([r.as_tuple() for r in rows], dtype=np.uint64)


def run_steps(workload, seed, steps, warmup, time_budget_s=150.0):
    """Time `steps` iterations after `warmup` ones with all host threads.
    If a full-size iteration would exceed the time budget, the grid is
    shrunk to a square sample with the same agent density (agent-steps/s is
    an intensive rate); the sample is reported."""
    o = dict(workload)
    nthr = threads()
    side = o["grid_x"]
    # probe the per-agent-step cost on a 1600x1600 sample
    probe = dict(o)
    f = 1600 * 1600 / (o["grid_x"] * o["grid_y"])
    probe.update(grid_x=1600, grid_y=1600, init_sheep=max(1, int(o["init_sheep"] * f)),
                 init_wolves=max(1, int(o["init_wolves"] * f)))
    po = pparams(probe)
    st = lib().pcp_create(C.byref(po), seed, 4 * (po.init_sheep + po.init_wolves) + 1024, nthr)
    s = PStats()
    lib().pcp_stats_now(st, C.byref(s))
    n = s.sheep + s.wolves
    t0 = time.perf_counter()
    for _ in range(3):
        lib().pcp_step(st, C.byref(s))
    dt = (time.perf_counter() - t0) / 3
    lib().pcp_destroy(st)
    per_cell_s = dt / (1600 * 1600)
    est = per_cell_s * o["grid_x"] * o["grid_y"] * (steps + warmup) * 1.5
    if est > time_budget_s:
        scale = (time_budget_s / est) ** 0.5
        side = max(200, int(o["grid_x"] * scale) // 100 * 100)
        f = side * side / (o["grid_x"] * o["grid_y"])
        o.update(grid_x=side, grid_y=side, init_sheep=max(1, int(o["init_sheep"] * f)),
                 init_wolves=max(1, int(o["init_wolves"] * f)))
    po = pparams(o)
    st = lib().pcp_create(C.byref(po), seed, 4 * (po.init_sheep + po.init_wolves) + 1024, nthr)
    if not st:
        raise MemoryError("cpu port allocation failed")
    lib().pcp_stats_now(st, C.byref(s))
    n = s.sheep + s.wolves
    for _ in range(warmup):
        lib().pcp_step(st, C.byref(s))
        n = s.sheep + s.wolves
    agent_steps = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        agent_steps += n
        lib().pcp_step(st, C.byref(s))
        n = s.sheep + s.wolves
    el = time.perf_counter() - t0
    lib().pcp_destroy(st)
    sample = ("%d iterations (after %d warm-up) of a %dx%d grid, v1 density (%s)"
              % (steps, warmup, side, side,
                 "full workload" if side == workload["grid_x"] else
                 "square sample of the 12800x12800 workload"))
    return {"value": agent_steps / el, "ms_per_step": el / steps * 1e3,
            "cores": nthr, "sample": sample}


def baseline_sample(workload, seed, iters=2):
    """Bounded CPU-baseline sample for the GPU arm's JSON line."""
    r = run_steps(workload, seed, steps=max(iters, 1), warmup=1, time_budget_s=30.0)
    return {"value": r["value"], "unit": "agent-steps/s", "cores": r["cores"],
            "kind": "port", "sample": r["sample"]}
