"""pphpc_gb300 -- GB300-native PPHPC simulation step behind a C ABI.

This module is a thin ctypes mirror of ``include/pphpc.h`` (the library's
C ABI). It loads ``libpphpc_gb300.so`` built in this package directory and
raises if the library is missing: there is no CPU fallback for the
simulation.

Reference interfaces mirrored (paths relative to the pphpc project root):
``PPParameters``/``PPStatistics`` (opencl/pp/pp_common.in.h:109-157),
``pp_load_params`` (opencl/pp/pp_common.c:39-195), ``pp_stats_save``
(opencl/pp/pp_common.c:205-240), the pp_gpu simulation loop
(opencl/pp/pp_gpu.c:573-987).
"""
import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libpphpc_gb300.so")
CLI_PATH = os.path.join(_PKG, "pp_gb300")

PP_SUCCESS = 0
PP_UNKNOWN_ARGS = -1
PP_INVALID_ARGS = -2
PP_LIBRARY_ERROR = -3
PP_UNABLE_TO_OPEN_PARAMS_FILE = -4
PP_INVALID_PARAMS_FILE = -5
PP_UNABLE_SAVE_STATS = -6
PP_OUT_OF_RESOURCES = -8
PP_ERR_CUDA = -9
PP_ERR_TIMEOUT = -10
PP_ERR_CANCELLED = -11

ERROR_NAMES = {
    0: "PP_SUCCESS", -1: "PP_UNKNOWN_ARGS", -2: "PP_INVALID_ARGS",
    -3: "PP_LIBRARY_ERROR", -4: "PP_UNABLE_TO_OPEN_PARAMS_FILE",
    -5: "PP_INVALID_PARAMS_FILE", -6: "PP_UNABLE_SAVE_STATS",
    -8: "PP_OUT_OF_RESOURCES", -9: "PP_ERR_CUDA", -10: "PP_ERR_TIMEOUT",
    -11: "PP_ERR_CANCELLED",
}

PARAM_FIELDS = ["init_sheep", "sheep_gain_from_food",
                "sheep_reproduce_threshold", "sheep_reproduce_prob",
                "init_wolves", "wolves_gain_from_food",
                "wolves_reproduce_threshold", "wolves_reproduce_prob",
                "grass_restart", "grid_x", "grid_y", "grid_xy", "iters"]


class PPError(RuntimeError):
    """A library call returned a negative pp_error_codes value."""

    def __init__(self, code, what=""):
        self.code = code
        super().__init__("%s failed: %s (%d)" % (what, ERROR_NAMES.get(code, "?"), code))


class PPParameters(C.Structure):
    _fields_ = [(f, C.c_uint32) for f in PARAM_FIELDS]

    def as_dict(self):
        return {f: getattr(self, f) for f in PARAM_FIELDS}


class PPStatistics(C.Structure):
    # the reference's field order (pp_common.in.h:109-124), sums widened
    _fields_ = [("sheep", C.c_uint32), ("wolves", C.c_uint32),
                ("grass", C.c_uint32), ("sheep_en", C.c_uint64),
                ("wolves_en", C.c_uint64), ("grass_en", C.c_uint64),
                ("errors", C.c_uint32)]

    def as_tuple(self):
        return (self.sheep, self.wolves, self.grass, self.sheep_en,
                self.wolves_en, self.grass_en)


class PPOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("max_agents", C.c_uint32),
                ("tile_cells", C.c_uint32), ("sort_digit_bits", C.c_uint32),
                ("use_graph", C.c_uint32), ("sort_pipeline", C.c_uint32),
                ("autotune", C.c_uint32), ("ss_from", C.c_uint32),
                ("agent_size", C.c_uint32)]


class PPRunDesc(C.Structure):
    _fields_ = [("params", PPParameters), ("seed", C.c_uint64)]


class PPBatchOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("pool_factor", C.c_uint32),
                ("tile_cells", C.c_uint32), ("sort_digit_bits", C.c_uint32),
                ("use_graph", C.c_uint32), ("stats_chunk", C.c_uint32),
                ("autotune", C.c_uint32), ("agent_size", C.c_uint32)]


class PPServeOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("mem_budget_bytes", C.c_uint64),
                ("max_runs", C.c_uint32), ("pool_factor", C.c_uint32),
                ("stats_chunk", C.c_uint32), ("ss_from", C.c_uint32),
                ("agent_size", C.c_uint32), ("tile_cells", C.c_uint32)]


class PPServeEvent(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int),
                ("n_rows", C.c_uint32), ("done", C.c_uint32)]


class PPTuning(C.Structure):
    _fields_ = [("tile_cells", C.c_uint32), ("sort_pipeline", C.c_uint32),
                ("sort_digit_bits", C.c_uint32), ("ns_per_agent_step", C.c_float)]


class PPFocal(C.Structure):
    _fields_ = [("max", C.c_double * 6), ("min", C.c_double * 6),
                ("ss_mean", C.c_double * 6), ("ss_std", C.c_double * 6),
                ("argmax", C.c_uint32 * 6), ("argmin", C.c_uint32 * 6),
                ("ss_n", C.c_uint32), ("pad", C.c_uint32)]

    def as_array(self):
        """(6 outputs, 6 measures): max, argmax, min, argmin, ss_mean,
        ss_std -- the layout of tests/focal.py."""
        import numpy as np
        return np.array([[self.max[k], self.argmax[k], self.min[k], self.argmin[k],
                          self.ss_mean[k], self.ss_std[k]] for k in range(6)])


class KernelProf(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint32),
                ("total_ms", C.c_double), ("bytes", C.c_double)]


STATS_CB = C.CFUNCTYPE(None, C.c_int, C.POINTER(PPStatistics), C.c_uint32,
                       C.c_void_p)

# Every function the C ABI exports: name -> (restype, argtypes).
_P = C.POINTER
_u32p = _P(C.c_uint32)
ABI = {
    "pp_load_params": (C.c_int, [_P(PPParameters), C.c_char_p, C.c_char_p, C.c_size_t]),
    "pp_params_check": (C.c_int, [_P(PPParameters), C.c_char_p, C.c_size_t]),
    "pp_stats_save": (C.c_int, [C.c_char_p, _P(PPStatistics), C.c_uint32, _P(PPParameters)]),
    "pp_stats_format_row": (C.c_int, [C.c_char_p, C.c_size_t, _P(PPStatistics), _P(PPParameters)]),
    "pp_opts_default": (None, [_P(PPOpts)]),
    "pp_sim_create": (C.c_int, [_P(PPParameters), C.c_uint64, _P(PPOpts), _P(C.c_void_p)]),
    "pp_sim_stats0": (C.c_int, [C.c_void_p, _P(PPStatistics)]),
    "pp_sim_step": (C.c_int, [C.c_void_p, C.c_uint32, _P(PPStatistics)]),
    "pp_sim_step_async": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "pp_sim_sync": (C.c_int, [C.c_void_p]),
    "pp_sim_info": (C.c_int, [C.c_void_p, _u32p, _u32p, _u32p]),
    "pp_sim_get_state": (C.c_int, [C.c_void_p, _u32p, _u32p, C.c_uint32, _u32p, _P(C.c_uint16)]),
    "pp_sim_stream": (C.c_void_p, [C.c_void_p]),
    "pp_sim_profile": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                 _P(C.c_double)]),
    "pp_sim_time": (C.c_int, [C.c_void_p, C.c_uint32, _P(C.c_float)]),
    "pp_sim_stats_range": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32,
                                     _P(PPStatistics)]),
    "pp_sim_io_bytes": (C.c_int, [C.c_void_p, _P(C.c_uint64), _P(C.c_uint64)]),
    "pp_sim_destroy": (C.c_int, [C.c_void_p]),
    "pp_release_cached_memory": (C.c_int, [C.c_int, _P(C.c_uint64)]),
    "pp_sim_snapshot_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "pp_sim_params": (C.c_int, [C.c_void_p, _P(PPParameters)]),
    "pp_sim_focal": (C.c_int, [C.c_void_p, _P(PPFocal)]),
    "pp_serve_focal": (C.c_int, [C.c_void_p, C.c_uint64, _P(PPFocal)]),
    "pp_sim_dump": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_char_p]),
    "pp_sim_restore": (C.c_int, [C.c_char_p, _P(PPOpts), _P(C.c_void_p)]),
    "pp_philox_fill": (C.c_int, [C.c_uint32] * 7 + [_u32p]),
    "pp_lookback_selftest": (C.c_int, [C.c_uint32, C.c_int32, _u32p]),
    "pp_move_host": (C.c_int, [_P(PPParameters), C.c_uint64, C.c_uint32, C.c_uint32,
                               _u32p, _u32p, _u32p, _u32p]),
    "pp_radix_sort_host": (C.c_int, [C.c_uint32, _u32p, _u32p, _u32p, _u32p,
                                     C.c_uint32, C.c_uint32]),
    "pp_cell_offsets_host": (C.c_int, [C.c_uint32, _u32p, C.c_uint32, _u32p]),
    "pp_radix_sort_noalloc": (C.c_int, [C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    "pp_batch_opts_default": (None, [_P(PPBatchOpts)]),
    "pp_batch_run": (C.c_int, [_P(PPRunDesc), C.c_int, _P(PPBatchOpts), STATS_CB, C.c_void_p]),
    "pp_serve_opts_default": (None, [_P(PPServeOpts)]),
    "pp_serve_create": (C.c_int, [_P(PPServeOpts), _P(C.c_void_p)]),
    "pp_serve_submit": (C.c_int, [C.c_void_p, _P(PPRunDesc), _P(C.c_uint64)]),
    "pp_serve_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pp_serve_poll": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pp_serve_read": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32,
                                _P(PPStatistics), _u32p]),
    "pp_serve_status": (C.c_int, [C.c_void_p, C.c_uint64, _P(PPServeEvent)]),
    "pp_serve_load": (C.c_int, [C.c_void_p, _u32p, _u32p]),
    "pp_serve_finished": (C.c_int, [C.c_void_p, _P(C.c_uint64), C.c_uint32, _u32p]),
    "pp_serve_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pp_serve_destroy": (C.c_int, [C.c_void_p]),
    "pp_autotune": (C.c_int, [_P(PPParameters), C.c_uint64, C.c_uint32, C.c_int,
                              _P(PPTuning)]),
    "pp_batch_autotune": (C.c_int, [_P(PPRunDesc), C.c_int, _P(PPBatchOpts), _P(PPTuning)]),
    "pp_version": (C.c_char_p, []),
}

_lib = None


def lib():
    """Load the library (once). Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libpphpc_gb300.so is not built; run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in ABI.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc, what):
    if rc != PP_SUCCESS:
        raise PPError(rc, what)


def make_params(**kw):
    p = PPParameters()
    for k, v in kw.items():
        setattr(p, k, v)
    p.grid_xy = p.grid_x * p.grid_y
    return p


def load_params(filename):
    """Parse a reference parameters file (`KEY = int`, 12 keys)."""
    p = PPParameters()
    msg = C.create_string_buffer(256)
    rc = lib().pp_load_params(C.byref(p), filename.encode(), msg, 256)
    if rc != PP_SUCCESS:
        raise PPError(rc, "pp_load_params: %s" % msg.value.decode())
    return p


def stats_save(filename, rows, params):
    arr = (PPStatistics * len(rows))(*rows)
    _check(lib().pp_stats_save(filename.encode(), arr, len(rows), C.byref(params)),
           "pp_stats_save")


def format_row(row, params):
    buf = C.create_string_buffer(256)
    lib().pp_stats_format_row(buf, 256, C.byref(row), C.byref(params))
    return buf.value.decode()


class Simulation:
    """One PPHPC run on the GPU (pp_sim_* of the C ABI). agent_size = the
    reference's -a/--agent-size: 64 or 32 give its 16- or 11-bit energy
    field, 0 a 30-bit one (pp_opts.agent_size)."""

    def __init__(self, params, seed=0, device=0, max_agents=0, tile_cells=0,
                 digit_bits=0, use_graph=True, sort_pipeline=False, autotune=False,
                 ss_from=1000, agent_size=0, _restore=None):
        L = lib()
        o = PPOpts()
        L.pp_opts_default(C.byref(o))
        o.device = device
        o.max_agents = max_agents
        o.tile_cells = tile_cells
        o.sort_digit_bits = digit_bits
        o.use_graph = 1 if use_graph else 0
        o.sort_pipeline = 1 if sort_pipeline else 0
        o.autotune = 1 if autotune else 0
        o.ss_from = ss_from
        o.agent_size = agent_size
        self.params = params
        self._h = C.c_void_p()
        if _restore is not None:
            _check(L.pp_sim_restore(os.fsencode(_restore), C.byref(o), C.byref(self._h)),
                   "pp_sim_restore")
        else:
            _check(L.pp_sim_create(C.byref(params), seed, C.byref(o), C.byref(self._h)),
                   "pp_sim_create")

    @classmethod
    def restore(cls, path, params, **kw):
        """A simulation continuing from a snapshot file (pp_sim_restore);
        `params` must be the saved simulation's parameters (the file holds
        them; they size the Python-side buffers)."""
        return cls(params, _restore=path, **kw)

    def focal(self):
        """PPHPC focal measures computed on the GPU (pp_sim_focal)."""
        f = PPFocal()
        _check(lib().pp_sim_focal(self._h, C.byref(f)), "pp_sim_focal")
        return f

    def dump(self, agents_path, cells_path, dump_type=0x01):
        """Append the state in the reference's PPG_DUMP formats (pp_sim_dump)."""
        _check(lib().pp_sim_dump(self._h, dump_type, os.fsencode(agents_path),
                                 os.fsencode(cells_path)), "pp_sim_dump")

    def save(self, path):
        """Write a snapshot of the current state (pp_sim_snapshot_save)."""
        _check(lib().pp_sim_snapshot_save(self._h, os.fsencode(path)),
               "pp_sim_snapshot_save")

    def stats0(self):
        s = PPStatistics()
        _check(lib().pp_sim_stats0(self._h, C.byref(s)), "pp_sim_stats0")
        return s

    def step(self, n):
        rows = (PPStatistics * max(n, 1))()
        _check(lib().pp_sim_step(self._h, n, rows), "pp_sim_step")
        return list(rows)[:n]

    def time(self, n):
        """Run n iterations between CUDA events on the simulation's
        stream; returns the device time in milliseconds."""
        ms = C.c_float()
        _check(lib().pp_sim_time(self._h, n, C.byref(ms)), "pp_sim_time")
        return ms.value

    def stats_range(self, first_iter, n):
        rows = (PPStatistics * max(n, 1))()
        _check(lib().pp_sim_stats_range(self._h, first_iter, n, rows),
               "pp_sim_stats_range")
        return list(rows)[:n]

    def profile(self, n):
        """Per-kernel CUDA-event timing over n iterations: a list of
        (name, launches, total_ms, algorithmic_bytes) and the agent-steps."""
        prof = (KernelProf * 5)()
        steps = C.c_double()
        _check(lib().pp_sim_profile(self._h, n, prof, 5, C.byref(steps)),
               "pp_sim_profile")
        return ([(k.name.decode(), k.launches, k.total_ms, k.bytes) for k in prof],
                steps.value)

    def io_bytes(self):
        h2d, d2h = C.c_uint64(), C.c_uint64()
        _check(lib().pp_sim_io_bytes(self._h, C.byref(h2d), C.byref(d2h)),
               "pp_sim_io_bytes")
        return h2d.value, d2h.value

    def info(self):
        it, na, cap = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(lib().pp_sim_info(self._h, C.byref(it), C.byref(na), C.byref(cap)),
               "pp_sim_info")
        return it.value, na.value, cap.value

    def state(self):
        import numpy as np
        cnt = C.c_uint32()
        _check(lib().pp_sim_get_state(self._h, None, None, 0, C.byref(cnt), None),
               "pp_sim_get_state")
        n = cnt.value
        cell = np.zeros(max(n, 1), np.uint32)
        en = np.zeros(max(n, 1), np.uint32)
        grass = np.zeros(self.params.grid_x * self.params.grid_y, np.uint16)
        nout = C.c_uint32()
        _check(lib().pp_sim_get_state(
            self._h, cell.ctypes.data_as(_u32p), en.ctypes.data_as(_u32p), n,
            C.byref(nout), grass.ctypes.data_as(_P(C.c_uint16))), "pp_sim_get_state")
        return cell[:nout.value], en[:nout.value], grass

    def close(self):
        if self._h:
            lib().pp_sim_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run(params, seed=0, iters=None, **kw):
    """Run a simulation; returns iters+1 stats rows (row 0 = initial)."""
    iters = params.iters if iters is None else iters
    with Simulation(params, seed, **kw) as sim:
        return [sim.stats0()] + sim.step(iters)


def lookback_selftest(n_chunks, stall_chunk=-1):
    """Bounded-wait self-test (pp_lookback_selftest): the chunks' exclusive
    prefixes; raises PPError(PP_ERR_TIMEOUT) when stall_chunk >= 0."""
    import numpy as np
    out = np.zeros(n_chunks, np.uint32)
    _check(lib().pp_lookback_selftest(n_chunks, stall_chunk, out.ctypes.data_as(_u32p)),
           "pp_lookback_selftest")
    return out


def release_cached_memory(device=-1):
    """Free the device buffers kept by the process cache of destroyed
    worlds (pp_release_cached_memory); returns the bytes released."""
    n = C.c_uint64()
    _check(lib().pp_release_cached_memory(device, C.byref(n)),
           "pp_release_cached_memory")
    return n.value


def batch_run(runs, pool_factor=4, tile_cells=0, digit_bits=0, use_graph=True,
              stats_chunk=1024, device=0, autotune=False, agent_size=0):
    """Run many independent simulations in one world. `runs` is a list of
    (PPParameters, seed); returns a list of row lists."""
    L = lib()
    descs = (PPRunDesc * len(runs))()
    for i, (p, s) in enumerate(runs):
        descs[i].params = p
        descs[i].seed = s
    o = PPBatchOpts()
    L.pp_batch_opts_default(C.byref(o))
    o.device = device
    o.pool_factor = pool_factor
    o.tile_cells = tile_cells
    o.sort_digit_bits = digit_bits
    o.use_graph = 1 if use_graph else 0
    o.stats_chunk = stats_chunk
    o.autotune = 1 if autotune else 0
    o.agent_size = agent_size
    out = [None] * len(runs)

    def cb(r, rows, n, user):
        out[r] = [PPStatistics.from_buffer_copy(rows[i]) for i in range(n)]

    ccb = STATS_CB(cb)
    _check(L.pp_batch_run(descs, len(runs), C.byref(o), ccb, None), "pp_batch_run")
    return out


class Server:
    """Continuous-batching server (pp_serve_* of the C ABI)."""

    def __init__(self, mem_budget_bytes=8 << 30, max_runs=256, pool_factor=4,
                 stats_chunk=64, device=0, ss_from=1000, agent_size=0, tile_cells=0):
        L = lib()
        o = PPServeOpts()
        L.pp_serve_opts_default(C.byref(o))
        o.device = device
        o.mem_budget_bytes = mem_budget_bytes
        o.max_runs = max_runs
        o.pool_factor = pool_factor
        o.stats_chunk = stats_chunk
        o.ss_from = ss_from
        o.agent_size = agent_size
        o.tile_cells = tile_cells
        self._h = C.c_void_p()
        _check(L.pp_serve_create(C.byref(o), C.byref(self._h)), "pp_serve_create")

    def submit(self, params, seed):
        d = PPRunDesc()
        d.params = params
        d.seed = seed
        rid = C.c_uint64()
        _check(lib().pp_serve_submit(self._h, C.byref(d), C.byref(rid)), "pp_serve_submit")
        return rid.value

    def cancel(self, rid):
        _check(lib().pp_serve_cancel(self._h, rid), "pp_serve_cancel")

    def poll(self, n_iters):
        _check(lib().pp_serve_poll(self._h, n_iters), "pp_serve_poll")

    def status(self, rid):
        ev = PPServeEvent()
        _check(lib().pp_serve_status(self._h, rid, C.byref(ev)), "pp_serve_status")
        return ev

    def finished(self, max_ids=4096):
        """Ids of requests finished since the last call (pp_serve_finished)."""
        ids = (C.c_uint64 * max_ids)()
        n = C.c_uint32()
        _check(lib().pp_serve_finished(self._h, ids, max_ids, C.byref(n)),
               "pp_serve_finished")
        return list(ids)[:n.value]

    def load(self):
        q, r = C.c_uint32(), C.c_uint32()
        _check(lib().pp_serve_load(self._h, C.byref(q), C.byref(r)), "pp_serve_load")
        return q.value, r.value

    def read(self, rid, first=0, n=None):
        ev = self.status(rid)
        n = ev.n_rows - first if n is None else n
        rows = (PPStatistics * max(n, 1))()
        got = C.c_uint32()
        _check(lib().pp_serve_read(self._h, rid, first, n, rows, C.byref(got)),
               "pp_serve_read")
        return list(rows)[:got.value]

    def focal(self, rid):
        """Focal measures of a finished request (pp_serve_focal)."""
        f = PPFocal()
        _check(lib().pp_serve_focal(self._h, rid, C.byref(f)), "pp_serve_focal")
        return f

    def release(self, rid):
        _check(lib().pp_serve_release(self._h, rid), "pp_serve_release")

    def close(self):
        if self._h:
            lib().pp_serve_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(params, seed=0, max_agents=0, device=0):
    """Measured launch geometry for a workload (pp_autotune): a dict with
    tile_cells, sort_pipeline, sort_digit_bits, ns_per_agent_step."""
    t = PPTuning()
    _check(lib().pp_autotune(C.byref(params), seed, max_agents, device, C.byref(t)),
           "pp_autotune")
    return {"tile_cells": t.tile_cells, "sort_pipeline": bool(t.sort_pipeline),
            "sort_digit_bits": t.sort_digit_bits,
            "ns_per_agent_step": t.ns_per_agent_step}


def batch_autotune(runs, pool_factor=4, device=0):
    """The geometry batch_run(..., autotune=True) uses for these runs."""
    descs = (PPRunDesc * len(runs))()
    for i, (p, sd) in enumerate(runs):
        descs[i].params = p
        descs[i].seed = sd
    o = PPBatchOpts()
    lib().pp_batch_opts_default(C.byref(o))
    o.device = device
    o.pool_factor = pool_factor
    t = PPTuning()
    _check(lib().pp_batch_autotune(descs, len(runs), C.byref(o), C.byref(t)),
           "pp_batch_autotune")
    return {"tile_cells": t.tile_cells, "sort_pipeline": bool(t.sort_pipeline),
            "sort_digit_bits": t.sort_digit_bits,
            "ns_per_agent_step": t.ns_per_agent_step}


def philox_fill(ctr, key, n):
    import numpy as np
    out = np.zeros(4 * n, np.uint32)
    _check(lib().pp_philox_fill(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], n,
                                out.ctypes.data_as(_u32p)), "pp_philox_fill")
    return out.reshape(n, 4)


def move(params, seed, it, cell, en):
    import numpy as np
    cell = np.ascontiguousarray(cell, np.uint32)
    en = np.ascontiguousarray(en, np.uint32)
    co = np.zeros_like(cell)
    eo = np.zeros_like(en)
    _check(lib().pp_move_host(C.byref(params), seed, it, len(cell),
                              cell.ctypes.data_as(_u32p), en.ctypes.data_as(_u32p),
                              co.ctypes.data_as(_u32p), eo.ctypes.data_as(_u32p)),
           "pp_move_host")
    return co, eo


def radix_sort(keys, vals, key_bits, digit_bits=0):
    import numpy as np
    keys = np.ascontiguousarray(keys, np.uint32)
    vals = np.ascontiguousarray(vals, np.uint32)
    ko = np.zeros_like(keys)
    vo = np.zeros_like(vals)
    _check(lib().pp_radix_sort_host(len(keys), keys.ctypes.data_as(_u32p),
                                    vals.ctypes.data_as(_u32p), ko.ctypes.data_as(_u32p),
                                    vo.ctypes.data_as(_u32p), key_bits, digit_bits),
           "pp_radix_sort_host")
    return ko, vo


def cell_offsets(sorted_keys, n_cells):
    import numpy as np
    k = np.ascontiguousarray(sorted_keys, np.uint32)
    off = np.zeros(n_cells + 1, np.uint32)
    _check(lib().pp_cell_offsets_host(len(k), k.ctypes.data_as(_u32p), n_cells,
                                      off.ctypes.data_as(_u32p)), "pp_cell_offsets_host")
    return off
