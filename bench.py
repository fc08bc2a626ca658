"""Benchmark of the PPHPC simulation step on GB300.

Workload: plain PPHPC, 12800 x 12800 toroidal grid (163.84 M cells),
parameter set v1 scaled by area (6,553,600 sheep, 3,276,800 wolves),
seed 2, agent pool 5x the initial agents (the v1 population peaks at 4.25x
the initial agents near iteration 147), uint32 SoA agents, uint16 grass.
A "step" is one simulation iteration over the whole grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       W untimed iterations, then K iterations timed with CUDA events
            on the simulation's stream (graph replay; state resident in
            HBM; the working set, ~2 GB, exceeds the 129 MB L2). value =
            agent-steps / s over all ranks. `e2e` is a whole job through the
            C ABI from the host: pp_sim_create (parameters and run tables
            copied in, state initialised on the GPU), the iterations with
            every stats row copied back to a host buffer, pp_sim_destroy.
            `roofline` comes from per-kernel CUDA events (pp_sim_profile)
            over a few further iterations; its algorithmic bytes are the
            per-iteration figure of the reference-shaped step,
            12 C + (16 + 16 P + 16) N bytes (C cells, N agents at the
            iteration's start, P = 4 sort passes at this grid size; the
            8 bytes per birth are left out), attributed to the fused
            act+move kernel, which does the whole iteration but the stats;
            `dram_frac` beside it is the kernel's measured DRAM traffic
            (ncu, profiles/ncu_traffic.json) over the same launch time.
            Further legs (each skippable):
            `full_run`  the whole 4000-iteration run of the workload, end to
                        end and device-timed;
            `batched`   the 64-run mix (32 x 200^2 v1, 16 x 800^2 v2,
                        8 x 1600^2 v1, 8 x 3200^2 v2, seeds 100..163,
                        --batch-iters iterations each) through pp_batch_run
                        (one world, every launch shared) and run by run
                        through pp_sim_*, both end to end, bit-exactness of
                        every run, per-shape plain times and the bound they
                        put on the batching speed-up;
            `configs`   the reference's two small plain configs (100^2 v1
                        seed 0, 400^2 v2 seed 1, 4000 iterations), whole
                        runs on the GPU and by the reference's CPU kernels;
            `served`    the 1000-request Poisson stream (below);
            `cpu_baseline` the reference's CPU kernels on a bounded sample
                        of the workload.
reference:  the reference's own CPU algorithm: opencl/pp/pp_cpu.cl compiled
            unmodified for the host (oracle/ref/build_ref.py; only its RNG,
            from the absent cl_ops library, is a stand-in), driven by the
            reference host's work sizes and launch loop with all host
            threads, on the same workload and window: W untimed iterations,
            then K iterations timed one by one (host clock).
With N > 1 (torchrun), every rank runs an independent replica (the runs
do not exchange data); the timed region is bracketed by barriers and the
slowest rank's time is used. The reference arm runs on rank 0 only.

  python bench.py --workload configs | served

prints only the `configs` or `served` leg as its own line. The served
workload: a Poisson stream (20 requests/s) of 1000 runs, side uniform in
{100, ..., 3200}, parameter set v1 or v2 (p = 0.5), iterations uniform in
[500, 4000], sequential seeds, admitted into one continuously batched world
under a 150 GB budget; p50 / p99 completion latency (arrival to last stats
row on the host) and aggregate agent-steps/s.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(init_sheep=6553600, sheep_gain_from_food=4,
                sheep_reproduce_threshold=2, sheep_reproduce_prob=4,
                init_wolves=3276800, wolves_gain_from_food=20,
                wolves_reproduce_threshold=2, wolves_reproduce_prob=5,
                grass_restart=10, grid_x=12800, grid_y=12800, iters=4000)
SEED = 2
WORKLOAD_NAME = "pphpc-12800x12800-v1"

# Parameter sets v1 and v2 (the reference's configs/config*v1.txt and
# *v2.txt); agents scale with the grid area (400 sheep and 200 wolves per
# 100 x 100 cells for both).
V1 = dict(sheep_gain_from_food=4, sheep_reproduce_threshold=2,
          sheep_reproduce_prob=4, wolves_gain_from_food=20,
          wolves_reproduce_threshold=2, wolves_reproduce_prob=5,
          grass_restart=10)
V2 = dict(sheep_gain_from_food=30, sheep_reproduce_threshold=2,
          sheep_reproduce_prob=10, wolves_gain_from_food=10,
          wolves_reproduce_threshold=2, wolves_reproduce_prob=5,
          grass_restart=15)
MIX = [(200, 1, 32), (800, 2, 16), (1600, 1, 8), (3200, 2, 8)]
POOL_FACTOR = 40     # v2 populations peak near 36x their initial agents


def scaled_params(pp, side, version, iters):
    area = side * side
    return pp.make_params(init_sheep=area * 4 // 100, init_wolves=area * 2 // 100,
                          grid_x=side, grid_y=side, iters=iters,
                          **(V1 if version == 1 else V2))


def spec_bytes_per_iter(cells, n_agents):
    """Per-iteration bytes of the reference-shaped step: 12 bytes per cell
    (grass read + write, cell offsets written and read) and 16 + 16 P + 16
    bytes per agent (move, P sort passes, act), P = ceil((ceil(log2 C) +
    1) / 8) 8-bit digit passes; births (8 bytes each) are not counted."""
    import math
    P = math.ceil((math.ceil(math.log2(cells)) + 1) / 8)
    return 12.0 * cells + (32.0 + 16.0 * P) * n_agents, P


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Barrier and max-reduction over ranks (gloo, CPU tensors)."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM traffic of each kernel from the committed ncu summary
    (profiles/ncu_traffic.json), as bytes per processed unit (agent, or
    cell and agent), scaled to this workload."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


E2E_JOBS = 3               # end-to-end jobs timed; the median is reported
REF_MAX_AGENTS = 1 << 27   # the reference's -m for the 12800^2 workload (1 GiB of slots)


def workload(pp, args):
    """The plain workload: 12800 x 12800 v1 by default; --side scales the
    grid (agents by area) for smaller cases of the same kernels, --params
    picks the parameter set."""
    if args.side == 12800 and args.params == "v1":
        return pp.make_params(**WORKLOAD), WORKLOAD_NAME
    p = scaled_params(pp, args.side, 1 if args.params == "v1" else 2, WORKLOAD["iters"])
    return p, "pphpc-%dx%d-%s" % (args.side, args.side, args.params)


def workload_dict(args):
    """The plain workload as a parameter dict (no library needed)."""
    wl, wname = dict(WORKLOAD), WORKLOAD_NAME
    if args.side != 12800 or args.params != "v1":
        a = args.side * args.side
        wl.update(grid_x=args.side, grid_y=args.side, init_sheep=a * 4 // 100,
                  init_wolves=a * 2 // 100, **(V1 if args.params == "v1" else V2))
        wname = "pphpc-%dx%d-%s" % (args.side, args.side, args.params)
    return wl, wname


def config_of(args, world):
    """The `config` object, identical in both arms."""
    wl, wname = workload_dict(args)
    return {"workload": wname, "grid": "%dx%d" % (wl["grid_x"], wl["grid_y"]),
            "params": args.params, "init_sheep": wl["init_sheep"],
            "init_wolves": wl["init_wolves"], "seed": SEED,
            "timed_iterations": "%d..%d" % (args.warmup + 1, args.warmup + args.steps),
            "l2": "inputs larger than L2 (working set ~2 GB on the GPU)",
            "parallelism": "replicas" if world > 1 else "single"}


def ref_max_agents(wl):
    """Agent slots for the reference's CPU kernels: its default (2^24) for
    the small configs, 2^27 for larger grids (its random slot allocation
    needs several times the live agents)."""
    n0 = wl["init_sheep"] + wl["init_wolves"]
    return REF_MAX_AGENTS if 8 * n0 > (1 << 24) else 0


def cpu_sample(wl, steps, warmup):
    """The reference's CPU kernels (all host threads) on `steps` iterations
    after `warmup`; falls back to the single-threaded oracle where the
    reference's kernels are unavailable."""
    from oracle import pp_ref
    if pp_ref.available():
        r = pp_ref.timed_steps(wl, SEED, steps, warmup, max_agents=ref_max_agents(wl))
        sample = ("iterations %d..%d of the %dx%d v1 workload (seed %d), each timed; "
                  "opencl/pp/pp_cpu.cl compiled unmodified, the reference host's "
                  "work sizes and launch loop, %d host threads, %d agent slots"
                  % (warmup + 1, warmup + steps, wl["grid_x"], wl["grid_y"], SEED,
                     r["cores"], ref_max_agents(wl) or 1 << 24))
        return dict(r, kind="reference", sample=sample)
    from oracle import pp_oracle as orc
    st = orc.State(wl, SEED, capacity=5 * (wl["init_sheep"] + wl["init_wolves"]))
    prev = st.stats()
    for _ in range(warmup):
        prev = st.step()
    agent_steps, t0 = 0.0, time.perf_counter()
    for _ in range(steps):
        agent_steps += prev[0] + prev[1]
        prev = st.step()
    el = time.perf_counter() - t0
    st.close()
    return {"value": agent_steps / el, "ms_per_step": 1e3 * el / steps, "cores": 1,
            "kind": "port", "sample": "iterations %d..%d, single-threaded oracle "
            "(the reference's kernels unavailable)" % (warmup + 1, warmup + steps)}


def kernel_traffic(name, cells, n_agents):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary
    (profiles/ncu_traffic.json), scaled to this launch's cells and agents."""
    tr = ncu_traffic().get(name)
    if not tr:
        return None
    unit = tr.get("per")
    if unit == "agent":
        return tr["bytes_per_unit"] * n_agents
    if unit == "cell+agent":
        return tr["bytes_per_cell"] * cells + tr["bytes_per_agent"] * n_agents
    if unit == "launch":
        return tr["bytes_per_launch"]
    return None


def run_ours(args, dist):
    import pphpc_gb300 as pp
    pp.lib()
    dev = dist.local
    p, wname = workload(pp, args)
    n0 = p.init_sheep + p.init_wolves
    # pool: 5x the initial agents for v1 (its population peaks at 4.25x),
    # 40x for v2 (it peaks at 27x to 36x), as the batched and served pools
    cap = (5 if args.params == "v1" else 40) * n0
    K, W = args.steps, args.warmup

    # -- launch geometry from the autotuner (or --tile-cells, or the sort
    # pipeline forced by --sort-pipeline for profiling its kernels) --
    tuning = None
    auto = args.tile_cells == 0 and not args.sort_pipeline
    if auto:
        tuning = pp.autotune(p, SEED, cap, dev)
    sim_kw = dict(device=dev, max_agents=cap, tile_cells=args.tile_cells, autotune=auto,
                  sort_pipeline=args.sort_pipeline)

    # -- device-timed throughput (state resident in HBM) --
    sim = pp.Simulation(p, SEED, **sim_kw)
    sim.step(W)
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    dist.barrier()
    ms = sim.time(K)
    dist.barrier()
    clk = clocks.stop()
    rows = sim.stats_range(W, K)       # rows W..W+K-1 = agents at the start of each timed iteration
    steps_local = float(sum(r.sheep + r.wolves for r in rows))
    ms_max = dist.max(ms)
    steps_all = dist.sum(steps_local)
    value = steps_all / (ms_max / 1e3)
    iters_per_s = K / (ms_max / 1e3)

    # -- per-kernel profile for the roofline --
    prof_iters = min(max(K // 2, 4), 16)
    kernels, prof_steps = sim.profile(prof_iters)
    sim.close()
    kernels = [k for k in kernels if k[1]]
    dom = max(kernels, key=lambda k: k[2])
    name, launches, tot_ms, byts = dom
    peak, peak_kind = measured_peaks()
    cells = p.grid_x * p.grid_y
    n_avg = prof_steps / prof_iters
    spec_b, P = spec_bytes_per_iter(cells, n_avg)
    launch_s = (tot_ms / launches) / 1e3
    achieved = spec_b / launch_s / 1e9
    # the committed DRAM figures are the fused pipeline's kernels
    traffic = None if args.sort_pipeline else kernel_traffic(name, cells, n_avg)
    step_bytes = sum(k[3] for k in kernels) / prof_iters
    step_ms = sum(k[2] for k in kernels) / prof_iters
    timed_spec_bytes = sum(spec_bytes_per_iter(cells, r.sheep + r.wolves)[0] for r in rows)
    naive_bytes = sum(12.0 * cells + 32.0 * (r.sheep + r.wolves) for r in rows)

    # -- end to end through the C ABI with host buffers: the whole job
    # (create, K iterations, stats rows to the host, destroy), run
    # E2E_JOBS times; the median job is reported, every job's time listed --
    e2e_times = []
    for _ in range(E2E_JOBS):
        dist.barrier()
        t0 = time.perf_counter()
        sim2 = pp.Simulation(p, SEED, **sim_kw)
        rows0 = [sim2.stats0()]
        rows_e = sim2.step(K)
        h2d, d2h = sim2.io_bytes()
        sim2.close()
        t1 = time.perf_counter()
        e2e_times.append(dist.max(t1 - t0))
    e2e_steps = float(sum(r.sheep + r.wolves for r in rows0 + rows_e[:-1]))
    e2e_t = sorted(e2e_times)[len(e2e_times) // 2]
    e2e_value = dist.sum(e2e_steps) / e2e_t

    out = {
        "metric": "agent-steps/s", "value": value, "unit": "agent-steps/s",
        "n_gpus": dist.world, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (model's own seeded init)",
        "config": config_of(args, dist.world),
        "setup": {"agent_pool": cap, "state": "uint32 SoA agents, uint16 grass",
                  "geometry": tuning if tuning else {"tile_cells": args.tile_cells,
                                                     "sort_pipeline": args.sort_pipeline}},
        "iters_per_s": iters_per_s,
        "e2e": {"value": e2e_value, "unit": "agent-steps/s",
                "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "includes": "pp_sim_create + %d iterations + stats to host + destroy" % K,
                "jobs_ms": [1e3 * x for x in e2e_times],
                "statistic": "median of %d jobs" % E2E_JOBS},
        "gpu_launches": None,
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "dram_achieved": traffic / launch_s / 1e9 if traffic else None,
                     "dram_frac": traffic / launch_s / 1e9 / peak if traffic else None,
                     "algorithmic_bytes_per_launch": spec_b,
                     "algorithmic_bytes": "12 C + (32 + 16 P) N, P = %d, N = %.0f" % (P, n_avg),
                     "avg_launch_ms": tot_ms / launches,
                     "note": "frac: the reference-shaped step's bytes over the launch "
                             "time; dram_frac: the kernel's measured DRAM bytes "
                             "(traffic) over the same time"},
        "timed_roofline": {"algorithmic_bytes": timed_spec_bytes,
                           "achieved_gbs": timed_spec_bytes / (ms_max / 1e3) / 1e9,
                           "frac": timed_spec_bytes / (ms_max / 1e3) / 1e9 / peak,
                           "note": "same per-iteration figure over the K timed "
                                   "iterations and their whole device time"},
        "naive_step": {"bytes": naive_bytes,
                       "gbs_equivalent": naive_bytes / (ms_max / 1e3) / 1e9,
                       "note": "12 C + 32 N per timed iteration: a step that streams "
                               "every cell's grass and offsets and every agent in and "
                               "out once; not a bound for this design, which reads "
                               "only occupied cells' grass (kernel_bytes)"},
        "kernel_bytes": {"moved_bytes_per_step": step_bytes,
                         "kernel_ms_per_step": step_ms,
                         "design_gbs": step_bytes / (step_ms / 1e3) / 1e9,
                         "note": "bytes the kernels must move in this design "
                                 "(records in and out, occupied cells' grass) over "
                                 "their time; not a DRAM measurement"},
        "kernels": [{"name": k[0], "launches": k[1], "ms": k[2], "design_bytes": k[3],
                     "design_gbs": (k[3] / (k[2] / 1e3) / 1e9) if k[2] > 0 else None}
                    for k in kernels],
        "clocks": clk,
    }
    launches_per_iter = sum(k[1] for k in kernels) // prof_iters
    out["gpu_launches"] = K * launches_per_iter
    if not args.no_full_run:
        out["full_run"] = full_run(args, dist, p, cap)
    if args.batch_iters > 0:
        out["batched"] = batched_vs_plain(args, dist)
    if dist.rank == 0 and not args.no_configs:
        out["configs"] = run_configs(args, dist)["configs"]
    if dist.rank == 0 and args.served_requests > 0:
        out["served"] = run_served(args, dist)
    if dist.rank == 0 and not args.no_cpu_baseline:
        wl, _ = workload_dict(args)
        r = cpu_sample(wl, args.cpu_steps, W)
        out["cpu_baseline"] = {"value": r["value"], "unit": "agent-steps/s",
                               "cores": r["cores"], "kind": r["kind"], "sample": r["sample"]}
    return out


def full_run(args, dist, p, cap):
    """The whole configured run (all its iterations) of the plain workload:
    end to end through the C ABI (create, every iteration, every stats row
    to the host, destroy) and device-timed (CUDA events over all
    iterations, state resident)."""
    import pphpc_gb300 as pp
    dev = dist.local
    kw = dict(device=dev, max_agents=cap, tile_cells=args.tile_cells,
              autotune=args.tile_cells == 0 and not args.sort_pipeline,
              sort_pipeline=args.sort_pipeline)
    dist.barrier()
    t0 = time.perf_counter()
    sim = pp.Simulation(p, SEED, **kw)
    rows = [sim.stats0()] + sim.step(p.iters)
    sim.close()
    wall = dist.max(time.perf_counter() - t0)
    steps = dist.sum(float(sum(r.sheep + r.wolves for r in rows[:-1])))
    sim = pp.Simulation(p, SEED, **kw)
    ms = dist.max(sim.time(p.iters))
    sim.close()
    n = [r.sheep + r.wolves for r in rows]
    return {"iterations": p.iters, "agent_steps": steps,
            "e2e_s": wall, "e2e_agent_steps_per_s": steps / wall,
            "e2e_iters_per_s": p.iters / wall,
            "device_ms": ms, "device_agent_steps_per_s": steps / (ms / 1e3),
            "device_ms_per_iter": ms / p.iters,
            "agents_first_last_peak": [n[0], n[-1], max(n)],
            "peak_at_iteration": n.index(max(n)),
            "includes": "e2e: pp_sim_create + %d iterations + %d stats rows to host "
                        "+ destroy; device: CUDA events around the %d iterations"
                        % (p.iters, p.iters + 1, p.iters)}


def batched_vs_plain(args, dist):
    """The 64-run mix through pp_batch_run (one world) and run by run
    through pp_sim_* (one world per run), both end to end with host stats
    buffers; aggregate agent-steps/s of each, whether every run's stats
    agree bit for bit, and the plain times per shape. The largest shape's
    runs fill the GPU alone, so the plain time of that shape bounds what
    batching can save."""
    import pphpc_gb300 as pp
    iters = args.batch_iters
    runs = []
    seed = 100
    for side, version, n in MIX:
        for _ in range(n):
            runs.append((scaled_params(pp, side, version, iters), seed))
            seed += 1
    dev = dist.local
    # geometries from the autotuner, measured once per workload shape before
    # the timed regions (the library caches them)
    tune_b = pp.batch_autotune(runs, POOL_FACTOR, dev)
    tune_p = {}
    for p, sd in runs:
        key = (p.grid_x, p.sheep_gain_from_food)
        if key not in tune_p:
            tune_p[key] = pp.autotune(p, sd, POOL_FACTOR * (p.init_sheep + p.init_wolves), dev)
    dist.barrier()
    t0 = time.perf_counter()
    out_b = pp.batch_run(runs, pool_factor=POOL_FACTOR, device=dev, autotune=True)
    t1 = time.perf_counter()
    out_p, t_p = [], []
    for p, sd in runs:
        n0 = p.init_sheep + p.init_wolves
        ta = time.perf_counter()
        out_p.append(pp.run(p, sd, device=dev, max_agents=POOL_FACTOR * n0, autotune=True))
        t_p.append(time.perf_counter() - ta)
    t2 = time.perf_counter()
    steps = 0
    exact = True
    run_steps = []
    for rb, rp in zip(out_b, out_p):
        st = sum(r.sheep + r.wolves for r in rb[:-1])
        run_steps.append(st)
        steps += st
        exact &= [r.as_tuple() for r in rb] == [r.as_tuple() for r in rp]
    tb = dist.max(t1 - t0)
    tp = dist.max(t2 - t1)
    steps_all = dist.sum(float(steps))
    shapes, k = [], 0
    for side, version, n in MIX:
        st = float(sum(run_steps[k:k + n]))
        sec = float(sum(t_p[k:k + n]))
        shapes.append({"shape": "%dx%d v%d" % (side, side, version), "runs": n,
                       "agent_steps": st, "plain_s": sec,
                       "plain_agent_steps_per_s": st / sec if sec > 0 else None,
                       "share_of_agent_steps": st / max(steps, 1)})
        k += n
    big = max(shapes, key=lambda d: d["agent_steps"])
    return {"runs": len(runs), "iterations": iters,
            "mix": "32x200^2 v1, 16x800^2 v2, 8x1600^2 v1, 8x3200^2 v2, seeds 100..163",
            "agent_steps": steps_all,
            "batched_s": tb, "plain_s": tp,
            "batched_agent_steps_per_s": steps_all / tb,
            "plain_agent_steps_per_s": steps_all / tp,
            "speedup": tp / tb, "bit_exact_batched_vs_plain": bool(exact),
            "per_shape_plain": shapes,
            "largest_shape": big["shape"],
            "largest_shape_share": big["share_of_agent_steps"],
            "speedup_if_small_runs_free": tp / big["plain_s"],
            "speedup_at_batched_rate_if_small_runs_free":
                tp / (big["agent_steps"] / (steps_all / tb)),
            "speedup_bound_note": "the largest shape's runs fill the GPU alone; with every "
                                  "other run free, the plain time would fall to theirs "
                                  "(speedup_if_small_runs_free), or to their agent-steps at "
                                  "the batched world's own rate",
            "geometry_batched": tune_b,
            "geometry_plain": {"%dx%d %s" % (k_[0], k_[0], "v1" if k_[1] == 4 else "v2"): v
                               for k_, v in tune_p.items()},
            "timing": "wall clock, end to end through the C ABI (create, "
                      "iterations, stats rows to host, destroy)"}


def run_configs(args, dist):
    """The reference's two small plain configs (100^2 v1 seed 0 and 400^2
    v2 seed 1, 4000 iterations), each run whole on the GPU (end to end
    through pp_sim_*, tuned geometry) and by the reference's CPU kernels
    on all host threads."""
    import pphpc_gb300 as pp
    from oracle import pp_ref
    if dist.rank != 0:
        return None
    out = {"workload": "configs", "metric": "agent-steps/s", "unit": "agent-steps/s",
           "n_gpus": 1, "configs": []}
    for side, version, seed in ((100, 1, 0), (400, 2, 1)):
        p = scaled_params(pp, side, version, 4000)
        n0 = p.init_sheep + p.init_wolves
        pp.autotune(p, seed, POOL_FACTOR * n0, dist.local)
        t0 = time.perf_counter()
        rows = pp.run(p, seed, device=dist.local, max_agents=POOL_FACTOR * n0, autotune=True)
        tg = time.perf_counter() - t0
        steps_g = sum(r.sheep + r.wolves for r in rows[:-1])
        c = {"config": "%dx%d v%d seed %d, 4000 iterations" % (side, side, version, seed),
             "gpu_agent_steps_per_s": steps_g / tg, "gpu_iters_per_s": 4000 / tg,
             "timing": "wall clock of the whole run (GPU: create, 4000 iterations, "
                       "stats to host, destroy; CPU: create, init, 4000 iterations)"}
        if pp_ref.available():
            t0 = time.perf_counter()
            crow = pp_ref.run(p, seed)
            tc = time.perf_counter() - t0
            steps_c = float(crow[:-1, 0].sum() + crow[:-1, 1].sum())
            s_ = pp_ref.Sim(p, seed, 1)
            cores = s_.threads()
            s_.close()
            c.update(cpu_agent_steps_per_s=steps_c / tc, cpu_iters_per_s=4000 / tc,
                     cpu_cores=cores, cpu_kind="reference")
        out["configs"].append(c)
    return out


def run_served(args, dist):
    """The served workload: Poisson arrivals into pp_serve_*; returns p50 /
    p99 completion latency and aggregate agent-steps/s."""
    import random
    import pphpc_gb300 as pp
    if dist.rank != 0:
        return None
    rng = random.Random(20)
    n_req = args.served_requests
    t_arr = 0.0
    reqs = []
    for i in range(n_req):
        t_arr += rng.expovariate(20.0)
        side = rng.choice([100, 200, 400, 800, 1600, 3200])
        version = 1 if rng.random() < 0.5 else 2
        iters = rng.randint(500, 4000)
        reqs.append((t_arr, scaled_params(pp, side, version, iters), 1000 + i))
    srv = pp.Server(mem_budget_bytes=150 << 30, max_runs=1024, pool_factor=POOL_FACTOR,
                    stats_chunk=64, device=dist.local, tile_cells=args.served_tile)
    pending = {}
    lat = []
    steps = 0
    nxt = 0
    t0 = time.perf_counter()
    while len(lat) < n_req:
        now = time.perf_counter() - t0
        while nxt < n_req and reqs[nxt][0] <= now:
            a, p, sd = reqs[nxt]
            pending[srv.submit(p, sd)] = a
            nxt += 1
        if not pending:
            time.sleep(max(0.0, reqs[nxt][0] - now))
            continue
        srv.poll(args.served_poll)
        now = time.perf_counter() - t0
        for rid in srv.finished():
            ev = srv.status(rid)
            if ev.status != 0:
                raise RuntimeError("request %d failed (%d)" % (rid, ev.status))
            rows = srv.read(rid)
            steps += sum(r.sheep + r.wolves for r in rows[:-1])
            lat.append(now - pending.pop(rid))
            srv.release(rid)
    wall = time.perf_counter() - t0
    srv.close()
    lat.sort()
    q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))]
    return {"metric": "completion latency", "workload": "served",
            "requests": n_req, "arrival_rate_per_s": 20.0,
            "p50_s": q(0.50), "p99_s": q(0.99), "mean_s": sum(lat) / len(lat),
            "agent_steps": steps, "wall_s": wall,
            "agent_steps_per_s": steps / wall, "unit": "s",
            "higher_is_better": False, "n_gpus": 1,
            "last_arrival_s": reqs[-1][0],
            "config": {"workload": "served: Poisson 20/s, side in {100..3200}, "
                                   "v1/v2 p=0.5, iters U[500,4000], 150 GB budget"}}


def run_reference(args, dist):
    """The reference's own CPU algorithm on the workload and window of the
    GPU arm, rank 0 only."""
    if dist.rank != 0:
        return None
    from oracle import pp_ref
    wl, _ = workload_dict(args)
    if not pp_ref.available():
        return {"impl": "reference",
                "unavailable": "the reference's CPU kernels could not be built "
                               "(no reference tree and no preprocessed copy)"}
    r = cpu_sample(wl, args.steps, args.warmup)
    return {
        "impl": "reference", "metric": "agent-steps/s", "value": r["value"],
        "unit": "agent-steps/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (model's own seeded init)",
        "config": config_of(args, dist.world),
        "cpu_baseline": {"value": r["value"], "unit": "agent-steps/s",
                         "cores": r["cores"], "kind": r["kind"], "sample": r["sample"]},
        "e2e": {"value": r["value"], "unit": "agent-steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=10,
                    help="timed iterations of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-full-run", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--batch-iters", type=int, default=4000,
                    help="iterations per run of the batched-vs-plain mix (0 = skip)")
    ap.add_argument("--workload", choices=["plain", "served", "configs"], default="plain")
    ap.add_argument("--served-requests", type=int, default=1000,
                    help="requests of the served stream (0 = skip the leg)")
    ap.add_argument("--served-tile", type=int, default=0,
                    help="cells per tile of the served world (0 = the library's default)")
    ap.add_argument("--served-poll", type=int, default=16,
                    help="iterations the served loop advances per poll")
    ap.add_argument("--side", type=int, default=12800,
                    help="grid side of the plain workload (agents scale by area)")
    ap.add_argument("--sort-pipeline", action="store_true",
                    help="run the plain workload on the per-iteration sort pipeline "
                         "(for profiling its kernels; no autotuning)")
    ap.add_argument("--params", choices=["v1", "v2"], default="v1",
                    help="parameter set of the plain workload")
    ap.add_argument("--tile-cells", type=int, default=0,
                    help="cells per act tile (0 = the library's choice)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        elif args.workload == "served":
            out = run_served(args, dist)
        elif args.workload == "configs":
            out = run_configs(args, dist)
        else:
            out = run_ours(args, dist)
        if dist.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
