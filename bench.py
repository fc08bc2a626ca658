"""Benchmark of the PPHPC simulation step on GB300.

Workload: plain PPHPC, 12800 x 12800 toroidal grid (163.84 M cells),
parameter set v1 scaled by area (6,553,600 sheep, 3,276,800 wolves),
seed 2, agent pool 5x the initial agents (the v1 population peaks at 4.25x
the initial agents near iteration 147), uint32 SoA agents, uint16 grass.
A "step" is one simulation iteration over the whole grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       W untimed iterations, then K iterations timed with CUDA events
            on the simulation's stream (graph replay; state resident in
            HBM; the working set, ~1.6 GB, exceeds the 129 MB L2). value =
            agent-steps / s over all ranks. `e2e` is a whole job through the
            C ABI from the host: pp_sim_create (parameters and run tables
            copied in, state initialised on the GPU), the iterations with
            every stats row copied back to a host buffer, pp_sim_destroy.
            `roofline` comes from per-kernel CUDA events (pp_sim_profile)
            over a few further iterations.
reference:  the CPU restatement of the reference's CPU algorithm
            (oracle/pp_cpu_port.c: row-banded pp_cpu semantics, OpenMP over
            all host cores; the reference itself cannot be built here) on
            the same workload, each step one iteration.
With N > 1 (torchrun), every rank runs an independent replica (the runs
do not exchange data); the timed region is bracketed by barriers and the
slowest rank's time is used.
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
    (profiles/ncu_traffic.json), as bytes per processed unit."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_ours(args, dist):
    import pphpc_gb300 as pp
    pp.lib()
    dev = dist.local
    p = pp.make_params(**WORKLOAD)
    n0 = p.init_sheep + p.init_wolves
    cap = 5 * n0
    K, W = args.steps, args.warmup

    # -- device-timed throughput (state resident in HBM) --
    sim = pp.Simulation(p, SEED, device=dev, max_agents=cap)
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
    dom = max(kernels, key=lambda k: k[2])
    name, launches, tot_ms, byts = dom
    peak, peak_kind = measured_peaks()
    achieved = (byts / launches) / ((tot_ms / launches) / 1e3) / 1e9
    traffic = None
    tr = ncu_traffic().get(name)
    if tr:
        unit = tr.get("per")
        if unit == "agent":
            traffic = tr["bytes_per_unit"] * (prof_steps / prof_iters)
        elif unit == "launch":
            traffic = tr["bytes_per_launch"]
    step_bytes = sum(k[3] for k in kernels) / prof_iters
    step_ms = sum(k[2] for k in kernels) / prof_iters

    # -- end to end through the C ABI with host buffers --
    dist.barrier()
    t0 = time.perf_counter()
    sim2 = pp.Simulation(p, SEED, device=dev, max_agents=cap)
    rows0 = [sim2.stats0()]
    rows_e = sim2.step(K)
    h2d, d2h = sim2.io_bytes()
    sim2.close()
    t1 = time.perf_counter()
    e2e_steps = float(sum(r.sheep + r.wolves for r in rows0 + rows_e[:-1]))
    e2e_t = dist.max(t1 - t0)
    e2e_value = dist.sum(e2e_steps) / e2e_t

    out = {
        "metric": "agent-steps/s", "value": value, "unit": "agent-steps/s",
        "n_gpus": dist.world, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (model's own seeded init)",
        "config": {"workload": WORKLOAD_NAME, "grid": "12800x12800", "params": "v1",
                   "init_sheep": p.init_sheep, "init_wolves": p.init_wolves,
                   "seed": SEED, "agent_pool": cap, "state": "uint32 SoA agents, uint16 grass",
                   "timed_iterations": "%d..%d" % (W + 1, W + K),
                   "l2": "inputs larger than L2 (~1.6 GB working set)",
                   "parallelism": "replicas" if dist.world > 1 else "single"},
        "iters_per_s": iters_per_s,
        "e2e": {"value": e2e_value, "unit": "agent-steps/s",
                "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "includes": "pp_sim_create + %d iterations + stats to host + destroy" % K},
        "gpu_launches": None,
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes_per_launch": byts / launches,
                     "avg_launch_ms": tot_ms / launches},
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "kernel_ms_per_step": step_ms,
                          "achieved_gbs": step_bytes / (step_ms / 1e3) / 1e9,
                          "frac": step_bytes / (step_ms / 1e3) / 1e9 / peak},
        "kernels": [{"name": k[0], "launches": k[1], "ms": k[2], "bytes": k[3],
                     "gbs": (k[3] / (k[2] / 1e3) / 1e9) if k[2] > 0 else None}
                    for k in kernels],
        "clocks": clk,
    }
    passes = next((k[1] for k in kernels if k[0] == "radix_pass"), 0) // prof_iters
    out["gpu_launches"] = K * (3 + passes)
    if dist.rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
    return out


def cpu_baseline(args):
    from oracle import cpu_port
    return cpu_port.baseline_sample(WORKLOAD, SEED, iters=args.cpu_iters)


def run_reference(args, dist):
    if dist.rank != 0:
        return None
    from oracle import cpu_port
    r = cpu_port.run_steps(WORKLOAD, SEED, args.steps, args.warmup)
    return {
        "impl": "reference", "metric": "agent-steps/s", "value": r["value"],
        "unit": "agent-steps/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (model's own seeded init)",
        "config": {"workload": WORKLOAD_NAME, "grid": "12800x12800", "params": "v1",
                   "seed": SEED},
        "cpu_baseline": {"value": r["value"], "unit": "agent-steps/s",
                         "cores": r["cores"], "kind": "port", "sample": r["sample"]},
        "e2e": {"value": r["value"], "unit": "agent-steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        else:
            out = run_ours(args, dist)
        if dist.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
