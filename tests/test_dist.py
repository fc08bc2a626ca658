"""The multi-process path of bench.py on CPU: replicas exchange no data, so
the only cross-rank operations are the barrier and the max / sum
reductions of the timings and counts (gloo, world size 2), and under
torchrun only rank 0 prints its line."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    out[rank] = (d.max(1.5 + rank), d.sum(10.0 * (rank + 1)), d.rank, d.world)
    d.close()


def test_dist_reductions_world_size_2():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        ps = [ctx.Process(target=_rank_main, args=(r, 2, port, out))
              for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        got = dict(out)
    for r in range(2):
        mx, sm, rank, world = got[r]
        assert (mx, sm, rank, world) == (2.5, 30.0, r, 2)




def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--side", "200",
           "--steps", "2", "--warmup", "3"]
    p = subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["config"]["grid"] == "200x200"
    # the reference's own CPU kernels, when they build here
    sys.path.insert(0, ROOT)
    from oracle import pp_ref
    if pp_ref.available():
        assert d["cpu_baseline"]["kind"] == "reference"
    # the same config object as the GPU arm prints for these arguments
    import argparse
    import bench
    a = argparse.Namespace(side=200, params="v1", steps=2, warmup=3)
    assert d["config"] == bench.config_of(a, 2)


def test_workload_options_name_the_workload():
    """The plain workload's options: --side scales the grid (agents by area),
    --params picks the parameter set, and both arms' config objects say so."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    a = argparse.Namespace(side=12800, params="v1", steps=20, warmup=5)
    wl, name = bench.workload_dict(a)
    assert name == "pphpc-12800x12800-v1" and wl == bench.WORKLOAD
    a = argparse.Namespace(side=3200, params="v2", steps=3, warmup=300)
    wl, name = bench.workload_dict(a)
    assert name == "pphpc-3200x3200-v2"
    assert (wl["grid_x"], wl["init_sheep"], wl["init_wolves"]) == (3200, 409600, 204800)
    assert wl["sheep_gain_from_food"] == bench.V2["sheep_gain_from_food"]
    c = bench.config_of(a, 1)
    assert c["params"] == "v2" and c["timed_iterations"] == "301..303"
