"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

The reference ships no tests or golden vectors, so these fixtures pin the
oracle (regression) and let the GPU tests check full-length runs without
running the oracle on the GPU host:

  config100v1.txt, config400v2.txt, config12800v1.txt
      parameter files in the reference's `KEY = value` format with the
      values of the reference's configs of the same names;
  stats_100v1_s0.npz   4001 stats rows, 100x100 v1, seed 0 (oracle);
  stats_400v2_s1.npz   4001 stats rows, 400x400 v2, seed 1 (oracle);
  stats_small.npz      short runs of small grids and edge cases (oracle);
  philox.npz           Philox4x32-10 words for a few counter/key ranges.

Large fixtures (each one oracle run, minutes to an hour of one CPU core;
made with `python tests/golden/make_golden.py large [name ...]`):

  stats_12800v1_s2_r300.npz  rows 0..300 of 12800x12800 v1, seed 2, pool 5x
      the initial agents (through the population peak near iteration 147),
      and the SHA-256 of the canonical state after iteration 300 (agents'
      cells and type|energy words, then the grass countdowns, as the
      oracle lists them);
  stats_12800v1_s2_full.npz  the same run for all 4000 iterations (several
      hours of one core); written every 250 iterations, so a file from an
      interrupted run holds rows 0..k and `iters_done` = k;
  stats_mix_<side>v<v>_s<seed>.npz  all 4001 rows of one run of each class
      of the 64-run batched mix: 200x200 v1 seed 100, 800x800 v2 seed 132,
      1600x1600 v1 seed 148, 3200x3200 v2 seed 156 (the mix's first run of
      each class).

Run from the repository root: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pp_oracle as orc  # noqa: E402

KEYS = ["INIT_SHEEP", "SHEEP_GAIN_FROM_FOOD", "SHEEP_REPRODUCE_THRESHOLD",
        "SHEEP_REPRODUCE_PROB", "INIT_WOLVES", "WOLVES_GAIN_FROM_FOOD",
        "WOLVES_REPRODUCE_THRESHOLD", "WOLVES_REPRODUCE_PROB", "GRASS_RESTART",
        "GRID_X", "GRID_Y", "ITERS"]
FIELDS = ["init_sheep", "sheep_gain_from_food", "sheep_reproduce_threshold",
          "sheep_reproduce_prob", "init_wolves", "wolves_gain_from_food",
          "wolves_reproduce_threshold", "wolves_reproduce_prob", "grass_restart",
          "grid_x", "grid_y", "iters"]

V1 = dict(sheep_gain_from_food=4, sheep_reproduce_threshold=2, sheep_reproduce_prob=4,
          wolves_gain_from_food=20, wolves_reproduce_threshold=2,
          wolves_reproduce_prob=5, grass_restart=10)
V2 = dict(sheep_gain_from_food=30, sheep_reproduce_threshold=2, sheep_reproduce_prob=10,
          wolves_gain_from_food=10, wolves_reproduce_threshold=2,
          wolves_reproduce_prob=5, grass_restart=15)


def cfg(side, v, iters=4000):
    d = dict(V1 if v == 1 else V2)
    d.update(init_sheep=side * side * 400 // 10000, init_wolves=side * side * 200 // 10000,
             grid_x=side, grid_y=side, iters=iters)
    return d


CONFIGS = {"config100v1": cfg(100, 1), "config400v2": cfg(400, 2),
           "config12800v1": cfg(12800, 1)}

SMALL = [  # name, params, seed, iters
    ("25v1_s0", cfg(25, 1, 500), 0, 500),
    ("50v2_s3", cfg(50, 2, 300), 3, 300),
    ("1x1", dict(cfg(1, 1, 100), init_sheep=5, init_wolves=3), 3, 100),
    ("1x50", dict(cfg(1, 1, 100), grid_x=1, grid_y=50, init_sheep=20, init_wolves=10), 3, 100),
    ("sheep_only", dict(cfg(30, 1, 150), init_wolves=0), 8, 150),
    ("wolves_only", dict(cfg(30, 1, 150), init_sheep=0), 8, 150),
    ("empty", dict(cfg(30, 1, 50), init_sheep=0, init_wolves=0), 8, 50),
]


LARGE = {  # name: (params, seed, iterations, agent pool or 0 for the oracle's default)
    "12800v1_s2_r300": (cfg(12800, 1), 2, 300, 5 * (6553600 + 3276800)),
    "mix_200v1_s100": (cfg(200, 1), 100, 4000, 0),
    "mix_800v2_s132": (cfg(800, 2), 132, 4000, 0),
    "mix_1600v1_s148": (cfg(1600, 1), 148, 4000, 0),
    "mix_3200v2_s156": (cfg(3200, 2), 156, 4000, 0),
}


def state_digest(cell, en, grass):
    """SHA-256 of a canonical state: cells, type|energy words, grass."""
    h = hashlib.sha256()
    for a in (cell, en, grass):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_full_12800(name="12800v1_s2_full", every=250):
    """Rows of the full-length 12800x12800 run, saved every `every`
    iterations. With `--threads` the oracle built with its independent
    loops on OpenMP threads runs it (identical results, several times
    faster; pp_oracle.use_threads)."""
    d, seed, _, pool = LARGE["12800v1_s2_r300"]
    iters = d["iters"]
    st = orc.State(d, seed, capacity=pool)
    rows = [st.stats()]
    path = os.path.join(HERE, "stats_%s.npz" % name)
    for k in range(1, iters + 1):
        rows.append(st.step())
        if k % every == 0 or k == iters:
            tmp = path + ".tmp.npz"
            np.savez_compressed(tmp, rows=np.array(rows, np.uint64),
                                params=np.array([d[f] for f in FIELDS], np.uint32),
                                seed=np.array([seed], np.uint64),
                                pool=np.array([pool], np.uint64),
                                iters_done=np.array([k], np.uint64))
            os.replace(tmp, path)
    st.close()


def make_large(name):
    if name == "12800v1_s2_full":
        return make_full_12800()
    d, seed, iters, pool = LARGE[name]
    st = orc.State(d, seed, capacity=pool)
    rows = [st.stats()]
    for _ in range(iters):
        rows.append(st.step())
    cell, en = st.agents()
    digest = state_digest(cell, en, st.grass())
    st.close()
    np.savez_compressed(os.path.join(HERE, "stats_%s.npz" % name),
                        rows=np.array(rows, np.uint64),
                        params=np.array([d[f] for f in FIELDS], np.uint32),
                        seed=np.array([seed], np.uint64), pool=np.array([pool], np.uint64),
                        state_sha256=np.array(digest))


def write_config(path, d):
    with open(path, "w") as f:
        for k, fld in zip(KEYS, FIELDS):
            f.write("%s = %d\n" % (k, d[fld]))


def main():
    for name, d in CONFIGS.items():
        write_config(os.path.join(HERE, name + ".txt"), d)
    np.savez_compressed(os.path.join(HERE, "stats_100v1_s0.npz"),
                        rows=orc.run(CONFIGS["config100v1"], 0))
    np.savez_compressed(os.path.join(HERE, "stats_400v2_s1.npz"),
                        rows=orc.run(CONFIGS["config400v2"], 1))
    small = {}
    for name, d, seed, iters in SMALL:
        small[name] = orc.run(d, seed, iters)
        small[name + "_params"] = np.array([d[f] for f in FIELDS], np.uint32)
        small[name + "_seed"] = np.array([seed], np.uint64)
    np.savez_compressed(os.path.join(HERE, "stats_small.npz"), **small)
    ph = {}
    for i, (ctr, key) in enumerate([((0, 0, 0, 0), (0, 0)), ((7, 3, 2, 0), (2, 0)),
                                    ((0xfffffffe, 0xffffffff, 0xffffffff, 0xffffffff),
                                     (0xffffffff, 0xffffffff))]):
        ph["ctr%d" % i] = np.array(ctr, np.uint32)
        ph["key%d" % i] = np.array(key, np.uint32)
        ph["out%d" % i] = orc.philox_fill(ctr, key, 64)
    np.savez_compressed(os.path.join(HERE, "philox.npz"), **ph)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "large":
        names = [a for a in sys.argv[2:] if not a.startswith("--")]
        if "--threads" in sys.argv:
            orc.use_threads()
        out = [a.split("=", 1)[1] for a in sys.argv[2:] if a.startswith("--out=")]
        for n in names or sorted(LARGE) + ["12800v1_s2_full"]:
            if n == "12800v1_s2_full" and out:
                make_full_12800(out[0])
            else:
                make_large(n)
    else:
        main()
