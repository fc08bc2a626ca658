"""Shared helpers for the tests: parameter sets and stats conversion."""
import numpy as np

import pphpc_gb300 as pp

# Parameter sets v1 and v2 of the PPHPC model (values of the reference's
# configs/config<side>v1.txt and v2.txt: gains, thresholds, probabilities,
# grass restart; agents scale with the grid area: 400/200 sheep/wolves per
# 100x100 for v1, 400/200 per 100x100 for v2 as well).
V1 = dict(sheep_gain_from_food=4, sheep_reproduce_threshold=2,
          sheep_reproduce_prob=4, wolves_gain_from_food=20,
          wolves_reproduce_threshold=2, wolves_reproduce_prob=5,
          grass_restart=10)
V2 = dict(sheep_gain_from_food=30, sheep_reproduce_threshold=2,
          sheep_reproduce_prob=10, wolves_gain_from_food=10,
          wolves_reproduce_threshold=2, wolves_reproduce_prob=5,
          grass_restart=15)


def params(side, version=1, iters=100, sheep=None, wolves=None, gx=None, gy=None):
    base = V1 if version == 1 else V2
    gx = side if gx is None else gx
    gy = side if gy is None else gy
    area = gx * gy
    s = area * 400 // 10000 if sheep is None else sheep
    w = area * 200 // 10000 if wolves is None else wolves
    return pp.make_params(init_sheep=s, init_wolves=w, grid_x=gx, grid_y=gy,
                          iters=iters, **base)


def rows_array(rows):
    return np.array([r.as_tuple() for r in rows], dtype=np.uint64)


def first_diff(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return "shape %s vs %s" % (a.shape, b.shape)
    bad = np.nonzero(np.any(a != b, axis=-1) if a.ndim > 1 else a != b)[0]
    if len(bad) == 0:
        return None
    i = int(bad[0])
    return "first difference at %d: %s vs %s" % (i, a[i], b[i])
