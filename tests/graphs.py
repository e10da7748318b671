"""Small hand-made and seeded graphs shared by the tests.  Each case is
(name, n, src, dst) with int32 numpy arrays."""
from __future__ import annotations

import numpy as np

import connectivity_gb300 as gb


def _e(n, pairs):
    a = np.array(pairs, dtype=np.int32).reshape(-1, 2)
    return n, a[:, 0].copy(), a[:, 1].copy()


def test_graph():
    # multistep/test.graph: "3 5" then 0 1 / 1 2 / 0 2 / 1 0 / 0 2
    return _e(3, [(0, 1), (1, 2), (0, 2), (1, 0), (0, 2)])


def cycle(n, offset=0):
    v = np.arange(n, dtype=np.int32)
    return n + offset, (v + offset).astype(np.int32), ((v + 1) % n + offset).astype(np.int32)


def path(n):
    v = np.arange(n - 1, dtype=np.int32)
    return n, v, v + 1


def erdos(n, m, seed):
    r = np.random.default_rng(seed)
    s = r.integers(0, n, m, dtype=np.int64).astype(np.int32)
    d = r.integers(0, n, m, dtype=np.int64).astype(np.int32)
    return n, s, d


def edge_cases():
    out = []
    out.append(("test_graph",) + test_graph())
    out.append(("single_vertex", 1, np.zeros(0, np.int32), np.zeros(0, np.int32)))
    out.append(("no_edges", 17, np.zeros(0, np.int32), np.zeros(0, np.int32)))
    out.append(("self_loops_only",) + _e(4, [(0, 0), (1, 1), (3, 3)]))
    out.append(("two_cycle",) + _e(2, [(0, 1), (1, 0)]))
    out.append(("dup_edges",) + _e(4, [(0, 1), (0, 1), (1, 0), (1, 0), (2, 3), (2, 3), (3, 2)]))
    out.append(("cycle_1000",) + cycle(1000))
    out.append(("path_1000",) + path(1000))
    n, s, d = cycle(300)
    n2, s2, d2 = cycle(500, offset=300)
    out.append(("two_cycles", n2, np.concatenate([s, s2]), np.concatenate([d, d2])))
    # a cycle with a self-loop and a pendant path on each side
    out.append(("cycle_tails",) + _e(9, [(0, 1), (1, 2), (2, 0), (2, 2), (3, 0), (4, 3), (1, 5),
                                         (5, 6), (7, 7), (8, 7), (7, 8)]))
    # star: hub 0 <-> leaves, plus leaf chains
    leaves = np.arange(1, 200, dtype=np.int32)
    out.append(("star", 200, np.concatenate([np.zeros(199, np.int32), leaves]),
                np.concatenate([leaves, np.zeros(199, np.int32)])))
    # DAG: every edge i -> j with i < j
    r = np.random.default_rng(3)
    a = r.integers(0, 400, 2000)
    b = r.integers(0, 400, 2000)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    keep = lo != hi
    out.append(("dag", 400, lo[keep].astype(np.int32), hi[keep].astype(np.int32)))
    # complete digraph on 20 vertices
    ii, jj = np.meshgrid(np.arange(20), np.arange(20))
    keep = ii != jj
    out.append(("complete20", 20, ii[keep].astype(np.int32).ravel(), jj[keep].astype(np.int32).ravel()))
    for i, (nn, mm) in enumerate([(50, 60), (1000, 1500), (1000, 4000), (5000, 5000), (20000, 60000)]):
        out.append((f"erdos_{nn}_{mm}",) + erdos(nn, mm, 100 + i))
    return out


def rmat(scale, ef=16, seed=1):
    return gb.rmat_edges(scale, ef, seed)


def grid(side, seed=2):
    return gb.grid_edges(side, side * side // 10, 64, seed)
