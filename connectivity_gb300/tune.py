"""Size-class tuning tables for the run's tunables.

The device autotuner (``gb_tune`` / ``gb_tune_batch``) times runs of one
graph or batch and returns the best options for it.  This module runs it on
one seeded R-MAT graph per size class and keeps the winners in a JSON table;
``opts_for`` then picks the options of the class nearest a graph's size (by
log2 of the vertex count), and ``install`` gives a context the table, so its
runs without options use their class's options.  Labels never depend on the
options.

    python -m connectivity_gb300.tune [out.json]

tunes every class on the current GPU and writes the table (by default over
tables/classes_scc.json, the table ``install`` reads).
"""
from __future__ import annotations

import json
import math
import os
import sys

from . import Batch, Context, Graph, Opts, opts

# (vertices, edge factor) of the classes tuned by default
CLASSES = [(1 << 10, 8), (1 << 12, 16), (1 << 14, 16), (1 << 16, 16), (1 << 18, 16),
           (1 << 20, 16), (1 << 22, 16), (1 << 24, 16)]

TUNED = ("t_block", "t_grid", "k_pull", "alpha", "beta", "grid_blocks", "expand_mode", "small_path",
         "colour_mode")


def opts_to_dict(o: Opts) -> dict:
    return {k: getattr(o, k) for k in TUNED}


def dict_to_opts(d: dict) -> Opts:
    return opts(**{k: d[k] for k in TUNED if k in d})


def tune_classes(ctx: Context, kind: int = 0, classes=CLASSES, reps: int = 3,
                 seed: int = 1) -> dict:
    """{"kind": kind, "classes": [{"n", "edge_factor", "ms", "default_ms", "opts"}]}"""
    out = []
    for n, ef in classes:
        g = Graph.rmat_n(ctx, n, ef, seed)
        o, ms, dms = ctx.tune(g, kind, reps)
        out.append({"n": int(n), "edge_factor": int(ef), "ms": ms, "default_ms": dms,
                    "opts": opts_to_dict(o)})
        g.close()
    return {"kind": int(kind), "classes": out}


def tune_batch(ctx: Context, b: Batch, kind: int = 0, reps: int = 3) -> dict:
    o, ms, dms = ctx.tune(b, kind, reps)
    return {"count": b.count, "n": b.n, "m": b.m, "ms": ms, "default_ms": dms,
            "opts": opts_to_dict(o)}


# vertex-count ranges of the batch size classes: [lo, hi)
SIZE_CLASSES = [(0, 1000), (1000, 10000), (10000, 100000), (100000, 1 << 31)]


def tune_batch_by_class(ctx: Context, ns, efs, seeds, kind: int = 0, reps: int = 2,
                        classes=SIZE_CLASSES) -> dict:
    """Per-size-class tuning of a batch: the graphs of each vertex-count
    class as a batch of their own, tuned (gb_tune_batch), against the
    defaults on the same sub-batch.  When the defaults are within a few
    percent of the tuned options in every class, options chosen per class
    inside one merged run cannot gain more than that."""
    import numpy as np
    ns = np.asarray(ns)
    out = {"classes": []}
    for lo, hi in classes:
        idx = np.flatnonzero((ns >= lo) & (ns < hi))
        if idx.size == 0:
            continue
        b = Batch.rmat(ctx, ns[idx], np.asarray(efs)[idx], np.asarray(seeds)[idx])
        o, ms, dms = ctx.tune(b, kind, reps)
        out["classes"].append({"n_range": [int(lo), int(hi)], "graphs": int(idx.size),
                               "vertices": int(b.n), "edges": int(b.m),
                               "default_ms": round(dms, 4), "tuned_ms": round(ms, 4),
                               "gain": round(1.0 - ms / dms, 4) if dms > 0 else 0.0,
                               "opts": opts_to_dict(o)})
        b.close()
    out["max_gain"] = max((c["gain"] for c in out["classes"]), default=0.0)
    return out


def save(table: dict, path: str) -> None:
    with open(path, "w") as f:
        json.dump(table, f, indent=1)


def load(path: str) -> dict:
    with open(path) as f:
        return json.load(f)


DEFAULT_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tables",
                             "classes_scc.json")


def class_bounds(table: dict) -> list[int]:
    """Upper vertex bound of each class: the geometric midpoint to the next
    class (the last class takes every larger graph)."""
    ns = [int(c["n"]) for c in table.get("classes", [])]
    out = []
    for i, n in enumerate(ns):
        out.append(int(math.sqrt(n * ns[i + 1])) if i + 1 < len(ns) else (1 << 62))
    return out


def install(ctx: Context, table: dict | None = None) -> None:
    """Gives ctx the table's options per size class (gb_ctx_set_class_opts):
    its runs that are given no options then use them.  Default: the committed
    table (tables/classes_scc.json)."""
    if table is None:
        table = load(DEFAULT_TABLE)
    classes = table.get("classes", [])
    ctx.set_class_opts(class_bounds(table), [dict_to_opts(c["opts"]) for c in classes])


def opts_for(table: dict, n: int) -> Opts:
    """Options of the class whose vertex count is nearest n on a log scale
    (the defaults when the table is empty)."""
    classes = table.get("classes", [])
    if not classes:
        return opts()
    ln = math.log2(max(n, 1))
    best = min(classes, key=lambda c: abs(math.log2(max(c["n"], 1)) - ln))
    return dict_to_opts(best["opts"])


def main(argv: list[str]) -> None:
    out = argv[0] if argv else DEFAULT_TABLE
    ctx = Context(0)
    table = tune_classes(ctx, 0)
    table["how"] = ("gb_tune on one seeded R-MAT graph per class (a=0.57 b=0.19 c=0.19, seed 1), "
                    "coordinate descent from the defaults, best of 3 device-timed runs per option set")
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    save(table, out)
    for c in table["classes"]:
        print(f"n={c['n']:>9} default {c['default_ms']:.4f} ms  tuned {c['ms']:.4f} ms  {c['opts']}")
    ctx.close()


if __name__ == "__main__":
    main(sys.argv[1:])
