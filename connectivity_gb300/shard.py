"""A batch of independent graphs sharded over devices.

Graphs of a batch share no edge, so a batch splits by graph with no
exchange between shards: every shard (one device, one context, or one rank
of a job) builds the disjoint union of its own graphs and runs it, and the
labels are gathered on the host in the batch's order.  The plan comes from
``gb_shard_plan`` (largest graph first, each to the least loaded shard) and
is deterministic, so the ranks of a job compute it without communicating.
The reference has no counterpart: it runs the graphs one after another
(multistep/scc_main.cpp:210).
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import Batch, Context, _check, _lib, _ptr

_lib.gb_shard_plan.restype = C.c_int32
_lib.gb_shard_plan.argtypes = [C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]


def graph_costs(ns, ms) -> np.ndarray:
    """Work of each graph: vertices + edges (both are passes of the run)."""
    return np.asarray(ns, np.int64) + np.asarray(ms, np.int64)


def plan(costs, shards: int) -> tuple[np.ndarray, np.ndarray]:
    """(shard of each graph, total cost of each shard)."""
    c = np.ascontiguousarray(costs, np.int64)
    of = np.zeros(c.size, np.int32)
    load = np.zeros(shards, np.int64)
    _check(_lib.gb_shard_plan(c.size, _ptr(c), shards, _ptr(of), _ptr(load)), "gb_shard_plan")
    return of, load


def members(shard_of: np.ndarray, shard: int) -> np.ndarray:
    """The graphs of one shard, in batch order."""
    return np.flatnonzero(np.asarray(shard_of) == shard).astype(np.int64)


def gather(parts: list[list[np.ndarray]], shard_of: np.ndarray) -> list[np.ndarray]:
    """Per-graph label arrays in batch order from each shard's per-graph
    arrays (parts[s][k] = labels of the k-th graph of shard s)."""
    shard_of = np.asarray(shard_of)
    out: list[np.ndarray | None] = [None] * shard_of.size
    for s, part in enumerate(parts):
        idx = members(shard_of, s)
        if len(idx) != len(part):
            raise ValueError(f"shard {s}: {len(part)} label arrays for {len(idx)} graphs")
        for i, lab in zip(idx, part):
            out[int(i)] = lab
    if any(x is None for x in out):
        raise ValueError("a graph has no labels")
    return out  # type: ignore[return-value]


def union_edges(graphs) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(vbase, src, dst) of the disjoint union of (n, src, dst) graphs."""
    ns = np.array([g[0] for g in graphs], np.int64)
    vbase = np.zeros(len(graphs) + 1, np.int64)
    np.cumsum(ns, out=vbase[1:])
    src = np.concatenate([np.asarray(g[1], np.int64) + vbase[i] for i, g in enumerate(graphs)]
                         or [np.zeros(0, np.int64)]).astype(np.int32)
    dst = np.concatenate([np.asarray(g[2], np.int64) + vbase[i] for i, g in enumerate(graphs)]
                         or [np.zeros(0, np.int64)]).astype(np.int32)
    return vbase, src, dst


def run_shard(ctx: Context, graphs, kind: int = 0, o=None) -> list[np.ndarray]:
    """One shard: the union of its graphs (n, src, dst) as one batch run on
    ctx's device; labels per graph (local ids)."""
    if not graphs:
        return []
    vbase, src, dst = union_edges(graphs)
    b = Batch.from_edges(ctx, vbase, src, dst)
    try:
        lab = ctx.batch_scc(b, o=o) if kind == 0 else ctx.batch_wcc(b, o=o)
    finally:
        b.close()
    return [lab[vbase[i]:vbase[i + 1]] for i in range(len(graphs))]


def run_sharded(ctxs: list[Context], graphs, kind: int = 0, o=None,
                concurrent: bool = True) -> list[np.ndarray]:
    """A batch over several contexts (one per device): each context runs its
    shard (host threads, one per context, when concurrent), and the labels
    come back in batch order.  Contexts on the same device run their shards
    one after another: each run is a cooperative launch over the whole
    device, and two of them are not made to share it."""
    costs = graph_costs([g[0] for g in graphs], [len(g[1]) for g in graphs])
    shard_of, _ = plan(costs, len(ctxs))
    parts: list[list[np.ndarray] | None] = [None] * len(ctxs)
    errors: list[BaseException] = []

    def work(s: int) -> None:
        try:
            parts[s] = run_shard(ctxs[s], [graphs[int(i)] for i in members(shard_of, s)], kind, o)
        except BaseException as e:  # reported after every shard has finished
            errors.append(e)

    if concurrent and len(ctxs) > 1 and len({c.device for c in ctxs}) == len(ctxs):
        ts = [threading.Thread(target=work, args=(s,)) for s in range(len(ctxs))]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    else:
        for s in range(len(ctxs)):
            work(s)
    if errors:
        raise errors[0]
    return gather(parts, shard_of)  # type: ignore[arg-type]


def gather_ranks(local: list[np.ndarray], shard_of: np.ndarray, rank: int, world: int):
    """Rank 0 receives every rank's per-graph labels (torch.distributed,
    objects over the process group's backend) and returns them in batch
    order; other ranks return None.  The only communication of a sharded
    batch."""
    import torch.distributed as tdist
    got = [None] * world if rank == 0 else None
    tdist.gather_object(local, got, dst=0)
    if rank != 0:
        return None
    return gather(got, shard_of)  # type: ignore[arg-type]
