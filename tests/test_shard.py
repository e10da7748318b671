"""Sharding a batch of independent graphs over devices (host logic, CPU):
the plan's balance and determinism, and the gather that puts every graph's
labels back in batch order.  The per-shard runs are the batch runs tested
on the GPU; here each shard's labels come from the oracle."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
from connectivity_gb300 import shard
import oracle


@pytest.mark.parametrize("shards", [1, 2, 3, 8])
def test_plan_is_balanced_and_deterministic(shards):
    ns, efs, _ = gb.batch_sizes(5000)
    costs = shard.graph_costs(ns, ns.astype(np.int64) * efs)
    of, load = shard.plan(costs, shards)
    of2, load2 = shard.plan(costs, shards)
    assert np.array_equal(of, of2) and np.array_equal(load, load2)
    assert of.min() >= 0 and of.max() < shards
    for s in range(shards):
        assert load[s] == costs[of == s].sum()
    # largest first, least loaded next: within one graph's cost of the mean
    assert load.max() <= costs.sum() / shards + costs.max()
    assert load.sum() == costs.sum()


def test_plan_edge_cases():
    of, load = shard.plan(np.zeros(0, np.int64), 4)
    assert of.size == 0 and load.tolist() == [0, 0, 0, 0]
    of, load = shard.plan(np.array([5, 5, 5, 5], np.int64), 2)
    assert sorted(load.tolist()) == [10, 10]
    # more shards than graphs: some stay empty
    of, load = shard.plan(np.array([3, 1], np.int64), 4)
    assert sorted(of.tolist()) == [0, 1] and load.tolist() == [3, 1, 0, 0]
    with pytest.raises(gb.GBError):
        shard.plan(np.array([1, -1], np.int64), 2)
    with pytest.raises(gb.GBError):
        shard.plan(np.array([1], np.int64), 0)


def test_gather_restores_batch_order():
    rng = np.random.default_rng(0)
    count, shards = 50, 3
    of = rng.integers(0, shards, count).astype(np.int32)
    labs = [np.full(i + 1, i, np.int32) for i in range(count)]
    parts = [[labs[int(i)] for i in shard.members(of, s)] for s in range(shards)]
    out = shard.gather(parts, of)
    assert all(np.array_equal(a, b) for a, b in zip(out, labs))
    with pytest.raises(ValueError):
        shard.gather(parts[:-1] + [parts[-1][:-1]], of)


def test_union_edges_offsets_ids():
    g = [(3, np.array([0, 1], np.int32), np.array([1, 2], np.int32)),
         (2, np.array([1], np.int32), np.array([0], np.int32))]
    vbase, s, d = shard.union_edges(g)
    assert vbase.tolist() == [0, 3, 5]
    assert s.tolist() == [0, 1, 4] and d.tolist() == [1, 2, 3]


def test_sharded_labels_equal_whole_batch_labels_on_cpu():
    """Split, per-shard oracle runs, gather: the labels of every graph equal
    the graph's own labels."""
    ns, efs, seeds = gb.batch_sizes(40, median=300.0, n_max=5000)
    graphs = [oracle.rmat_edges_n(int(n), int(e), int(s)) for n, e, s in zip(ns, efs, seeds)]
    costs = shard.graph_costs(ns, [g[1].size for g in graphs])
    of, _ = shard.plan(costs, 3)
    parts = []
    for s in range(3):
        parts.append([oracle.scc(oracle.CpuGraph(*graphs[int(i)])) for i in shard.members(of, s)])
    out = shard.gather(parts, of)
    for g, lab in zip(graphs, out):
        assert np.array_equal(lab, oracle.scc(oracle.CpuGraph(*g)))
