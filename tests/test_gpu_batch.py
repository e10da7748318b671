"""Batched SCC / WCC: every graph of a batch must get exactly the labels it
gets alone -- from the oracle, and from a per-graph GPU run -- in local ids."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu


def small_batch(count, seed, median=300.0, n_max=20000):
    ns, efs, seeds = gb.batch_sizes(count, seed=seed, median=median, sigma=1.5, n_min=2,
                                    n_max=n_max)
    return ns, efs, seeds


@pytest.mark.parametrize("count,seed", [(1, 1), (7, 2), (300, 3)])
def test_batch_rmat_matches_oracle_per_graph(ctx, count, seed):
    ns, efs, seeds = small_batch(count, seed)
    b = gb.Batch.rmat(ctx, ns, efs, seeds)
    assert b.count == count and b.n == int(ns.sum())
    scc = b.split(ctx.batch_scc(b))
    wcc = b.split(ctx.batch_wcc(b))
    for i in range(count):
        n, s, d = gb.rmat_edges_n(int(ns[i]), int(efs[i]), int(seeds[i]))
        assert np.array_equal(scc[i], oracle.scc(oracle.CpuGraph(n, s, d))), i
        assert np.array_equal(wcc[i], oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))), i
    b.close()


def test_batch_matches_per_graph_gpu_runs(ctx):
    ns, efs, seeds = small_batch(40, 9, median=2000.0, n_max=60000)
    b = gb.Batch.rmat(ctx, ns, efs, seeds)
    lab = b.split(ctx.batch_scc(b))
    for i in range(b.count):
        g = gb.Graph.rmat_n(ctx, int(ns[i]), int(efs[i]), int(seeds[i]))
        assert np.array_equal(lab[i], ctx.scc(g)), i
        g.close()
    b.close()


def test_batch_from_edges_edge_cases(ctx):
    cases = graphs.edge_cases()
    vb, ss, dd = [0], [], []
    for _, n, s, d in cases:
        ss.append(s.astype(np.int64) + vb[-1])
        dd.append(d.astype(np.int64) + vb[-1])
        vb.append(vb[-1] + n)
    b = gb.Batch.from_edges(ctx, np.array(vb), np.concatenate(ss).astype(np.int32),
                            np.concatenate(dd).astype(np.int32))
    for variant in ({}, {"trim_level": 2}, {"t_block": 33, "t_grid": 64},
                    {"alpha": 1e9, "beta": 1e-3, "k_pull": 1}, {"trim_level": 0},
                    {"trim_pairs": 1}, {"expand_mode": 1}, {"fwbw_rounds": 3}):
        scc = b.split(ctx.batch_scc(b, o=gb.opts(**variant)))
        wcc = b.split(ctx.batch_wcc(b, o=gb.opts(**variant)))
        for i, (name, n, s, d) in enumerate(cases):
            assert np.array_equal(scc[i], oracle.scc(oracle.CpuGraph(n, s, d))), (name, variant)
            assert np.array_equal(wcc[i], oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))), name
    b.close()


def test_batch_rejects_cross_graph_edge(ctx):
    with pytest.raises(gb.GBError):
        gb.Batch.from_edges(ctx, np.array([0, 3, 6]), np.array([0, 2], np.int32),
                            np.array([1, 4], np.int32))


def test_batch_device_labels_async(ctx):
    torch = pytest.importorskip("torch")
    ns, efs, seeds = small_batch(50, 11)
    b = gb.Batch.rmat(ctx, ns, efs, seeds)
    want = ctx.batch_scc(b)
    out = torch.full((b.n,), -3, dtype=torch.int32, device="cuda:0")
    for _ in range(2):
        ctx.batch_scc_async(b, out.data_ptr())
    ctx.sync()
    assert np.array_equal(out.cpu().numpy(), want)
    b.close()


def test_sharded_batch_on_two_contexts_equals_one_batch(ctx):
    """Two shards as two contexts on one GPU (run one after the other): every
    graph's labels equal the single batch's and the oracle's."""
    from connectivity_gb300 import shard
    ns, efs, seeds = gb.batch_sizes(300, median=1500.0, n_max=60000)
    graphs = [gb.rmat_edges_n(int(n), int(e), int(s)) for n, e, s in zip(ns, efs, seeds)]
    whole = shard.run_shard(ctx, graphs, 0)
    c2 = [gb.Context(0), gb.Context(0)]
    parts = shard.run_sharded(c2, graphs, 0)
    wparts = shard.run_sharded(c2, graphs, 1)
    for c in c2:
        c.close()
    for i, g in enumerate(graphs):
        assert np.array_equal(parts[i], whole[i])
        if i % 10 == 0:
            assert np.array_equal(parts[i], oracle.scc(oracle.CpuGraph(*g)))
            assert np.array_equal(wparts[i], oracle.cc(oracle.CpuGraph(*g, mirror=True)))
