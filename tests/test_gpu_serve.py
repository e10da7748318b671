"""Serving: a Poisson stream of SCC / WCC requests through gb_server.  Each
request must get exactly the labels its graph gets alone (a per-graph GPU
run and the oracle), whatever it was merged with."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu


def requests(count, seed, median=600.0, n_max=30000, wcc_frac=0.2):
    ns, efs, seeds = gb.batch_sizes(count, seed=seed, median=median, sigma=1.5, n_min=2,
                                    n_max=n_max)
    rng = np.random.default_rng(seed)
    kinds = (rng.random(count) < wcc_frac).astype(np.int32)
    out = []
    for i in range(count):
        n, s, d = gb.rmat_edges_n(int(ns[i]), int(efs[i]), int(seeds[i]))
        out.append((int(kinds[i]), n, s, d))
    return out


def alone(ctx, kind, n, s, d):
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab = ctx.scc(g) if kind == gb.Server.SCC else ctx.wcc(g)
    g.close()
    return lab


@pytest.mark.parametrize("rate,budget", [(5000.0, 0), (50000.0, 64 << 20)])
def test_served_labels_match_alone(ctx, rate, budget):
    reqs = requests(120, seed=11)
    want = [alone(ctx, *r) for r in reqs]
    sctx = gb.Context(0)
    sv = gb.Server(sctx, budget_bytes=budget, max_graphs=64)
    rng = np.random.default_rng(3)
    t = np.cumsum(rng.exponential(1e9 / rate, len(reqs))).astype(np.int64)
    ids = [sv.submit(k, n, s, d, arrival_ns=int(t[i])) for i, (k, n, s, d) in enumerate(reqs)]
    sv.start()
    for i, rid in enumerate(ids):
        lab, lat = sv.wait(rid)
        assert lat >= 0.0
        assert np.array_equal(lab, want[i]), i
    st = sv.stats()
    assert st.completed == len(reqs)
    assert st.batches >= 1 and st.mean_batch >= 1.0
    assert 0.0 <= st.p50_ms <= st.p99_ms <= st.max_ms
    sv.close()
    sctx.close()


def test_served_matches_oracle_and_edge_cases():
    cases = graphs.edge_cases()
    sctx = gb.Context(0)
    sv = gb.Server(sctx, max_graphs=8)
    sv.start()
    ids = []
    for _, n, s, d in cases:
        ids.append((sv.submit(gb.Server.SCC, n, s, d), n, s, d, 0))
        ids.append((sv.submit(gb.Server.WCC, n, s, d), n, s, d, 1))
    for rid, n, s, d, kind in ids:
        lab, _ = sv.wait(rid)
        ref = (oracle.scc(oracle.CpuGraph(n, s, d)) if kind == 0
               else oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)))
        assert np.array_equal(lab, ref), (rid, kind)
    sv.drain()
    sv.close()
    sctx.close()


def test_served_bad_request_is_isolated(ctx):
    reqs = requests(10, seed=5)
    sctx = gb.Context(0)
    sv = gb.Server(sctx, max_graphs=64)
    ids = [sv.submit(k, n, s, d, arrival_ns=0) for k, n, s, d in reqs]
    bad = sv.submit(gb.Server.SCC, 4, np.array([0, 1, 7], np.int32), np.array([1, 0, 2], np.int32),
                    arrival_ns=0)
    sv.start()
    with pytest.raises(gb.GBError) as e:
        sv.wait(bad)
    assert e.value.status == gb.GB_ERR_INVALID
    for rid, r in zip(ids, reqs):
        lab, _ = sv.wait(rid)
        assert np.array_equal(lab, alone(ctx, *r))
    sv.close()
    sctx.close()


def test_server_rejects_oversize_and_bad_arguments():
    sctx = gb.Context(0)
    sv = gb.Server(sctx, budget_bytes=1 << 20, max_graphs=4)
    n, s, d = gb.rmat_edges_n(50000, 16, 1)
    with pytest.raises(gb.GBError) as e:
        sv.submit(gb.Server.SCC, n, s, d)
    assert e.value.status == gb.GB_ERR_CAPACITY
    with pytest.raises(gb.GBError):
        sv.submit(3, 4, np.zeros(1, np.int32), np.zeros(1, np.int32))
    with pytest.raises(gb.GBError):
        sv.submit(gb.Server.SCC, 0, np.zeros(0, np.int32), np.zeros(0, np.int32))
    sv.close()
    sctx.close()


@pytest.mark.parametrize("small_path", [1, 0])
@pytest.mark.parametrize("count,max_graphs", [(40, 64), (700, 700)])
def test_served_one_block_and_union_paths(ctx, small_path, count, max_graphs):
    """Merged sets that mix small requests (one block each) with large ones
    (the union), and sets with more small requests than one launch wave
    (all on the union), all arriving at once: every request gets its labels
    alone."""
    reqs = requests(count, seed=21, median=1500.0, n_max=40000)
    sctx = gb.Context(0)
    sv = gb.Server(sctx, max_graphs=max_graphs)
    sv.set_opts(gb.opts(small_path=small_path))
    ids = [sv.submit(k, n, s, d, arrival_ns=0) for k, n, s, d in reqs]
    sv.start()
    for i, (rid, r) in enumerate(zip(ids, reqs)):
        lab, _ = sv.wait(rid)
        if i % 7 == 0 or r[1] > 6144:
            assert np.array_equal(lab, alone(ctx, *r)), i
    sv.close()
    sctx.close()
