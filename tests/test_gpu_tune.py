"""Autotuner: tuned options must keep the labels, and the tuner's best time
is never worse than the defaults' time it measured."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
from connectivity_gb300 import tune
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu


def test_tune_graph_keeps_labels(ctx):
    n, s, d = graphs.rmat(14, 16, 3)
    g = gb.Graph.from_edges(ctx, n, s, d)
    for kind in (0, 1):
        o, ms, dms = ctx.tune(g, kind, reps=2)
        assert 0 < ms <= dms
        assert o.t_grid > o.t_block > 0 and o.k_pull >= 1 and o.alpha > 0 and o.beta > 0
        run = ctx.scc if kind == 0 else ctx.wcc
        want = (oracle.scc(oracle.CpuGraph(n, s, d)) if kind == 0
                else oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)))
        assert np.array_equal(run(g, o=o), want)
    g.close()


def test_tune_batch_and_classes(ctx, tmp_path):
    ns, efs, seeds = gb.batch_sizes(50, seed=6, median=500.0, sigma=1.2, n_min=16, n_max=20000)
    b = gb.Batch.rmat(ctx, ns, efs, seeds)
    rec = tune.tune_batch(ctx, b, 0, reps=2)
    assert rec["ms"] <= rec["default_ms"]
    o = tune.dict_to_opts(rec["opts"])
    lab = b.split(ctx.batch_scc(b, o=o))
    ref = b.split(ctx.batch_scc(b))
    assert all(np.array_equal(x, y) for x, y in zip(lab, ref))
    table = tune.tune_classes(ctx, 0, classes=[(1 << 10, 8), (1 << 13, 16)], reps=1)
    tune.save(table, tmp_path / "t.json")
    back = tune.load(tmp_path / "t.json")
    assert [c["n"] for c in back["classes"]] == [1 << 10, 1 << 13]
    b.close()


def test_class_table_applies_to_runs_without_options(ctx):
    """A context's class table gives runs without options their class's
    options (here: the one-block path off for small graphs, on for larger
    ones); runs given options keep them; labels never change."""
    c2 = gb.Context(0)
    n, s, d = graphs.rmat(11, 8, 2)  # 2,048 vertices
    g = gb.Graph.from_edges(c2, n, s, d)
    want = oracle.scc(oracle.CpuGraph(n, s, d))
    assert c2.scc(g, stats=True)[1].grid_blocks == 1  # no table: the one-block path
    c2.set_class_opts([4096, 1 << 62], [gb.opts(small_path=0), gb.opts()])
    lab, st = c2.scc(g, stats=True)
    assert st.grid_blocks > 1 and np.array_equal(lab, want)
    assert c2.scc(g, o=gb.opts(small_path=2), stats=True)[1].grid_blocks == 1
    assert np.array_equal(c2.scc_edges(n, s, d), want)
    with pytest.raises(gb.GBError):
        c2.set_class_opts([10, 5], [gb.opts(), gb.opts()])
    c2.set_class_opts([], [])
    assert c2.scc(g, stats=True)[1].grid_blocks == 1
    # the committed table, installed
    tune.install(c2)
    assert np.array_equal(c2.scc(g), want)
    g.close()
    c2.close()
