"""Failure paths of the run kernel, made without faulting the GPU: a device
step cap that runs out.  Every fixed-point loop of the run kernel checks the
cap in lockstep on all blocks; the block that stops sets the error word,
whose bit in the grid-barrier word releases every other block.  The host
must read GB_ERR_ITER_LIMIT, and the same context must then give correct
labels.  The one-block path (graphs of at most 6144 vertices) caps its
loops the same way."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu

CASES = {name: (n, s, d) for name, n, s, d in graphs.edge_cases()}


@pytest.mark.parametrize("case", ["path_1000", "cycle_1000"])
@pytest.mark.parametrize("kind", ["scc", "wcc"])
def test_step_cap_reports_iter_limit_then_context_recovers(ctx, case, kind):
    n, s, d = CASES[case]
    g = gb.Graph.from_edges(ctx, n, s, d)
    fn = ctx.scc if kind == "scc" else ctx.wcc
    for _ in range(2):
        with pytest.raises(gb.GBError) as e:
            fn(g, o=gb.opts(max_steps=2, small_path=0, wcc_mode=0))
        assert e.value.status == 5, str(e.value)  # GB_ERR_ITER_LIMIT
        lab = fn(g)
        want = (oracle.scc(oracle.CpuGraph(n, s, d)) if kind == "scc"
                else oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)))
        assert np.array_equal(lab, want)
    g.close()


def test_step_cap_in_async_runs_is_reported_by_sync(ctx):
    """An asynchronous run that hits the cap is reported by the next
    gb_ctx_sync; the runs queued after it are unaffected."""
    torch = pytest.importorskip("torch")
    n, s, d = CASES["cycle_1000"]
    g = gb.Graph.from_edges(ctx, n, s, d)
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    ctx.scc_async(g, out.data_ptr(), gb.opts(max_steps=2, small_path=0))
    with pytest.raises(gb.GBError) as e:
        ctx.sync()
    assert e.value.status == 5
    ctx.scc_async(g, out.data_ptr(), gb.opts(small_path=0))
    ctx.sync()
    assert out.cpu().numpy().tolist() == [0] * n
    g.close()


def test_step_cap_in_a_batch(ctx):
    parts = [CASES["cycle_1000"], CASES["path_1000"], CASES["test_graph"]]
    vbase = np.cumsum([0] + [p[0] for p in parts]).astype(np.int64)
    src = np.concatenate([p[1] + vbase[i] for i, p in enumerate(parts)]).astype(np.int32)
    dst = np.concatenate([p[2] + vbase[i] for i, p in enumerate(parts)]).astype(np.int32)
    b = gb.Batch.from_edges(ctx, vbase, src, dst)
    with pytest.raises(gb.GBError) as e:
        ctx.batch_scc(b, o=gb.opts(max_steps=2))
    assert e.value.status == 5
    lab = ctx.batch_scc(b)
    for i, (n, s, d) in enumerate(parts):
        assert np.array_equal(lab[vbase[i]:vbase[i + 1]], oracle.scc(oracle.CpuGraph(n, s, d)))
    b.close()


@pytest.mark.parametrize("case", ["path_1000", "cycle_1000"])
def test_step_cap_in_the_one_block_path(ctx, case):
    """The one-block path's loops (trim, searches, colour rounds) stop at
    the cap with GB_ERR_ITER_LIMIT, from a device graph and from edges; the
    next run on the same context is correct."""
    n, s, d = CASES[case]
    g = gb.Graph.from_edges(ctx, n, s, d)
    want = oracle.scc(oracle.CpuGraph(n, s, d))
    for _ in range(2):
        with pytest.raises(gb.GBError) as e:
            ctx.scc(g, o=gb.opts(max_steps=2, small_path=1))
        assert e.value.status == 5
        with pytest.raises(gb.GBError) as e:
            ctx.scc_edges(n, s, d, o=gb.opts(max_steps=2))
        assert e.value.status == 5
        assert np.array_equal(ctx.scc(g), want)
        assert np.array_equal(ctx.scc_edges(n, s, d), want)
    g.close()
