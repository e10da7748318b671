"""Sampled union-find for WCC / CC: gb_run_cc on host arrays the device
reads in place, and gb_wcc on device graphs (directed: the union of the
out- and in-lists; symmetric CSRs).  On cc's mirrored CSR (every vertex links its first neighbour, then
only the vertices outside the sampled largest component link the rest).
Labels must equal the oracle's on every graph, whichever component the
sample picks; bad offsets, and out-of-range ids among the entries it reads,
are refused."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu


def _mirrored(n, s, d):
    mg = oracle.CpuGraph(n, s, d, mirror=True)
    return mg, mg.out_off.astype(np.uint32), mg.out_adj


def _pin(kind):
    torch = pytest.importorskip("torch")
    if kind == "pinned":
        return lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    return lambda a: np.ascontiguousarray(a).copy()


def _two_big_components():
    """Two R-MAT graphs side by side: the sample may pick either."""
    n1, s1, d1 = graphs.rmat(12, 8, 3)
    n2, s2, d2 = graphs.rmat(12, 16, 4)
    return n1 + n2, np.concatenate([s1, s2 + n1]), np.concatenate([d1, d2 + n1])


CASES = [c for c in graphs.edge_cases() if c[1] > 0] + [
    ("rmat14", *graphs.rmat(14, 16, 21)),
    ("grid64", *graphs.grid(64)),
    ("two_big", *_two_big_components()),
    ("isolated", 5000, np.zeros(0, np.int32), np.zeros(0, np.int32)),
]


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_run_cc_sampled_matches_oracle(case, kind):
    name, n, s, d = case
    mg, off, adj = _mirrored(n, s, d)
    pin = _pin(kind)
    lab = gb.run_cc_ref(n, pin(adj if adj.size else np.zeros(1, np.int32)), pin(off))
    assert np.array_equal(lab, oracle.cc(mg)), name


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
def test_run_cc_refuses_a_bad_csr(kind):
    pin = _pin(kind)
    n, s, d = graphs.rmat(11, 8, 2)
    mg, off, adj = _mirrored(n, s, d)
    # an id the union-find reads (a list's first entry) is checked; ids in
    # the skipped part of the largest component's lists are never read
    bad = adj.copy()
    v = int(np.flatnonzero(np.diff(off.astype(np.int64)) > 0)[len(off) // 5 % 7])
    bad[off[v]] = n + 2
    with pytest.raises(gb.GBError) as e:
        gb.run_cc_ref(n, pin(bad), pin(off))
    assert e.value.status == gb.GB_ERR_INVALID
    off2 = off.copy()
    off2[n // 2] = off2[n // 2 + 1] + 1
    with pytest.raises(gb.GBError) as e:
        gb.run_cc_ref(n, pin(adj), pin(off2))
    assert e.value.status == gb.GB_ERR_INVALID
    assert np.array_equal(gb.run_cc_ref(n, pin(adj), pin(off)), oracle.cc(mg))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_wcc_sampled_on_device_graphs(ctx, case):
    """gb_wcc with wcc_mode 1 on a directed device graph and on its
    mirrored, symmetric CSR: the oracle's labels, the same as the
    reference's phases (wcc_mode 0, the default)."""
    name, n, s, d = case
    want = oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab = ctx.wcc(g, o=gb.opts(small_path=0, wcc_mode=1))
    assert np.array_equal(lab, want), name
    assert np.array_equal(ctx.wcc(g, o=gb.opts(small_path=0, wcc_mode=0)), want), name
    g.close()
    mg = oracle.CpuGraph(n, s, d, mirror=True)
    sg = gb.Graph.from_csr(ctx, n, mg.out_off, mg.out_adj)
    assert np.array_equal(ctx.wcc(sg, o=gb.opts(small_path=0, wcc_mode=1)), want), name
    sg.close()
