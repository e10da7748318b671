"""The one-block path for graphs of at most 6144 vertices (small.cu): the
whole pipeline in one thread block -- trim to the fixed point, FW-BW, colour
rounds; WCC by union-find -- from a device graph's CSR (gb_scc / gb_wcc) and
straight from an edge list (gb_scc_edges / gb_wcc_edges).  Labels must equal
the oracle's bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu

MAX_N = 6144
CASES = graphs.edge_cases()


def _want(kind, n, s, d):
    if kind == "scc":
        return oracle.scc(oracle.CpuGraph(n, s, d))
    return oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))


def _check_all(ctx, kind, n, s, d):
    want = _want(kind, n, s, d)
    g = gb.Graph.from_edges(ctx, n, s, d)
    run = ctx.scc if kind == "scc" else ctx.wcc
    lab, st = run(g, o=gb.opts(small_path=2), stats=True)
    assert np.array_equal(lab, want)
    assert st.grid_blocks == 1  # the one-block path ran
    edges = ctx.scc_edges if kind == "scc" else ctx.wcc_edges
    assert np.array_equal(edges(n, s, d), want)
    g.close()
    return want


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("kind", ["scc", "wcc"])
def test_edge_cases(ctx, case, kind):
    name, n, s, d = case
    if n > MAX_N:
        pytest.skip("larger than the one-block path")
    want = _check_all(ctx, kind, n, s, d)
    lab = ctx.scc_edges(n, s, d) if kind == "scc" else ctx.wcc_edges(n, s, d)
    if kind == "scc":
        assert gb.scc_verify(lab) == gb.scc_verify(want)


@pytest.mark.parametrize("n,ef,seed", [(64, 4, 1), (300, 16, 2), (2000, 16, 3), (2000, 32, 4),
                                       (4096, 16, 1), (MAX_N, 8, 5), (MAX_N, 32, 6)])
@pytest.mark.parametrize("kind", ["scc", "wcc"])
def test_rmat(ctx, n, ef, seed, kind):
    _, s, d = gb.rmat_edges_n(n, ef, seed)
    _check_all(ctx, kind, n, s, d)


@pytest.mark.parametrize("side", [8, 16, 32, 64])
def test_grids_with_chains(ctx, side):
    """High-diameter lattices: many trim, search and colour steps."""
    n, s, d = graphs.grid(side)
    assert n <= MAX_N
    for kind in ("scc", "wcc"):
        _check_all(ctx, kind, n, s, d)


@pytest.mark.parametrize("seed", range(10))
def test_random_against_scipy(ctx, seed):
    sp = pytest.importorskip("scipy.sparse")
    csg = pytest.importorskip("scipy.sparse.csgraph")
    r = np.random.default_rng(500 + seed)
    n = int(r.integers(1, MAX_N + 1))
    m = int(r.integers(0, 5 * n))
    s = r.integers(0, n, m).astype(np.int32)
    d = r.integers(0, n, m).astype(np.int32)
    for _ in range(int(r.integers(0, 10))):  # planted cycles
        k = int(r.integers(2, min(60, n) + 1)) if n >= 2 else 1
        cyc = r.choice(n, size=k, replace=False).astype(np.int32)
        s = np.concatenate([s, cyc])
        d = np.concatenate([d, np.roll(cyc, -1)])
    a = sp.csr_matrix((np.ones(s.size, np.int8), (s, d)), shape=(n, n))
    _, lab = csg.connected_components(a, directed=True, connection="strong")
    assert np.array_equal(ctx.scc_edges(n, s, d), oracle.canonical(lab.astype(np.int32)))
    _, lab = csg.connected_components(a, directed=True, connection="weak")
    assert np.array_equal(ctx.wcc_edges(n, s, d), oracle.canonical(lab.astype(np.int32)))


def test_hub_and_long_cycle(ctx):
    """A hub with thousands of edges next to a long cycle: edge-balanced
    steps and many levels in one block."""
    n = MAX_N
    v = np.arange(1, n, dtype=np.int32)
    s = np.concatenate([np.zeros(n - 1, np.int32), v, v])
    d = np.concatenate([v, np.zeros(n - 1, np.int32), np.roll(v, -1)])
    for kind in ("scc", "wcc"):
        _check_all(ctx, kind, n, s, d)


def test_boundary_sizes(ctx):
    """n = 6144 takes the one-block path, n = 6145 the cooperative kernel;
    both give the oracle's labels."""
    for n in (MAX_N, MAX_N + 1):
        _, s, d = gb.rmat_edges_n(n, 8, 9)
        g = gb.Graph.from_edges(ctx, n, s, d)
        lab, st = ctx.scc(g, o=gb.opts(small_path=2), stats=True)
        assert np.array_equal(lab, _want("scc", n, s, d))
        assert (st.grid_blocks == 1) == (n <= MAX_N)
        assert np.array_equal(ctx.scc_edges(n, s, d), lab)
        g.close()


def test_device_edges_and_labels(ctx):
    torch = pytest.importorskip("torch")
    _, s, d = gb.rmat_edges_n(3000, 16, 12)
    ds, dd = torch.from_numpy(s).cuda(), torch.from_numpy(d).cuda()
    out = torch.full((3000,), -1, dtype=torch.int32, device="cuda")
    ctx.scc_edges(3000, (ds.data_ptr(), s.size), (dd.data_ptr(), d.size), labels=out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), _want("scc", 3000, s, d))
    ctx.wcc_edges(3000, (ds.data_ptr(), s.size), (dd.data_ptr(), d.size), labels=out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), _want("wcc", 3000, s, d))


def test_bad_ids_are_refused(ctx):
    s = np.array([0, 1, 5], np.int32)
    d = np.array([1, 2, 0], np.int32)
    for fn in (ctx.scc_edges, ctx.wcc_edges):
        with pytest.raises(gb.GBError) as e:
            fn(3, s, d)
        assert e.value.status == 1
    # and the context still works
    assert ctx.scc_edges(3, s[:2], d[:2]).tolist() == [0, 1, 2]


def test_async_and_canonical_off_use_the_grid(ctx):
    """canonical = 0 (labels as the phases make them) runs the cooperative
    kernel; asynchronous runs on device labels take the one-block path."""
    torch = pytest.importorskip("torch")
    n, s, d = graphs.test_graph()
    g = gb.Graph.from_edges(ctx, n, s, d)
    _, st = ctx.scc(g, o=gb.opts(canonical=0), stats=True)
    assert st.grid_blocks > 1
    out = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    for _ in range(3):
        ctx.scc_async(g, out.data_ptr())
    ctx.sync()
    assert out.cpu().tolist() == [0, 0, 2]
    g.close()


def test_automatic_choice_by_edges(ctx):
    """small_path 1 (the default) takes the one-block path for a device graph
    of at most 65536 edges and the grid above; both give the same labels."""
    for n, ef, want_small in ((3000, 4, True), (6000, 32, False)):
        _, s, d = gb.rmat_edges_n(n, ef, 13)
        g = gb.Graph.from_edges(ctx, n, s, d)
        assert (s.size <= 65536) == want_small
        lab, st = ctx.scc(g, stats=True)
        assert (st.grid_blocks == 1) == want_small
        assert np.array_equal(lab, _want("scc", n, s, d))
        g.close()


def _chain_between_cycles(L):
    n = L + 6
    s = [0, 1, 2, n - 3, n - 2, n - 1, 2]
    d = [1, 2, 0, n - 2, n - 1, n - 3, 3]
    s += list(range(3, 3 + L - 1)) + [3 + L - 1]
    d += list(range(4, 3 + L)) + [n - 3]
    return n, np.array(s, np.int32), np.array(d, np.int32)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_one_block_colour_modes_agree(ctx, mode):
    """The one-block path takes gb_opts.colour_mode: colour rounds to the
    end (0), signature rounds from the start (1), or four colour rounds and
    then signature rounds (2); the labels are the oracle's in each."""
    for n, s, d in (_chain_between_cycles(300), graphs.rmat(11, 8, 6), graphs.grid(40)):
        g = gb.Graph.from_edges(ctx, n, s, d)
        lab = ctx.scc(g, o=gb.opts(small_path=2, colour_mode=mode))
        assert np.array_equal(lab, oracle.scc(oracle.CpuGraph(n, s, d)))
        g.close()


@pytest.mark.parametrize("path", [0, 2])
def test_chain_between_cycles(ctx, path):
    """Two 3-cycles joined by a 4,000-vertex chain: nothing is trimmed, and
    every chain vertex is a component of its own, so colour rounds would
    take one round per chain vertex; the signature rounds that follow the
    first colour rounds finish it.  One-block path and cooperative kernel."""
    n, s, d = _chain_between_cycles(4000)
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab = ctx.scc(g, o=gb.opts(small_path=path))
    assert np.array_equal(lab, oracle.scc(oracle.CpuGraph(n, s, d)))
    g.close()
