"""In-lists derived on the device from the out-CSR (gb_graph_from_csr32 with
in_array NULL, and gb_run_scc for a share of the in-edges): the in-lists are
written while the out-lists are read, and the rest of in_array is copied.

Checked: every derived in-list holds the same sources as the transpose
(as a multiset, the order within a list is free), the labels equal the
oracle's whatever in_array holds, and in-offsets that do not describe the
out-CSR's transpose are refused.  The graphs cover the hub path (targets of
at least 2,048 in-edges counted per tile), its overflow (more distinct hubs
in one tile than the shared table holds), ragged tails, long runs of
vertices without out-edges, self-loops and duplicates, and pinned,
unaligned-pinned and pageable inputs."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu


def _star_in(n_src):
    """n_src sources, each with one edge to vertex 0 (a hub far above the
    per-tile threshold); vertex 0 points back at every third source, so
    those form one component with it and the others are trimmed."""
    n = n_src + 1
    back = np.arange(3, n, 3, dtype=np.int32)
    s = np.concatenate([np.arange(1, n, dtype=np.int32), np.zeros(back.size, np.int32)])
    d = np.concatenate([np.zeros(n_src, np.int32), back])
    return n, s, d


def _many_hubs(hubs=1000, sources=2500):
    """Every source points at every hub: each hub has `sources` in-edges
    (above the threshold), and one tile of edges meets about a thousand
    distinct hubs, more than the shared table holds."""
    src = np.repeat(np.arange(hubs, hubs + sources, dtype=np.int32), hubs)
    dst = np.tile(np.arange(hubs, dtype=np.int32), sources)
    # a few hub -> source edges make cycles through the hubs
    back_s = np.arange(0, hubs, 7, dtype=np.int32)
    back_d = (hubs + (back_s * 13) % sources).astype(np.int32)
    return hubs + sources, np.concatenate([src, back_s]), np.concatenate([dst, back_d])


def _sparse_runs():
    """Out-edges only on a few vertices, with runs of thousands of vertices
    without out-edges between them, and a ragged edge count."""
    n = 50000
    rng = np.random.default_rng(3)
    owners = np.sort(rng.choice(n, 40, replace=False)).astype(np.int32)
    deg = rng.integers(1, 3000, owners.size)
    s = np.repeat(owners, deg)
    d = rng.integers(0, n, s.size).astype(np.int32)
    return n, s, d


def _dups_and_loops():
    n, s, d = graphs.erdos(3001, 20011, 12)
    s = np.concatenate([s, s[:500], np.arange(0, 300, dtype=np.int32)])
    d = np.concatenate([d, d[:500], np.arange(0, 300, dtype=np.int32)])
    return n, s, d


GRAPHS = {
    "rmat14": lambda: graphs.rmat(14, 16, 21),
    "star": lambda: _star_in(9000),
    "many_hubs": _many_hubs,
    "sparse_runs": _sparse_runs,
    "dups_loops": _dups_and_loops,
    "one_edge": lambda: (3, np.array([2], np.int32), np.array([0], np.int32)),
    "no_edges": lambda: (5, np.zeros(0, np.int32), np.zeros(0, np.int32)),
    "empty": lambda: (0, np.zeros(0, np.int32), np.zeros(0, np.int32)),
}


def _pinner(kind):
    torch = pytest.importorskip("torch")
    if kind == "pageable":
        return lambda a: np.ascontiguousarray(a)
    if kind == "pinned":
        return lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    def unaligned(a):
        # one element into a pinned buffer: off every 16-byte boundary
        a = np.ascontiguousarray(a)
        raw = torch.empty((a.size + 1) * a.itemsize, dtype=torch.uint8).pin_memory().numpy()
        buf = raw.view(a.dtype)
        buf[1:] = a
        return buf[1:]
    return unaligned


def _sorted_lists(off, adj):
    """Each vertex's list sorted, so lists compare as multisets."""
    out = adj.copy()
    for v in range(off.size - 1):
        a, b = off[v], off[v + 1]
        if b - a > 1:
            out[a:b] = np.sort(out[a:b])
    return out


@pytest.mark.parametrize("kind", ["pinned", "unaligned", "pageable"])
@pytest.mark.parametrize("name", list(GRAPHS))
def test_derived_in_lists_are_the_transpose(ctx, name, kind):
    n, s, d = GRAPHS[name]()
    cg = oracle.CpuGraph(n, s, d)
    pin = _pinner(kind)
    g = gb.Graph.from_csr32(ctx, n, pin(cg.out_adj), pin(cg.out_off.astype(np.uint32)),
                            None, pin(cg.in_off.astype(np.uint32)))
    oo, oa, io, ia = g.to_host()
    assert np.array_equal(oo, cg.out_off) and np.array_equal(oa, cg.out_adj)
    assert np.array_equal(io, cg.in_off)
    assert np.array_equal(_sorted_lists(io, ia), _sorted_lists(cg.in_off, cg.in_adj)), name
    lab = ctx.scc(g, o=gb.opts(small_path=0))
    assert np.array_equal(lab, oracle.scc(cg)), name
    g.close()


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
@pytest.mark.parametrize("share", [1.0, 0.75, 0.3, 0.0])
def test_run_scc_split_between_derived_and_copied(kind, share):
    """gb_run_scc derives the in-lists of the first `share` of the in-edges
    and copies the rest of in_array: the oracle's labels at every share; at
    share 1 in_array is not read (garbage or NULL), and NULL in_array always
    means derive everything."""
    pin = _pinner(kind)
    gb.dropin_set_derive_share(share)
    try:
        for n, s, d in (graphs.rmat(13, 16, 31), _star_in(5000), _many_hubs(600, 2200),
                        _sparse_runs()):
            cg = oracle.CpuGraph(n, s, d)
            odl, idl = pin(cg.out_off.astype(np.uint32)), pin(cg.in_off.astype(np.uint32))
            oa = pin(cg.out_adj)
            want = oracle.scc(cg)
            assert np.array_equal(gb.run_scc_ref(n, oa, pin(cg.in_adj), odl, idl), want)
            assert np.array_equal(gb.run_scc_ref(n, oa, None, odl, idl), want)
            if share == 1.0:
                junk = pin(np.full(max(cg.m, 1), 7, np.int32))
                assert np.array_equal(gb.run_scc_ref(n, oa, junk, odl, idl), want)
    finally:
        gb.dropin_set_derive_share(0.8)
    with pytest.raises(gb.GBError) as e:
        gb.dropin_set_derive_share(1.5)
    assert e.value.status == gb.GB_ERR_INVALID


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
def test_bad_id_in_the_copied_in_lists_is_refused(kind):
    """With a split, the copied part of in_array is checked for ids outside
    [0, n)."""
    pin = _pinner(kind)
    n, s, d = graphs.rmat(12, 16, 8)
    cg = oracle.CpuGraph(n, s, d)
    odl, idl = pin(cg.out_off.astype(np.uint32)), pin(cg.in_off.astype(np.uint32))
    oa = pin(cg.out_adj)
    ia = pin(cg.in_adj.copy())
    ia[-3] = n + 9  # in the copied tail at any share below 1
    gb.dropin_set_derive_share(0.5)
    try:
        with pytest.raises(gb.GBError) as e:
            gb.run_scc_ref(n, oa, ia, odl, idl)
        assert e.value.status == gb.GB_ERR_INVALID
        ia[-3] = cg.in_adj[-3]
        assert np.array_equal(gb.run_scc_ref(n, oa, ia, odl, idl), oracle.scc(cg))
    finally:
        gb.dropin_set_derive_share(0.8)


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
def test_in_offsets_that_do_not_match_are_refused(kind):
    """In-offsets that are monotone and end at m but move an in-edge from
    one vertex to another (or to the hub) are not the transpose's: refused,
    and the next call with the right offsets works."""
    pin = _pinner(kind)
    for n, s, d in (graphs.rmat(13, 16, 31), _star_in(5000)):
        cg = oracle.CpuGraph(n, s, d)
        odl, idl = pin(cg.out_off.astype(np.uint32)), pin(cg.in_off.astype(np.uint32))
        oa = pin(cg.out_adj)
        deg = np.diff(cg.in_off)
        for i in (0, int(np.flatnonzero(deg > 1)[-1])):
            if deg[i] == 0:
                continue
            j = (i + 1) % n
            bad = cg.in_off.copy()
            if j > i:
                bad[i + 1:j + 1] -= 1  # vertex i loses an in-edge, vertex j gains one
            assert (np.diff(bad) >= 0).all() and bad[-1] == cg.in_off[-1]
            if np.array_equal(bad, cg.in_off):
                continue
            with pytest.raises(gb.GBError) as e:
                gb.run_scc_ref(n, oa, None, odl, pin(bad.astype(np.uint32)))
            assert e.value.status == gb.GB_ERR_INVALID
        assert np.array_equal(gb.run_scc_ref(n, oa, None, odl, idl), oracle.scc(cg))
    # a bad out-list id and non-monotone in-offsets
    n, s, d = graphs.rmat(10, 8, 3)
    cg = oracle.CpuGraph(n, s, d)
    odl, idl = pin(cg.out_off.astype(np.uint32)), pin(cg.in_off.astype(np.uint32))
    oa = pin(cg.out_adj.copy())
    oa[len(oa) // 2] = n + 5
    with pytest.raises(gb.GBError) as e:
        gb.run_scc_ref(n, oa, None, odl, idl)
    assert e.value.status == gb.GB_ERR_INVALID
    oa[len(oa) // 2] = cg.out_adj[len(oa) // 2]
    idl2 = pin(cg.in_off.astype(np.uint32))
    k = int(np.flatnonzero(np.diff(cg.in_off) > 0)[0])
    idl2[k + 1] = idl2[k] - 1 if idl2[k] > 0 else np.uint32(cg.m + 1)
    with pytest.raises(gb.GBError) as e:
        gb.run_scc_ref(n, oa, None, odl, idl2)
    assert e.value.status == gb.GB_ERR_INVALID
    assert np.array_equal(gb.run_scc_ref(n, oa, None, odl, idl), oracle.scc(cg))


def test_device_arrays_take_the_staged_derivation(ctx):
    """A CSR already in device memory is staged on the device (no host view)
    and the in-lists are derived from the staged out-lists: the transpose's
    lists, and the oracle's labels."""
    torch = pytest.importorskip("torch")
    for n, s, d in (graphs.rmat(13, 16, 31), _star_in(5000), _sparse_runs()):
        cg = oracle.CpuGraph(n, s, d)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
        oa = dev(cg.out_adj)
        odl = dev(cg.out_off.astype(np.int64)).to(torch.int32)
        idl = dev(cg.in_off.astype(np.int64)).to(torch.int32)
        g = gb.Graph.from_csr32(ctx, n, oa, odl, None, idl)
        oo, oa2, io, ia = g.to_host()
        assert np.array_equal(oa2, cg.out_adj) and np.array_equal(io, cg.in_off)
        assert np.array_equal(_sorted_lists(io, ia), _sorted_lists(cg.in_off, cg.in_adj))
        assert np.array_equal(ctx.scc(g, o=gb.opts(small_path=0)), oracle.scc(cg))
        g.close()
