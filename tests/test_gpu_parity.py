"""Parity of the CUDA path with the oracle: canonical labels must be
bit-identical, and the verify lines byte-identical, on every case.  Calls go
through the C ABI (libgbconn.so via ctypes)."""
from __future__ import annotations

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu


def opts(**kw):
    """Options of a run of the cooperative kernel: this file tests that
    kernel on small graphs too (the one-block path, which small graphs take
    by default, has its own tests in test_gpu_small.py), and its WCC too
    (the sampled union-find, the default for WCC, is tested in
    test_gpu_cc_dropin.py)."""
    kw.setdefault("small_path", 0)
    kw.setdefault("wcc_mode", 0)
    return gb.opts(**kw)

CASES = graphs.edge_cases()

VARIANTS = {
    "default": {},
    "trim0": {"trim_level": 0},
    "trim2": {"trim_level": 2},
    "pairs": {"trim_pairs": 1},
    "pairs2": {"trim_level": 2, "trim_pairs": 1},
    "rounds": {"fwbw_rounds": 4},
    "balanced": {"expand_mode": 1},
    "balanced_rounds": {"expand_mode": 1, "fwbw_rounds": 3, "trim_pairs": 1},
    # tiny tiers push every vertex through the block and grid-slice paths
    "tiers": {"t_block": 33, "t_grid": 64},
    "pull_early": {"alpha": 1e9, "beta": 1e-3, "k_pull": 1},
    "push_only": {"alpha": 1e-9},
    "small_grid": {"grid_blocks": 3},
    "signature": {"colour_mode": 1},
    "signature_trim2": {"colour_mode": 1, "trim_level": 2, "fwbw_rounds": 2},
}


def _scc_want(n, s, d):
    return oracle.scc(oracle.CpuGraph(n, s, d))


def _wcc_want(n, s, d):
    return oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("variant", list(VARIANTS))
def test_scc_edge_cases(ctx, case, variant):
    name, n, s, d = case
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab, st = ctx.scc(g, o=opts(**VARIANTS[variant]), stats=True)
    want = _scc_want(n, s, d)
    assert np.array_equal(lab, want), name
    assert gb.scc_verify(lab) == gb.scc_verify(want)
    assert st.unassigned == 0


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("variant", ["default", "tiers", "pull_early", "small_grid", "balanced"])
def test_wcc_edge_cases(ctx, case, variant):
    name, n, s, d = case
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab = ctx.wcc(g, o=opts(**VARIANTS[variant]))
    want = _wcc_want(n, s, d)
    assert np.array_equal(lab, want), name
    assert gb.cc_verify(lab) == gb.cc_verify(want)


def test_reference_golden_vector(ctx):
    # multistep/test.graph: SCC {0,1},{2}; CC one component
    n, s, d = graphs.test_graph()
    g = gb.Graph.from_edges(ctx, n, s, d)
    assert ctx.scc(g, o=opts()).tolist() == [0, 0, 2]
    assert ctx.wcc(g, o=opts()).tolist() == [0, 0, 0]
    assert gb.scc_verify(ctx.scc(g, o=opts())) == "Num SCCs: 2, Nontrivial: 1, Max SCC: 2, Unassigned 0\n"


@pytest.mark.parametrize("scale,ef", [(10, 16), (12, 4), (14, 16), (16, 16), (16, 32), (18, 8)])
@pytest.mark.parametrize("variant", ["default", "trim0", "trim2", "pairs", "rounds", "balanced",
                                     "balanced_rounds", "tiers", "pull_early", "small_grid"])
def test_rmat_scc(ctx, scale, ef, variant):
    n, s, d = graphs.rmat(scale, ef)
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab = ctx.scc(g, o=opts(**VARIANTS[variant]))
    want = _scc_want(n, s, d)
    assert np.array_equal(lab, want)


@pytest.mark.parametrize("scale,ef", [(10, 16), (14, 16), (16, 16), (18, 8)])
@pytest.mark.parametrize("variant", ["default", "pull_early", "rounds", "balanced"])
def test_rmat_wcc(ctx, scale, ef, variant):
    n, s, d = graphs.rmat(scale, ef)
    g = gb.Graph.from_edges(ctx, n, s, d)
    assert np.array_equal(ctx.wcc(g, o=opts(**VARIANTS[variant])), _wcc_want(n, s, d))


@pytest.mark.parametrize("side", [16, 64, 128])
@pytest.mark.parametrize("variant", ["default", "trim0", "trim2", "pairs", "pairs2", "balanced"])
def test_grid_scc(ctx, side, variant):
    n, s, d = graphs.grid(side)
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab = ctx.scc(g, o=opts(**VARIANTS[variant]))
    want = _scc_want(n, s, d)
    assert np.array_equal(lab, want)


@pytest.mark.parametrize("trim", [1, 2])
def test_grid_1024_scc(ctx, trim):
    """The high-diameter lattice with chains at 1024^2 (1.15 M vertices): the
    colour rounds with local continuation against the oracle."""
    n, s, d = graphs.grid(1024)
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab, st = ctx.scc(g, o=opts(trim_level=trim), stats=True)
    assert st.colour_rounds > 10  # the colour phase does the work here
    assert np.array_equal(lab, _scc_want(n, s, d))


@pytest.mark.parametrize("side", [64, 256, 1024])
def test_grid_wcc(ctx, side):
    n, s, d = graphs.grid(side)
    g = gb.Graph.from_edges(ctx, n, s, d)
    assert np.array_equal(ctx.wcc(g, o=opts()), _wcc_want(n, s, d))


def test_device_rmat_matches_host_generator(ctx):
    g = gb.Graph.rmat(ctx, 14, 16, 5)
    n, s, d = gb.rmat_edges(14, 16, 5)
    oo, oa, io, ia = g.to_host()
    off, adj = gb.csr_from_edges(n, s, d)
    assert np.array_equal(oo, off) and np.array_equal(oa, adj)
    off, adj = gb.csr_from_edges(n, d, s)
    assert np.array_equal(io, off) and np.array_equal(ia, adj)


def test_from_csr_and_pivot(ctx):
    n, s, d = graphs.rmat(12, 16, 3)
    cg = oracle.CpuGraph(n, s, d)
    g = gb.Graph.from_csr(ctx, n, cg.out_off, cg.out_adj, cg.in_off, cg.in_adj)
    assert np.array_equal(ctx.scc(g, o=opts()), _scc_want(n, s, d))
    assert ctx.pivot(g, 0)[0] == cg.pivot_scc()[0]
    mg = oracle.CpuGraph(n, s, d, mirror=True)
    assert ctx.pivot(g, 1)[0] == mg.pivot_cc()[0]
    # symmetric CSR (cc's mirrored graph) gives the same WCC
    sg = gb.Graph.from_csr(ctx, n, mg.out_off, mg.out_adj)
    assert sg.symmetric
    assert np.array_equal(ctx.wcc(sg, o=opts()), _wcc_want(n, s, d))


def test_reference_shaped_dropins():
    n, s, d = graphs.rmat(12, 16, 9)
    cg = oracle.CpuGraph(n, s, d)
    odl = cg.out_off.astype(np.uint32)
    idl = cg.in_off.astype(np.uint32)
    piv, avg = cg.pivot_scc()
    lab = gb.run_scc_ref(n, cg.out_adj, cg.in_adj, odl, idl, piv, avg, 10000)
    assert np.array_equal(lab, _scc_want(n, s, d))
    mg = oracle.CpuGraph(n, s, d, mirror=True)
    piv, avg = mg.pivot_cc()
    lab = gb.run_cc_ref(n, mg.out_adj, mg.out_off.astype(np.uint32), piv, avg)
    assert np.array_equal(lab, _wcc_want(n, s, d))


def test_reference_shaped_dropins_pinned():
    """Pinned host buffers take the direct ingest (read over the host link
    by the device, checked on the way); the labels must not change, and a
    bad CSR must still be refused."""
    torch = pytest.importorskip("torch")
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    for n, s, d in (graphs.rmat(14, 16, 21), graphs.erdos(1001, 7003, 5)):
        cg = oracle.CpuGraph(n, s, d)
        odl, idl = pin(cg.out_off.astype(np.uint32)), pin(cg.in_off.astype(np.uint32))
        oa, ia = pin(cg.out_adj), pin(cg.in_adj)
        # odd offsets into the arrays exercise the unaligned copy path too
        out = pin(np.empty(n, np.int32))
        piv, avg = cg.pivot_scc()
        lab = gb.run_scc_ref(n, oa, ia, odl, idl, piv, avg, 10000, out)
        assert np.array_equal(lab, _scc_want(n, s, d))
        mg = oracle.CpuGraph(n, s, d, mirror=True)
        mo, ma = pin(mg.out_off.astype(np.uint32)), pin(mg.out_adj)
        piv, avg = mg.pivot_cc()
        lab = gb.run_cc_ref(n, ma, mo, piv, avg, pin(np.empty(n, np.int32)))
        assert np.array_equal(lab, _wcc_want(n, s, d))
    # an id out of range, and a non-monotone offset array, in pinned memory
    n, s, d = graphs.rmat(10, 8, 3)
    cg = oracle.CpuGraph(n, s, d)
    odl, idl = pin(cg.out_off.astype(np.uint32)), pin(cg.in_off.astype(np.uint32))
    oa, ia = pin(cg.out_adj), pin(cg.in_adj)
    oa[len(oa) // 2] = n + 5
    with pytest.raises(gb.GBError) as e:
        gb.run_scc_ref(n, oa, ia, odl, idl)
    assert e.value.status == gb.GB_ERR_INVALID
    oa[len(oa) // 2] = 0
    idl[n // 2], idl[n // 2 + 1] = idl[n // 2 + 1] + 1, idl[n // 2]
    with pytest.raises(gb.GBError) as e:
        gb.run_scc_ref(n, oa, ia, odl, idl)
    assert e.value.status == gb.GB_ERR_INVALID


def test_pinned_unaligned_adjacency(ctx):
    """An adjacency array that starts off a 16-byte boundary takes the
    scalar ingest."""
    torch = pytest.importorskip("torch")
    n, s, d = graphs.rmat(12, 16, 4)
    cg = oracle.CpuGraph(n, s, d)
    big = torch.empty(len(cg.out_adj) + 1, dtype=torch.int32).pin_memory().numpy()
    oa = big[1:]
    oa[:] = cg.out_adj
    big2 = torch.empty(len(cg.in_adj) + 3, dtype=torch.int32).pin_memory().numpy()
    ia = big2[3:]
    ia[:] = cg.in_adj
    odl = torch.from_numpy(cg.out_off.astype(np.uint32)).pin_memory().numpy()
    idl = torch.from_numpy(cg.in_off.astype(np.uint32)).pin_memory().numpy()
    lab = gb.run_scc_ref(n, oa, ia, odl, idl)
    assert np.array_equal(lab, _scc_want(n, s, d))


def test_device_labels_and_async(ctx):
    torch = pytest.importorskip("torch")
    n, s, d = graphs.rmat(14, 16, 11)
    g = gb.Graph.from_edges(ctx, n, s, d)
    want = _scc_want(n, s, d)
    out = torch.full((n,), -7, dtype=torch.int32, device="cuda:0")
    ctx.scc(g, labels=out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), want)
    out2 = torch.full((n,), -7, dtype=torch.int32, device="cuda:0")
    for _ in range(3):
        ctx.scc_async(g, out2.data_ptr())
    ctx.sync()
    assert np.array_equal(out2.cpu().numpy(), want)


def test_raw_labels_partition(ctx):
    n, s, d = graphs.rmat(14, 16, 13)
    g = gb.Graph.from_edges(ctx, n, s, d)
    raw = ctx.scc(g, o=opts(canonical=0))
    assert np.array_equal(gb.canonicalize(raw), _scc_want(n, s, d))


def test_bad_edges_rejected(ctx):
    with pytest.raises(gb.GBError):
        gb.Graph.from_edges(ctx, 4, np.array([0, 5], np.int32), np.array([1, 2], np.int32))
    off = np.array([0, 2, 1], np.int64)  # decreasing offsets
    with pytest.raises(gb.GBError):
        gb.Graph.from_csr(ctx, 2, off, np.array([1, 0], np.int32))


def test_repeat_runs_identical(ctx):
    n, s, d = graphs.rmat(16, 16, 21)
    g = gb.Graph.from_edges(ctx, n, s, d)
    first = ctx.scc(g, o=opts())
    for _ in range(5):
        assert np.array_equal(ctx.scc(g, o=opts()), first)


def test_rmat_s20_scc_and_wcc(ctx):
    n, s, d = graphs.rmat(20, 16, 1)
    g = gb.Graph.from_edges(ctx, n, s, d)
    assert np.array_equal(ctx.scc(g, o=opts()), _scc_want(n, s, d))
    assert np.array_equal(ctx.wcc(g, o=opts()), _wcc_want(n, s, d))


def _hub_graph(core=300, up=4000, down=3000, seed=12):
    """A hub pivot (vertex 0: >= 64 in- and out-edges inside a core SCC) with a
    large region upstream (reaches the core only) and one downstream (reached
    only), both made of 2-cycles so that trim keeps them: the forward and
    backward sets differ a lot and the component is their intersection."""
    r = np.random.default_rng(seed)
    e = []
    c = np.arange(core)
    e += list(zip(c, np.roll(c, -1)))                       # a cycle through the core
    e += [(0, int(x)) for x in r.choice(np.arange(1, core), 80, replace=False)]
    e += [(int(x), 0) for x in r.choice(np.arange(1, core), 80, replace=False)]
    base = core
    for i in range(up // 2):                                 # upstream 2-cycles -> core
        a, b = base + 2 * i, base + 2 * i + 1
        e += [(a, b), (b, a), (b, int(r.integers(0, core)))]
    base += up
    for i in range(down // 2):                               # core -> downstream 2-cycles
        a, b = base + 2 * i, base + 2 * i + 1
        e += [(a, b), (b, a), (int(r.integers(0, core)), a)]
    n = base + down
    perm = r.permutation(n).astype(np.int32)                 # hide the structure in the ids
    perm[perm == 0], perm[0] = perm[0], 0                    # keep the hub's id 0
    s = perm[np.array([x for x, _ in e], np.int64)].astype(np.int32)
    d = perm[np.array([y for _, y in e], np.int64)].astype(np.int32)
    return n, s, d


def test_searches_together_from_hub_pivot(ctx):
    n, s, d = _hub_graph()
    g = gb.Graph.from_edges(ctx, n, s, d)
    piv, _ = ctx.pivot(g, 0)
    lab, st = ctx.scc(g, stats=True, o=opts())
    assert np.array_equal(lab, _scc_want(n, s, d))
    # the pivot is a hub, so the two searches ran together: the forward set
    # holds the core and the downstream region, the component the core only
    assert st.n_fwbw == 300 and st.n_visit_fw == 300 + 3000
    assert np.array_equal(ctx.scc(g, o=opts(trim_level=2)), lab)


def _planted_pairs(npairs, nrest, seed):
    """npairs two-cycles (2i, 2i+1) on top of a random graph over the other
    nrest vertices: the first half take edges only from their partner (in
    pattern) and point into the rest, the second half point only to their
    partner (out pattern) and are pointed to from the rest."""
    rng = np.random.default_rng(seed)
    n = 2 * npairs + nrest
    base = 2 * npairs
    s, d = [], []
    for i in range(npairs):
        u, v = 2 * i, 2 * i + 1
        s += [u, v]
        d += [v, u]
        other = base + rng.integers(0, nrest, 3)
        if i < npairs // 2:
            s += [u, v, u]
            d += other.tolist()
        else:
            s += other.tolist()
            d += [u, v, v]
    m = 4 * nrest
    s += (base + rng.integers(0, nrest, m)).tolist()
    d += (base + rng.integers(0, nrest, m)).tolist()
    s = np.array(s, np.int32)
    d = np.array(d, np.int32)
    keep = s != d
    e = np.unique(np.stack([s[keep], d[keep]], 1), axis=0)
    return n, e[:, 0].copy(), e[:, 1].copy()


@pytest.mark.parametrize("trim", [1, 2])
def test_trim_pairs_planted(ctx, trim):
    """Every planted two-cycle leaves with the trim (the size-2 pass adds at
    least 2 per pair to the trim count, and no more than the graph's size-2
    SCCs), and the labels still equal the oracle's."""
    n, s, d = _planted_pairs(500, 3000, 11)
    g = gb.Graph.from_edges(ctx, n, s, d)
    want = _scc_want(n, s, d)
    lab0, st0 = ctx.scc(g, o=opts(trim_level=trim), stats=True)
    lab1, st1 = ctx.scc(g, o=opts(trim_level=trim, trim_pairs=1), stats=True)
    assert np.array_equal(lab0, want) and np.array_equal(lab1, want)
    sizes = np.bincount(want, minlength=n)
    found = st1.n_trim - st0.n_trim
    assert 2 * 500 <= found <= 2 * int((sizes == 2).sum())
    assert found % 2 == 0


def test_trim_pairs_only_pairs(ctx):
    """A graph of nothing but two-cycles: the size-2 pass removes every
    vertex, the pivot among them, and nothing is left for FW-BW or colour."""
    npairs = 1000
    u = np.arange(0, 2 * npairs, 2, dtype=np.int32)
    s = np.concatenate([u, u + 1])
    d = np.concatenate([u + 1, u])
    n = 2 * npairs
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab, st = ctx.scc(g, o=opts(trim_pairs=1), stats=True)
    assert np.array_equal(lab, np.repeat(u, 2))
    assert st.n_trim == n and st.n_fwbw == 0 and st.colour_rounds == 0
    lab0, st0 = ctx.scc(g, o=opts(trim_level=0), stats=True)
    assert np.array_equal(lab0, lab) and st0.n_trim == 0


def _disjoint_rmats(k, scale, ef):
    """k R-MAT graphs with different seeds, side by side (k large SCCs)."""
    ss, dd, n = [], [], 0
    for i in range(k):
        m, s, d = graphs.rmat(scale, ef, seed=10 + i)
        ss.append(s + n)
        dd.append(d + n)
        n += m
    return n, np.concatenate(ss).astype(np.int32), np.concatenate(dd).astype(np.int32)


@pytest.mark.parametrize("kind", ["scc", "wcc"])
def test_repivot_rounds_take_the_next_components(ctx, kind):
    """Four disjoint R-MATs: each FW-BW round after the first starts from
    the next pivot by the reference rule and takes another large component
    out before the colour rounds; labels stay equal to the oracle's."""
    n, s, d = _disjoint_rmats(4, 14, 8)
    g = gb.Graph.from_edges(ctx, n, s, d)
    fn = ctx.scc if kind == "scc" else ctx.wcc
    want = _scc_want(n, s, d) if kind == "scc" else _wcc_want(n, s, d)
    lab1, st1 = fn(g, o=opts(fwbw_rounds=1), stats=True)
    lab4, st4 = fn(g, o=opts(fwbw_rounds=4), stats=True)
    assert np.array_equal(lab1, want) and np.array_equal(lab4, want)
    assert st1.fwbw_rounds == 1 and st4.fwbw_rounds == 4
    sizes = np.sort(np.bincount(want))[::-1]
    assert st1.n_fwbw in set(sizes[:4].tolist())
    # each round labels one whole component: four of the largest
    assert st4.n_fwbw > st1.n_fwbw
    assert st4.n_fwbw <= sizes[:4].sum()


def test_repivot_stops_when_little_is_left(ctx):
    """Rounds stop once fewer than 4096 vertices are valid (the colour
    rounds take the rest), whatever the option asks for."""
    n, s, d = graphs.rmat(10, 16)
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab, st = ctx.scc(g, o=opts(fwbw_rounds=50), stats=True)
    assert np.array_equal(lab, _scc_want(n, s, d))
    assert st.fwbw_rounds == 1


@pytest.mark.parametrize("kind", ["scc", "wcc"])
def test_balanced_push_same_work(ctx, kind):
    """The edge-balanced push walks each reached vertex's edges once, as the
    tiers do: same labels and the same visited edge counts (push steps
    only)."""
    n, s, d = graphs.rmat(16, 16)
    g = gb.Graph.from_edges(ctx, n, s, d)
    fn = ctx.scc if kind == "scc" else ctx.wcc
    o_t = opts(alpha=1e-9)
    o_b = opts(alpha=1e-9, expand_mode=1)
    lt, st_t = fn(g, o=o_t, stats=True)
    lb, st_b = fn(g, o=o_b, stats=True)
    assert np.array_equal(lt, lb)
    assert st_b.m_visit_fw == st_t.m_visit_fw and st_b.m_visit_bw == st_t.m_visit_bw
    assert st_b.pull_steps == 0 and st_t.pull_steps == 0


def _degree_key(deg):
    """The hint rule's degree key: the total degree below 32, above it eight
    steps per power of two (exponent and the next three bits)."""
    deg = np.asarray(deg, np.int64)
    key = deg.copy()
    big = deg >= 32
    e = np.frexp(deg[big].astype(np.float64))[1].astype(np.int64) - 1
    e = np.minimum(e, 30)
    key[big] = 32 + 8 * (e - 5) + ((np.minimum(deg[big], (1 << 31) - 1) >> (e - 3)) & 7)
    return key


def _hints_want(n, off, adj, deg):
    """The hint rule restated: the neighbour of largest degree key (see
    _degree_key), the first in adjacency order on ties, -1 without
    neighbours."""
    want = np.full(n, -1, np.int64)
    d = np.diff(off)
    nz = np.flatnonzero(d > 0)
    if nz.size:
        k = np.arange(adj.size, dtype=np.int64) - np.repeat(off[:-1], d)
        key = deg[adj].astype(np.int64) * (1 << 32) + ((1 << 32) - 1 - k)
        best = np.maximum.reduceat(key, off[nz])
        kk = (1 << 32) - 1 - (best & ((1 << 32) - 1))
        want[nz] = adj[off[nz] + kk]
    return want.astype(np.int32)


@pytest.mark.parametrize("case", ["rmat16", "rmat20", "hub", "hub_big", "star"])
def test_pull_hints_follow_the_rule(ctx, case):
    if case == "hub_big":
        # a list of 300,000 entries (hundreds of 1,024-entry chunks, equal
        # keys in many of them) and in-lists of every size around it
        n = 400000
        r = np.random.default_rng(5)
        s = np.concatenate([np.zeros(300000, np.int32), r.integers(0, n, 400000).astype(np.int32),
                            np.full(3000, 11, np.int32)])
        d = np.concatenate([np.arange(1, 300001, dtype=np.int32),
                            r.integers(0, n, 400000).astype(np.int32),
                            r.integers(0, 50, 3000).astype(np.int32)])
    elif case == "rmat16":
        n, s, d = gb.rmat_edges(16, 16, 1)
    elif case == "rmat20":
        n, s, d = gb.rmat_edges(20, 16, 1)
    elif case == "hub":
        # hubs above the block-per-vertex cutoff next to degree-1 vertices
        n = 20000
        r = np.random.default_rng(1)
        s = np.concatenate([np.zeros(9000, np.int32), np.full(5000, 7, np.int32),
                            r.integers(0, n, 30000).astype(np.int32)])
        d = np.concatenate([np.arange(1, 9001, dtype=np.int32), r.integers(0, n, 5000).astype(np.int32),
                            r.integers(0, n, 30000).astype(np.int32)])
    else:
        n, s, d = [c for c in graphs.edge_cases() if c[0] == "star"][0][1:]
    g = gb.Graph.from_edges(ctx, n, s, d)
    oo, oa, io, ia = g.to_host()
    deg = _degree_key(np.diff(oo) + np.diff(io))
    ho, hi = g.hints()
    assert np.array_equal(ho, _hints_want(n, oo, oa, deg))
    assert np.array_equal(hi, _hints_want(n, io, ia, deg))
    g.close()


@pytest.mark.parametrize("mode", [2, 1])
def test_long_chain_residual(ctx, mode):
    """A residual that is one long chain of single-vertex components (every
    vertex also points at a sink hub): colour rounds would label one vertex
    per round; the default switches to signature rounds after a few colour
    rounds, which need two.  Labels equal the oracle's."""
    n = 20001
    s = np.concatenate([np.arange(1, n, dtype=np.int32), np.arange(1, n - 1, dtype=np.int32)])
    d = np.concatenate([np.zeros(n - 1, np.int32), np.arange(2, n, dtype=np.int32)])
    g = gb.Graph.from_edges(ctx, n, s, d)
    lab, st = ctx.scc(g, o=opts(colour_mode=mode), stats=True)
    assert np.array_equal(lab, _scc_want(n, s, d))
    assert st.colour_rounds <= 8
    g.close()
