"""The oracle (oracle/multistep.c) pinned against the reference: its golden
vector, the golden fixtures produced by the unmodified reference code
(tests/golden/, see make_golden.py), and -- where the reference tree is
present -- the reference harness itself.  CPU only."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs
from tests.golden.make_golden import cases, digest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INDEX = json.load(open(os.path.join(GOLD, "index.json")))
CASES = list(cases())


def test_reference_golden_vector():
    # multistep/test.graph: SCC {0,1},{2}, CC one component; canonical labels
    # 0 0 2 and 0 0 0 (the reference prints exactly these)
    n, s, d = graphs.test_graph()
    assert oracle.scc(oracle.CpuGraph(n, s, d)).tolist() == [0, 0, 2]
    assert oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)).tolist() == [0, 0, 0]
    assert INDEX["test_graph_text"]["scc"] == [0, 0, 2]
    assert INDEX["test_graph_text"]["cc"] == [0, 0, 0]


def test_text_reader_on_reference_fixture():
    n, s, d = gb.read_edge(os.path.join(GOLD, "test_graph.txt"))
    n2, s2, d2 = graphs.test_graph()
    assert n == n2 and s.tolist() == s2.tolist() and d.tolist() == d2.tolist()
    lab = oracle.scc(oracle.CpuGraph(n, s, d))
    assert gb.scc_verify(lab) == INDEX["test_graph_text"]["scc_verify"]
    assert gb.cc_verify(oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))) == \
        INDEX["test_graph_text"]["cc_verify"]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_fixture(case):
    name, (n, s, d) = case
    ent = INDEX[name]
    assert digest(n, s, d) == ent["digest"], "generator output changed"
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    scc = oracle.scc(oracle.CpuGraph(n, s, d))
    assert np.array_equal(scc, gold["scc"])
    assert gb.scc_verify(scc) == ent["scc_verify"]
    cc = oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))
    assert np.array_equal(cc, gold["cc"])
    assert gb.cc_verify(cc) == ent["cc_verify"]


@pytest.mark.parametrize("case", CASES[:9], ids=[c[0] for c in CASES[:9]])
def test_oracle_variants_agree(case):
    name, (n, s, d) = case
    g = oracle.CpuGraph(n, s, d)
    base = oracle.scc(g)
    # no trim, fixed-point trim, no serial step, and an independent Tarjan
    lab0, t0 = oracle.scc(g, trim_level=0, times=True)
    assert np.array_equal(lab0, base) and t0.num_trim == 0
    assert np.array_equal(oracle.scc(g, trim_level=2), base)
    assert np.array_equal(oracle.scc(g, vert_cutoff=0), base)
    assert np.array_equal(oracle.tarjan(g), base)


@pytest.mark.parametrize("case", CASES[:9], ids=[c[0] for c in CASES[:9]])
def test_oracle_against_scipy(case):
    sp = pytest.importorskip("scipy.sparse")
    csg = pytest.importorskip("scipy.sparse.csgraph")
    name, (n, s, d) = case
    a = sp.csr_matrix((np.ones(s.size, np.int8), (s, d)), shape=(n, n))
    _, lab = csg.connected_components(a, directed=True, connection="strong")
    assert np.array_equal(oracle.canonical(lab.astype(np.int32)),
                          oracle.scc(oracle.CpuGraph(n, s, d)))
    _, lab = csg.connected_components(a, directed=True, connection="weak")
    assert np.array_equal(oracle.canonical(lab.astype(np.int32)),
                          oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)))


def test_pivot_rules():
    # SCC pivot: lowest id of maximum out*in (scc_main.cpp:169-182)
    n, s, d = 4, np.array([0, 1, 1, 2, 3, 3, 0], np.int32), np.array([1, 0, 2, 1, 0, 1, 3], np.int32)
    g = oracle.CpuGraph(n, s, d)
    # out: 0:2 1:2 2:1 3:2; in: 0:2 1:3 2:1 3:1 -> products 4 6 1 2
    assert g.pivot_scc()[0] == 1
    # cc pivot: lowest id of maximum mirrored degree (cc_main.cpp:148-160)
    gm = oracle.CpuGraph(n, s, d, mirror=True)
    assert gm.pivot_cc()[0] == 1
    # no positive product -> no pivot
    g0 = oracle.CpuGraph(3, np.array([0, 0], np.int32), np.array([1, 2], np.int32))
    assert g0.pivot_scc()[0] == -1


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present")
@pytest.mark.parametrize("seed", [5, 6])
def test_oracle_against_live_reference(seed):
    n, s, d = gb.rmat_edges(13, 8, seed)
    raw, line, _ = oracle.ref_run("scc", n, s, d, threads=4)
    assert np.array_equal(oracle.canonical(raw), oracle.scc(oracle.CpuGraph(n, s, d)))
    raw, line, _ = oracle.ref_run("cc", n, s, d, threads=4)
    assert np.array_equal(oracle.canonical(raw), oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)))


@pytest.mark.parametrize("seed", range(12))
def test_oracle_random_graphs_against_scipy(seed):
    """Random graphs of mixed shape (sparse, dense, planted cycles and
    two-cycles, self-loops and duplicate edges): the oracle's SCC labels at
    every trim level, and its CC labels, equal scipy's components in
    canonical form."""
    sp = pytest.importorskip("scipy.sparse")
    csg = pytest.importorskip("scipy.sparse.csgraph")
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 3000))
    m = int(rng.integers(0, 4 * n))
    s = rng.integers(0, n, m)
    d = rng.integers(0, n, m)
    # a few planted cycles and two-cycles
    for _ in range(int(rng.integers(0, 20))):
        k = int(rng.integers(2, 40))
        cyc = rng.choice(n, size=min(k, n), replace=False)
        s = np.concatenate([s, cyc])
        d = np.concatenate([d, np.roll(cyc, -1)])
    s = s.astype(np.int32)
    d = d.astype(np.int32)
    a = sp.csr_matrix((np.ones(s.size, np.int8), (s, d)), shape=(n, n))
    _, lab = csg.connected_components(a, directed=True, connection="strong")
    want = oracle.canonical(lab.astype(np.int32))
    g = oracle.CpuGraph(n, s, d)
    for trim in (0, 1, 2):
        assert np.array_equal(oracle.scc(g, trim_level=trim), want), trim
    _, lab = csg.connected_components(a, directed=True, connection="weak")
    assert np.array_equal(oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)),
                          oracle.canonical(lab.astype(np.int32)))


@pytest.mark.parametrize("n,ef,seed", [(1 << 10, 16, 1), (1 << 14, 16, 1), (3000, 7, 5), (64, 4, 9),
                                       (1 << 16, 16, 1)])
def test_oracle_generator_equals_product_generator(n, ef, seed):
    """oracle/gen.c (bucketed by source, per-bucket sort) gives the product
    generator's R-MAT edge list (64-bit key radix sort), so the reference arm
    of the benchmark runs the same graph without loading the product."""
    a = oracle.rmat_edges_n(n, ef, seed)
    b = gb.rmat_edges_n(n, ef, seed)
    assert digest(*a) == digest(*b)


def test_pins_cover_the_full_size_workloads():
    """tests/golden/pins.json holds the reference's label digests and verify
    lines for the full-size workloads; the generators still give the pinned
    edge lists where that is cheap to check."""
    pins = json.load(open(os.path.join(GOLD, "pins.json")))
    for key in ("rmat_s20_ef16_seed1", "rmat_s22_ef16_seed1", "rmat_s24_ef16_seed1",
                "grid_1024_seed2", "grid_2048_seed2"):
        assert key in pins, key
        e = pins[key]
        for f in ("edges", "scc_labels", "cc_labels", "scc_verify", "cc_verify"):
            assert f in e, (key, f)
        assert e["scc_verify"].endswith("Unassigned 0\n")
    n, s, d = oracle.rmat_edges(20, 16, 1)
    assert digest(n, s, d) == pins["rmat_s20_ef16_seed1"]["edges"]
    n, s, d = gb.grid_edges(1024, 1024 * 1024 // 10, 64, 2)
    assert digest(n, s, d) == pins["grid_1024_seed2"]["edges"]
    # the oracle gives the pinned labels at these two sizes
    import hashlib

    def lab_digest(x):
        return hashlib.sha256(np.ascontiguousarray(x, "<i4").tobytes()).hexdigest()
    n, s, d = oracle.rmat_edges(20, 16, 1)
    assert lab_digest(oracle.scc(oracle.CpuGraph(n, s, d))) == \
        pins["rmat_s20_ef16_seed1"]["scc_labels"]
    assert lab_digest(oracle.cc(oracle.CpuGraph(n, s, d, mirror=True))) == \
        pins["rmat_s20_ef16_seed1"]["cc_labels"]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference not built")
@pytest.mark.parametrize("mode", ["seq", "par"])
def test_reference_batch_mode(mode):
    """The harness's batch mode (a loop of run_scc / run_cc over many graphs,
    or one thread per graph) gives every graph's own labels."""
    gs = [(n, s, d) for _, n, s, d in graphs.edge_cases()]
    gs += [oracle.rmat_edges_n(n, ef, seed) for n, ef, seed in [(3000, 8, 1), (700, 4, 3)]]
    for kind in ("scc", "cc"):
        labs, total, per = oracle.ref_batch(kind, gs, mode, threads=2)
        assert total is not None and total >= 0
        assert (per is not None) == (mode == "seq")
        for (n, s, d), lab in zip(gs, labs):
            want = (oracle.scc(oracle.CpuGraph(n, s, d)) if kind == "scc"
                    else oracle.cc(oracle.CpuGraph(n, s, d, mirror=True)))
            assert np.array_equal(oracle.canonical(lab), want)
