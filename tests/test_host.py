"""Host side of libgbconn without a GPU: the C ABI loads and exports every
declared symbol, the reader / writer / verify / generator functions behave,
and the compute entry points fail loudly instead of falling back to the CPU."""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbconn.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(gb.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_the_library():
    """The ctypes mirrors of gb_opts, gb_stats and gb_server_stats have the
    sizes the library was built with, and gb_opts_default fills the mirror
    with the documented defaults without writing past it."""
    sizes = (ctypes.c_int64 * 3)()
    gb._lib.gb_struct_sizes(sizes)
    assert list(sizes) == [ctypes.sizeof(gb.Opts), ctypes.sizeof(gb.Stats),
                           ctypes.sizeof(gb.ServerStats)]
    buf = (ctypes.c_ubyte * (ctypes.sizeof(gb.Opts) + 16))(*([0xAB] * (ctypes.sizeof(gb.Opts) + 16)))
    o = gb.Opts.from_buffer(buf)
    gb._lib.gb_opts_default(ctypes.byref(o))
    assert bytes(buf[ctypes.sizeof(gb.Opts):]) == b"\xab" * 16
    assert (o.trim_level, o.canonical, o.pivot, o.k_pull, o.trim_pairs, o.fwbw_rounds,
            o.expand_mode) == (1, 1, -1, 4, 0, 1, 0)
    assert o.alpha == 15.0 and o.beta == 25.0


def test_status_strings():
    lib = ctypes.CDLL(gb.LIB_PATH)
    lib.gb_status_string.restype = ctypes.c_char_p
    assert lib.gb_status_string(0) == b"ok"
    assert lib.gb_status_string(4) == b"device wait timed out"


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback_without_gpu():
    with pytest.raises(gb.GBError) as e:
        gb.Context(0)
    assert e.value.status in (2, 7, 8)


def test_read_edge_and_errors(tmp_path):
    p = tmp_path / "g.txt"
    p.write_text("4 3\n0 1\n1  2\n3 0\n")
    n, s, d = gb.read_edge(str(p))
    assert n == 4 and s.tolist() == [0, 1, 3] and d.tolist() == [1, 2, 0]
    p.write_text("4 3\n0 1\n1 9\n3 0\n")
    with pytest.raises(gb.GBError) as e:
        gb.read_edge(str(p))
    assert e.value.status == 1  # id out of range
    p.write_text("4 3\n0 1\n")
    with pytest.raises(gb.GBError) as e:
        gb.read_edge(str(p))
    assert e.value.status == 6  # truncated
    with pytest.raises(gb.GBError) as e:
        gb.read_edge(str(tmp_path / "missing.txt"))
    assert e.value.status == 6
    # a header m that the file cannot hold is refused before any array is
    # sized from it (2^62 * 4 bytes would wrap to 0)
    for m in (1 << 62, (1 << 62) - 1, 1 << 40, 1000):
        p.write_text(f"4 {m}\n0 1\n1 2\n")
        with pytest.raises(gb.GBError) as e:
            gb.read_edge(str(p))
        assert e.value.status == 6


def _seq_read(text):
    """The reader's sequential semantics, restated: (status, n, src, dst)."""
    blank = " \t\r\n"
    pos = [0]

    def num():
        i = pos[0]
        while i < len(text) and text[i] in blank:
            i += 1
        if i >= len(text):
            pos[0] = i
            return None
        j = i
        if text[j] in "+-":
            j += 1
        k = j
        while k < len(text) and text[k].isdigit():
            k += 1
        if k == j or int(text[j:k]) > (1 << 62):
            pos[0] = i
            return None
        pos[0] = k
        return int(text[i:k])

    nn, mm = num(), num()
    if nn is None or mm is None or nn < 0 or nn > 0x7FFFFFFF or mm < 0:
        return 6, None, None, None
    # every edge takes at least 4 bytes of the body: a larger m is refused
    # before the body is read
    if mm > (len(text) - pos[0]) // 4:
        return 6, None, None, None
    src, dst = [], []
    for _ in range(mm):
        a = num()
        b = num() if a is not None else None
        if a is None or b is None:
            return 6, None, None, None
        if not (0 <= a < nn and 0 <= b < nn):
            return 1, None, None, None
        src.append(a)
        dst.append(b)
    return 0, nn, src, dst


def test_read_edge_pieces_match_sequential(tmp_path):
    """The body parsed in any number of pieces gives the sequential reader's
    arrays and status, on good files and on every kind of bad one."""
    rng = np.random.default_rng(5)
    texts = []
    for t in range(40):
        n = int(rng.integers(1, 50))
        m = int(rng.integers(0, 60))
        toks = [str(int(x)) for x in rng.integers(0, n, 2 * m)]
        kind = t % 8
        if kind == 1 and toks:  # an id out of range somewhere
            toks[int(rng.integers(0, len(toks)))] = str(n + int(rng.integers(0, 5)))
        elif kind == 2 and toks:  # garbage somewhere
            toks[int(rng.integers(0, len(toks)))] = rng.choice(["x", "1a", "+", "-", "--3"])
        elif kind == 3:  # truncated
            toks = toks[: int(rng.integers(0, len(toks) + 1))]
        elif kind == 4 and len(toks) >= 4:  # out of range, then garbage later (or earlier)
            i, j = sorted(rng.choice(len(toks), 2, replace=False))
            toks[int(i)], toks[int(j)] = (str(n), "x") if t % 16 < 8 else ("x", str(n))
        elif kind == 5:  # extra tokens after the edges
            toks += ["7", "x", "-1"]
        elif kind == 6 and toks:  # signs and glued numbers
            toks[int(rng.integers(0, len(toks)))] = rng.choice(["+0", "-0", "0-0", "1+0"])
        seps = [rng.choice([" ", "  ", "\t", "\n", "\r\n", " \n "]) for _ in toks]
        body = "".join(sep + tok for sep, tok in zip(seps, toks))
        texts.append(f"{n} {m}{body}\n")
    for i, text in enumerate(texts):
        p = tmp_path / f"g{i}.txt"
        p.write_text(text)
        want = _seq_read(text)
        for pieces in (1, 2, 3, 7, 64, 1000):
            if want[0] == 0:
                n, s_, d_ = gb.read_edge(str(p), pieces=pieces)
                assert n == want[1] and s_.tolist() == want[2] and d_.tolist() == want[3], (i, pieces)
            else:
                with pytest.raises(gb.GBError) as e:
                    gb.read_edge(str(p), pieces=pieces)
                assert e.value.status == want[0], (i, pieces, text)


def test_output_labels(tmp_path):
    p = tmp_path / "out.txt"
    gb.output_labels(str(p), np.array([0, 0, 2, -1], np.int32))
    assert p.read_text() == "0\n0\n2\n-1\n"
    # more than one 1 MB block, and the int32 extremes
    lab = np.random.default_rng(3).integers(-5, 1 << 31, 400_000).astype(np.int32)
    lab[:3] = [np.iinfo(np.int32).min, np.iinfo(np.int32).max, 0]
    gb.output_labels(str(p), lab)
    assert p.read_text() == "".join(f"{x}\n" for x in lab.tolist())
    gb.output_labels(str(p), np.zeros(0, np.int32))
    assert p.read_text() == ""


def test_verify_lines():
    lab = np.array([0, 0, 2, 3, 3, 3, -1], np.int32)
    assert gb.scc_verify(lab) == "Num SCCs: 3, Nontrivial: 2, Max SCC: 3, Unassigned 1\n"
    assert gb.cc_verify(lab) == "Num CCs: 3, Max CC: 3, Unassigned 1\n"
    assert oracle.stats(lab) == (3, 2, 3, 1)


def test_canonicalize():
    lab = np.array([5, 5, 2, 5, 2, 7, 7, 7], np.int32)
    assert gb.canonicalize(lab).tolist() == [0, 0, 2, 0, 2, 5, 5, 5]


def test_rmat_generator_properties():
    n, s, d = gb.rmat_edges(12, 16, 1)
    assert n == 4096
    n2, s2, d2 = gb.rmat_edges(12, 16, 1)
    assert np.array_equal(s, s2) and np.array_equal(d, d2)
    assert not np.any(s == d)
    key = s.astype(np.int64) * n + d
    assert np.all(np.diff(key) > 0)  # sorted by (src, dst), no duplicates
    assert s.size > 0.7 * 16 * n
    # seed changes the graph
    _, s3, _ = gb.rmat_edges(12, 16, 2)
    assert s3.size != s.size or not np.array_equal(s3, s)


def test_grid_generator_properties():
    side = 50
    n, s, d = gb.grid_edges(side, 250, 64, 2)
    assert n == side * side + 250
    lattice = (s < side * side) & (d < side * side)
    # lattice edges join horizontal or vertical neighbours only
    ds = np.abs(s[lattice].astype(np.int64) - d[lattice])
    assert set(np.unique(ds)) <= {1, side}
    # every chain vertex has exactly one in- or one out-edge to the rest
    assert s.size == np.count_nonzero(lattice) + 250
    # about 3/4 of the 2*side*(side-1) lattice pairs carry 1.33 arcs on average
    pairs = 2 * side * (side - 1)
    assert 0.8 * pairs < np.count_nonzero(lattice) < 1.2 * pairs


def test_batch_sizes_deterministic_and_clipped():
    ns, efs, seeds = gb.batch_sizes(20000, seed=4)
    ns2, efs2, seeds2 = gb.batch_sizes(20000, seed=4)
    assert np.array_equal(ns, ns2) and np.array_equal(efs, efs2) and np.array_equal(seeds, seeds2)
    assert ns.min() >= 64 and ns.max() <= 500_000
    assert efs.min() >= 4 and efs.max() <= 32
    med = np.median(ns)
    assert 1500 < med < 2700
    assert 0.10 < np.mean(ns > 10_000) < 0.20


def test_cli_usage_without_arguments():
    for tool in ("scc", "cc"):
        exe = os.path.join(ROOT, "connectivity_gb300", "bin", tool)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0
        assert r.stdout == f"Usage: {exe} [graph] [optional: output file]\n"


def test_file_writers_round_trip(tmp_path):
    """gb_write_text writes what the host reader reads back; gb_write_binary
    writes the documented layout."""
    n, s, d = 1000, np.arange(0, 999, dtype=np.int32), np.arange(1, 1000, dtype=np.int32)
    gb.write_text(tmp_path / "g.txt", n, s, d)
    hn, hs, hd = gb.read_edge(str(tmp_path / "g.txt"))
    assert hn == n and np.array_equal(hs, s) and np.array_equal(hd, d)
    with open(tmp_path / "g.txt") as f:
        assert f.readline() == "1000 999\n" and f.readline() == "0 1\n"
    gb.write_binary(tmp_path / "g.bin", n, s, d)
    raw = open(tmp_path / "g.bin", "rb").read()
    assert raw[:8] == b"GBEDGES1"
    assert np.frombuffer(raw[8:24], np.int64).tolist() == [n, 999]
    assert np.array_equal(np.frombuffer(raw[24:24 + 4 * 999], np.int32), s)
    assert np.array_equal(np.frombuffer(raw[24 + 4 * 999:], np.int32), d)


def test_tune_table_lookup():
    """Size-class tables: options of the class nearest on a log scale."""
    from connectivity_gb300 import tune
    assert tune.opts_for({}, 100).t_block == gb.opts().t_block
    table = {"kind": 0, "classes": [
        {"n": 1 << 10, "opts": {"t_block": 128, "t_grid": 8192, "k_pull": 2, "alpha": 5.0,
                                "beta": 10.0, "grid_blocks": 0}},
        {"n": 1 << 20, "opts": {"t_block": 2048, "t_grid": 131072, "k_pull": 4, "alpha": 50.0,
                                "beta": 100.0, "grid_blocks": 76, "expand_mode": 1}}]}
    assert tune.opts_for(table, 600).t_block == 128
    assert tune.opts_for(table, 600).expand_mode == 0  # (a table written before the field)
    assert tune.opts_for(table, 1 << 19).t_block == 2048
    o = tune.opts_for(table, 1 << 22)
    assert (o.t_grid, o.k_pull, o.grid_blocks, o.expand_mode) == (131072, 4, 76, 1)
    back = tune.dict_to_opts(tune.opts_to_dict(o))
    assert back.beta == 100.0 and back.expand_mode == 1
    # options outside the tuned set keep their defaults
    assert (back.trim_level, back.fwbw_rounds, back.trim_pairs) == (1, 1, 0)
    # class bounds: geometric midpoints, the last class open-ended
    assert tune.class_bounds(table) == [1 << 15, 1 << 62]
    assert tune.class_bounds({}) == []


def test_committed_class_table():
    """The committed size-class table (written by the autotuner on a GB300)
    covers rising classes with options every field of which is set."""
    from connectivity_gb300 import tune
    table = tune.load(tune.DEFAULT_TABLE)
    ns = [c["n"] for c in table["classes"]]
    assert ns == sorted(ns) and len(ns) >= 4
    for c in table["classes"]:
        assert set(tune.TUNED) <= set(c["opts"])
        assert c["ms"] <= c["default_ms"]
    b = tune.class_bounds(table)
    assert all(x < y for x, y in zip(b, b[1:]))
