"""Graph files parsed on the device (gb_graph_from_file): the reference's text
format and the binary format must give exactly the CSR the host reader
gives, whatever the blanks and however tokens fall across the tokenizer's
byte chunks; malformed files must be refused."""
from __future__ import annotations

import os

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests import graphs

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def write_text(path, n, s, d, sep=" ", eol="\n", final_eol=True, extra=""):
    body = eol.join(f"{a}{sep}{b}" for a, b in zip(s.tolist(), d.tolist()))
    with open(path, "w", newline="") as f:
        f.write(f"{n} {len(s)}{eol}{body}{eol if final_eol and len(s) else ''}{extra}")


def same_graph(ctx, g, n, s, d):
    want = gb.Graph.from_edges(ctx, n, s, d)
    a, b = g.to_host(), want.to_host()
    want.close()
    for x, y in zip(a, b):
        assert (x is None and y is None) or np.array_equal(x, y)


@pytest.mark.parametrize("chunk", [0, 1, 3, 7, 64])
def test_text_matches_host_reader(ctx, tmp_path, chunk):
    n, s, d = graphs.rmat(12, 8, 31)
    p = tmp_path / "g.txt"
    write_text(p, n, s, d)
    g = gb.Graph.from_file(ctx, p, chunk=chunk)
    hn, hs, hd = gb.read_edge(str(p))
    assert g.n == hn == n and g.m == len(hs)
    same_graph(ctx, g, hn, hs, hd)
    assert np.array_equal(ctx.scc(g), oracle.scc(oracle.CpuGraph(n, s, d)))


@pytest.mark.parametrize("sep,eol,final", [("\t", "\n", True), ("  ", "\r\n", True),
                                           (" ", "\n", False), (" \t ", "\n\n", True)])
def test_text_blanks(ctx, tmp_path, sep, eol, final):
    n, s, d = graphs.erdos(300, 1500, 2)
    p = tmp_path / "g.txt"
    write_text(p, n, s, d, sep=sep, eol=eol, final_eol=final)
    for chunk in (0, 2, 5):
        g = gb.Graph.from_file(ctx, p, chunk=chunk)
        same_graph(ctx, g, n, s, d)


def test_text_extra_tokens_ignored_and_signs(ctx, tmp_path):
    p = tmp_path / "g.txt"
    with open(p, "w") as f:
        f.write("4 3\n0 1\n+1 2\n2 -0\n3 3\n9 9 trailing words\n")
    g = gb.Graph.from_file(ctx, p, chunk=3)
    same_graph(ctx, g, 4, np.array([0, 1, 2], np.int32), np.array([1, 2, 0], np.int32))


def test_text_edge_cases(ctx, tmp_path):
    p = tmp_path / "g.txt"
    with open(p, "w") as f:
        f.write("7 0\n")
    g = gb.Graph.from_file(ctx, p)
    assert g.n == 7 and g.m == 0
    assert np.array_equal(ctx.scc(g), np.arange(7, dtype=np.int32))
    # the reference's own test graph
    g = gb.Graph.from_file(ctx, os.path.join(HERE, "golden", "test_graph.txt"))
    n, s, d = gb.read_edge(os.path.join(HERE, "golden", "test_graph.txt"))
    same_graph(ctx, g, n, s, d)


@pytest.mark.parametrize("content,status", [
    ("5 3\n0 1\n1 2\n", gb.GB_ERR_IO),         # fewer edges than m
    ("5 2\n0 1\n1 5\n", gb.GB_ERR_INVALID),    # id == n
    ("5 2\n0 1\n1 x\n", gb.GB_ERR_INVALID),    # not a number
    ("5 2\n0 1\n-1 2\n", gb.GB_ERR_INVALID),   # negative id
    ("5 2\n0 1\n12a 2\n", gb.GB_ERR_INVALID),  # trailing garbage in a token
    ("x y\n0 1\n", gb.GB_ERR_IO),              # bad header
    ("", gb.GB_ERR_IO),                        # empty file
])
def test_text_rejected(ctx, tmp_path, content, status):
    p = tmp_path / "bad.txt"
    with open(p, "w") as f:
        f.write(content)
    with pytest.raises(gb.GBError) as e:
        gb.Graph.from_file(ctx, p, chunk=2)
    assert e.value.status == status


def test_missing_file(ctx, tmp_path):
    with pytest.raises(gb.GBError) as e:
        gb.Graph.from_file(ctx, tmp_path / "absent.txt")
    assert e.value.status == gb.GB_ERR_IO


def test_binary_round_trip(ctx, tmp_path):
    n, s, d = graphs.rmat(13, 16, 7)
    p = tmp_path / "g.bin"
    gb.write_binary(p, n, s, d)
    g = gb.Graph.from_file(ctx, p)
    same_graph(ctx, g, n, s, d)
    # truncated file
    raw = open(p, "rb").read()
    with open(tmp_path / "short.bin", "wb") as f:
        f.write(raw[: len(raw) - 4])
    with pytest.raises(gb.GBError) as e:
        gb.Graph.from_file(ctx, tmp_path / "short.bin")
    assert e.value.status == gb.GB_ERR_IO
    # an id out of range
    bad = s.copy()
    bad[5] = n
    gb.write_binary(tmp_path / "bad.bin", n, bad, d)
    with pytest.raises(gb.GBError) as e:
        gb.Graph.from_file(ctx, tmp_path / "bad.bin")
    assert e.value.status == gb.GB_ERR_INVALID
