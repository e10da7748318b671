"""The drop-in executables connectivity_gb300/bin/scc and bin/cc on graph
files: the reference's command line, its two stdout lines ("Multistep SCC
time: %9.6lf" / "Multistep CC time: %9.6lf", multistep/scc_main.cpp:377 and
cc_main.cpp:301, then the verify line) and its label file (one label per
line, scc_main.cpp:193-202), checked against the reference's own outputs in
tests/golden/."""
from __future__ import annotations

import json
import os
import re
import subprocess

import numpy as np
import pytest

import connectivity_gb300 as gb
import oracle
from tests.golden.make_golden import digest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
INDEX = json.load(open(os.path.join(GOLD, "index.json")))
BIN = os.path.join(os.path.dirname(gb.LIB_PATH), "bin")
TIME_LINE = {"scc": r"Multistep SCC time: +\d+\.\d{6}", "cc": r"Multistep CC time: +\d+\.\d{6}"}


def _run(tool, *args):
    r = subprocess.run([os.path.join(BIN, tool), *args], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.splitlines()


def _graph_file(tmp_path, case):
    if case == "test_graph_text":
        return os.path.join(GOLD, "test_graph.txt"), INDEX[case]
    sc = {"rmat_s16_ef16_seed1": (16, 16, 1), "rmat_s12_ef4_seed2": (12, 4, 2)}[case]
    n, s, d = gb.rmat_edges(*sc)
    assert digest(n, s, d) == INDEX[case]["digest"]
    p = str(tmp_path / f"{case}.txt")
    gb.write_text(p, n, s, d)
    return p, INDEX[case]


@pytest.mark.parametrize("case", ["test_graph_text", "rmat_s16_ef16_seed1", "rmat_s12_ef4_seed2"])
@pytest.mark.parametrize("tool", ["scc", "cc"])
def test_executable_lines_and_label_file(tmp_path, tool, case):
    path, ent = _graph_file(tmp_path, case)
    out = str(tmp_path / "labels.txt")
    lines = _run(tool, path, out)
    assert len(lines) == 2, lines
    assert re.fullmatch(TIME_LINE[tool], lines[0]), lines[0]
    assert lines[1] + "\n" == ent[f"{tool}_verify"]
    lab = np.loadtxt(out, dtype=np.int32, ndmin=1)
    if case == "test_graph_text":
        want = oracle.canonical(np.array(ent[tool], np.int32))
    else:
        want = np.load(os.path.join(GOLD, f"{case}.npz"))[tool]
    assert np.array_equal(oracle.canonical(lab), want)
    # the labels are already canonical (minimum member id)
    assert np.array_equal(lab, want)


@pytest.mark.parametrize("tool", ["scc", "cc"])
def test_executable_without_output_file_and_binary_input(tmp_path, tool):
    n, s, d = gb.rmat_edges(14, 16, 1)
    p = str(tmp_path / "g.bin")
    gb.write_binary(p, n, s, d)
    lines = _run(tool, p)
    assert len(lines) == 2
    assert re.fullmatch(TIME_LINE[tool], lines[0])
    assert lines[1] + "\n" == INDEX["rmat_s14_ef16_seed1"][f"{tool}_verify"]


def test_executable_reports_a_bad_file(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("3 2\n0 1\n1 7\n")
    r = subprocess.run([os.path.join(BIN, "scc"), str(p)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode != 0
    # gb_status_string(GB_ERR_INVALID) and the reader's detail
    assert "invalid argument" in r.stderr and "[0, n)" in r.stderr
