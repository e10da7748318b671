"""ctypes wrapper of oracle/liboracle.so, the CPU restatement of the Multistep
pipeline (oracle/multistep.c), and of the reference harness binaries in
oracle/_ref/.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  The product never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_SCC = os.path.join(HERE, "_ref", "ref_scc")
REF_CC = os.path.join(HERE, "_ref", "ref_cc")

_lib = None


class Graph(C.Structure):
    _fields_ = [("n", C.c_int32), ("m", C.c_int64), ("out_off", C.c_void_p),
                ("out_adj", C.c_void_p), ("in_off", C.c_void_p), ("in_adj", C.c_void_p)]


class Times(C.Structure):
    _fields_ = [("trim", C.c_double), ("fwbw", C.c_double), ("colour", C.c_double),
                ("serial", C.c_double), ("total", C.c_double), ("num_trim", C.c_int64),
                ("num_fwbw", C.c_int64), ("num_colour_sccs", C.c_int64),
                ("num_serial_sccs", C.c_int64), ("pivot", C.c_int32),
                ("colour_rounds", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} missing; build with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_build_csr.argtypes = [C.c_int32, C.c_int64, P, P, P, P]
        L.orc_build_csr.restype = C.c_int
        L.orc_pivot_scc.argtypes = [C.POINTER(Graph), C.POINTER(C.c_double)]
        L.orc_pivot_scc.restype = C.c_int32
        L.orc_pivot_cc.argtypes = [C.POINTER(Graph), C.POINTER(C.c_double)]
        L.orc_pivot_cc.restype = C.c_int32
        L.orc_scc.argtypes = [C.POINTER(Graph), P, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                              C.POINTER(Times)]
        L.orc_scc.restype = C.c_int
        L.orc_cc.argtypes = [C.POINTER(Graph), P, C.c_int32, C.c_double, C.POINTER(Times)]
        L.orc_cc.restype = C.c_int
        L.orc_canonicalize.argtypes = [C.c_int32, P]
        L.orc_label_stats.argtypes = [C.c_int32, P, P]
        L.orc_scc_tarjan.argtypes = [C.POINTER(Graph), P]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_rmat_edges.argtypes = [C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                     C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_void_p)]
        L.orc_rmat_edges.restype = C.c_int
        L.orc_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def rmat_edges_n(n: int, edge_factor: int, seed: int,
                 abc: tuple[float, float, float] = (0.57, 0.19, 0.19)):
    """Seeded R-MAT edge list (oracle/gen.c): the product generator's edges,
    built independently of it.  Returns (n, src, dst), sorted by (src, dst)."""
    m = C.c_int64()
    s, d = C.c_void_p(), C.c_void_p()
    if lib().orc_rmat_edges(n, edge_factor, seed, abc[0], abc[1], abc[2], C.byref(m),
                            C.byref(s), C.byref(d)) != 0:
        raise MemoryError("orc_rmat_edges failed")
    out = []
    for p in (s, d):
        a = np.empty(m.value, np.int32)
        if m.value:
            C.memmove(a.ctypes.data, p, m.value * 4)
        lib().orc_free(p)
        out.append(a)
    return n, out[0], out[1]


def rmat_edges(scale: int, edge_factor: int = 16, seed: int = 1,
               abc: tuple[float, float, float] = (0.57, 0.19, 0.19)):
    """R-MAT with 2^scale vertices (see rmat_edges_n)."""
    return rmat_edges_n(1 << scale, edge_factor, seed, abc)


def build_csr(n: int, src: np.ndarray, dst: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """create_csr's counting sort (scc_main.cpp:127-166): stable, input order."""
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    off = np.zeros(n + 1, np.int64)
    adj = np.zeros(max(1, src.size), np.int32)
    if lib().orc_build_csr(n, src.size, _p(src), _p(dst), _p(off), _p(adj)) != 0:
        raise ValueError("bad edge list")
    return off, adj[: src.size]


class CpuGraph:
    """Out- and in-CSR on the host (the reference's graph struct, int64 offsets)."""

    def __init__(self, n: int, src: np.ndarray, dst: np.ndarray, mirror: bool = False):
        self.n = n
        if mirror:  # cc's reader mirrors every edge (cc_main.cpp:102-118)
            s2 = np.empty(2 * src.size, np.int32)
            d2 = np.empty(2 * src.size, np.int32)
            s2[0::2], d2[0::2] = src, dst
            s2[1::2], d2[1::2] = dst, src
            src, dst = s2, d2
        self.m = int(src.size)
        self.out_off, self.out_adj = build_csr(n, src, dst)
        if mirror:
            self.in_off, self.in_adj = None, None
        else:
            self.in_off, self.in_adj = build_csr(n, dst, src)
        self._s = Graph(n, self.m, _p(self.out_off).value, _p(self.out_adj).value,
                        None if self.in_off is None else _p(self.in_off).value,
                        None if self.in_adj is None else _p(self.in_adj).value)

    @classmethod
    def from_csr(cls, n, out_off, out_adj, in_off=None, in_adj=None) -> "CpuGraph":
        g = cls.__new__(cls)
        g.n, g.m = n, int(out_adj.size)
        g.out_off = np.ascontiguousarray(out_off, np.int64)
        g.out_adj = np.ascontiguousarray(out_adj, np.int32)
        g.in_off = None if in_off is None else np.ascontiguousarray(in_off, np.int64)
        g.in_adj = None if in_adj is None else np.ascontiguousarray(in_adj, np.int32)
        g._s = Graph(n, g.m, _p(g.out_off).value, _p(g.out_adj).value,
                     None if g.in_off is None else _p(g.in_off).value,
                     None if g.in_adj is None else _p(g.in_adj).value)
        return g

    def pivot_scc(self) -> tuple[int, float]:
        a = C.c_double()
        return lib().orc_pivot_scc(C.byref(self._s), C.byref(a)), a.value

    def pivot_cc(self) -> tuple[int, float]:
        a = C.c_double()
        return lib().orc_pivot_cc(C.byref(self._s), C.byref(a)), a.value


def scc(g: CpuGraph, trim_level: int = 1, vert_cutoff: int = 10000, canonical: bool = True,
        times: bool = False):
    """run_scc restated (scc_main.cpp:210-317)."""
    lab = np.full(g.n, -1, np.int32)
    piv, avg = g.pivot_scc()
    t = Times()
    if lib().orc_scc(C.byref(g._s), _p(lab), piv, avg, vert_cutoff, trim_level, C.byref(t)) != 0:
        raise RuntimeError("oracle scc failed")
    if canonical:
        lib().orc_canonicalize(g.n, _p(lab))
    return (lab, t) if times else lab


def cc(g: CpuGraph, canonical: bool = True, times: bool = False):
    """run_cc restated (cc_main.cpp:184-245); g must be the mirrored graph."""
    lab = np.full(g.n, -1, np.int32)
    piv, avg = g.pivot_cc()
    t = Times()
    if lib().orc_cc(C.byref(g._s), _p(lab), piv, avg, C.byref(t)) != 0:
        raise RuntimeError("oracle cc failed")
    if canonical:
        lib().orc_canonicalize(g.n, _p(lab))
    return (lab, t) if times else lab


def tarjan(g: CpuGraph) -> np.ndarray:
    """Independent serial SCC (iterative Tarjan), canonical labels."""
    lab = np.full(g.n, -1, np.int32)
    lib().orc_scc_tarjan(C.byref(g._s), _p(lab))
    lib().orc_canonicalize(g.n, _p(lab))
    return lab


def canonical(labels: np.ndarray) -> np.ndarray:
    lab = np.array(labels, np.int32, copy=True)
    lib().orc_canonicalize(lab.size, _p(lab))
    return lab


def stats(labels: np.ndarray) -> tuple[int, int, int, int]:
    lab = np.ascontiguousarray(labels, np.int32)
    out = np.zeros(4, np.int64)
    lib().orc_label_stats(lab.size, _p(lab), _p(out))
    return tuple(int(x) for x in out)


def set_threads(t: int) -> None:
    lib().orc_set_threads(t)


def num_threads() -> int:
    return lib().orc_num_threads()


# ---- the unmodified reference (oracle/_ref, built where the tree exists) ----
def ref_available() -> bool:
    return os.path.exists(REF_SCC) and os.path.exists(REF_CC)


def write_bin(path: str, n: int, src: np.ndarray, dst: np.ndarray) -> None:
    with open(path, "wb") as f:
        np.array([n, src.size], np.int64).tofile(f)
        np.ascontiguousarray(src, np.int32).tofile(f)
        np.ascontiguousarray(dst, np.int32).tofile(f)


def ref_run(kind: str, n: int, src: np.ndarray, dst: np.ndarray, reps: int = 1,
            threads: int | None = None) -> tuple[np.ndarray, str, float]:
    """Runs the reference's run_scc / run_cc through the harness.  Returns
    (labels as produced, verify line, best time in seconds)."""
    lab, line, times = ref_run_times(kind, n, src, dst, reps, threads)
    return lab, line, min(times)


def ref_run_times(kind: str, n: int, src: np.ndarray, dst: np.ndarray, reps: int = 1,
                  threads: int | None = None) -> tuple[np.ndarray, str, list[float]]:
    """As ref_run, with the time of every rep (seconds, in order): the CSR is
    built once and run_scc / run_cc runs reps times on it."""
    exe = REF_SCC if kind == "scc" else REF_CC
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    with tempfile.TemporaryDirectory() as d:
        eb, lb = os.path.join(d, "e.bin"), os.path.join(d, "l.bin")
        write_bin(eb, n, src, dst)
        r = subprocess.run([exe, "--bin", eb, lb, str(reps)], capture_output=True, text=True,
                           env=env, check=True)
        lab = np.fromfile(lb, dtype=np.int32)
    lines = r.stdout.splitlines()
    times = [float(x) for x in lines[2].split(":")[1].split()] if len(lines) > 2 else \
        [float(lines[0].split(":")[1])]
    return lab, lines[1] + "\n", times


def ref_batch(kind: str, graphs, mode: str = "seq", threads: int | None = None, exe_dir=None):
    """The reference's run_scc / run_cc once per graph of a batch, in one
    process (the harness's --batch mode).  graphs: (n, src, dst) with local
    ids.  mode "seq": one graph after another, each with all threads; "par":
    one thread per graph over all threads.  Returns (labels per graph as
    produced, seconds of the whole loop, seconds per graph or None)."""
    d0 = exe_dir or os.path.join(HERE, "_ref")
    exe = os.path.join(d0, "ref_scc" if kind == "scc" else "ref_cc")
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    with tempfile.TemporaryDirectory() as d:
        gb_, lb = os.path.join(d, "g.bin"), os.path.join(d, "l.bin")
        with open(gb_, "wb") as f:
            np.array([len(graphs)], np.int64).tofile(f)
            for n, s, t in graphs:
                np.array([n, len(s)], np.int64).tofile(f)
                np.ascontiguousarray(s, np.int32).tofile(f)
                np.ascontiguousarray(t, np.int32).tofile(f)
        r = subprocess.run([exe, "--batch", gb_, lb, mode], capture_output=True, text=True,
                           env=env, check=True)
        flat = np.fromfile(lb, dtype=np.int32)
    out, at = [], 0
    for n, _, _ in graphs:
        out.append(flat[at:at + n])
        at += n
    total, per = None, None
    for line in r.stdout.splitlines():
        if line.startswith("batch_seconds:"):
            total = float(line.split(":")[1])
        elif line.startswith("graph_seconds:"):
            per = [float(x) for x in line.split(":")[1].split()]
    return out, total, per


def ref_text(kind: str, graph_path: str) -> tuple[np.ndarray, str]:
    """The reference main on a text graph file (unchanged code path)."""
    exe = REF_SCC if kind == "scc" else REF_CC
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "labels.txt")
        r = subprocess.run([exe, "--text", graph_path, out], capture_output=True, text=True,
                           check=True)
        lab = np.loadtxt(out, dtype=np.int32, ndmin=1)
    return lab, r.stdout.splitlines()[1] + "\n"
