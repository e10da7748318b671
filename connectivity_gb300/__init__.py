"""Python binding of libgbconn, the GB300 Multistep SCC / WCC library.

The compute path is the CUDA library behind the C ABI in include/gbconn.h;
this module only loads it with ctypes and converts numpy arrays.  There is no
CPU fallback: if libgbconn.so is missing, importing this module raises, and
without a GB300 the run functions raise GBError.

Reference surface (HPCGraphAnalysis/Connectivity, multistep/):
    read_edge      scc_main.cpp:94-125      -> read_edge()
    create_csr     scc_main.cpp:127-191     -> Graph.from_edges() / from_csr()
    run_scc        scc_main.cpp:210-317     -> Context.scc()
    run_cc         cc_main.cpp:184-245      -> Context.wcc() / Context.cc()
    scc_verify     scc_verify.cpp:47-77     -> scc_verify()
    cc_verify      cc_verify.cpp:47-74      -> cc_verify()
    output_scc     scc_main.cpp:193-202     -> output_labels()
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbconn.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build it with "
        "`python -c 'import __graft_entry__ as g; g.build()'` or "
        "`python connectivity_gb300/build.py`")

_lib = C.CDLL(LIB_PATH)

GB_OK = 0
(GB_ERR_INVALID, GB_ERR_CUDA, GB_ERR_OOM, GB_ERR_TIMEOUT, GB_ERR_ITER_LIMIT, GB_ERR_IO,
 GB_ERR_NO_DEVICE, GB_ERR_UNSUPPORTED, GB_ERR_CAPACITY) = range(1, 10)
STATUS_NAMES = {
    0: "GB_OK", 1: "GB_ERR_INVALID", 2: "GB_ERR_CUDA", 3: "GB_ERR_OOM",
    4: "GB_ERR_TIMEOUT", 5: "GB_ERR_ITER_LIMIT", 6: "GB_ERR_IO",
    7: "GB_ERR_NO_DEVICE", 8: "GB_ERR_UNSUPPORTED", 9: "GB_ERR_CAPACITY",
}


class GBError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        detail = _lib.gb_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({detail})")


class Opts(C.Structure):
    _fields_ = [
        ("trim_level", C.c_int32), ("canonical", C.c_int32), ("pivot", C.c_int32),
        ("vert_cutoff", C.c_int32), ("t_block", C.c_int32), ("t_grid", C.c_int32),
        ("k_pull", C.c_int32), ("alpha", C.c_float), ("beta", C.c_float),
        ("max_steps", C.c_int32), ("grid_blocks", C.c_int32), ("trim_pairs", C.c_int32),
        ("fwbw_rounds", C.c_int32), ("expand_mode", C.c_int32), ("small_path", C.c_int32),
        ("colour_mode", C.c_int32), ("wcc_mode", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("ms_trim", C.c_double), ("ms_reach", C.c_double), ("ms_colour", C.c_double),
        ("ms_canon", C.c_double), ("ms_total", C.c_double),
        ("pivot", C.c_int32), ("colour_rounds", C.c_int32),
        ("n_trim", C.c_int64), ("n_visit_fw", C.c_int64), ("n_fwbw", C.c_int64),
        ("unassigned", C.c_int64), ("vtx_reads", C.c_int64), ("edge_reads", C.c_int64),
        ("list_rw", C.c_int64), ("bytes_trim", C.c_int64), ("bytes_reach", C.c_int64),
        ("bytes_colour", C.c_int64), ("bytes_canon", C.c_int64), ("trim_steps", C.c_int64), ("fw_steps", C.c_int64),
        ("bw_steps", C.c_int64), ("pull_steps", C.c_int64), ("colour_steps", C.c_int64),
        ("mark_steps", C.c_int64), ("grid_blocks", C.c_int32), ("err_where", C.c_int32),
        ("m_visit_fw", C.c_int64), ("m_visit_bw", C.c_int64), ("pull_edges", C.c_int64),
        ("fwbw_rounds", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)


def _sig(name, res, args):
    f = getattr(_lib, name)
    f.restype = res
    f.argtypes = args
    return f


_sig("gb_status_string", C.c_char_p, [C.c_int32])
_sig("gb_last_error", C.c_char_p, [])
_sig("gb_opts_default", None, [C.POINTER(Opts)])
_sig("gb_struct_sizes", None, [C.POINTER(C.c_int64)])
_sig("gb_ctx_create", C.c_int32, [C.c_int, C.POINTER(_P)])
_sig("gb_ctx_destroy", C.c_int32, [_P])
_sig("gb_ctx_set_stream", C.c_int32, [_P, _P])
_sig("gb_ctx_stream", _P, [_P])
_sig("gb_ctx_sync", C.c_int32, [_P])
_sig("gb_ctx_phase_times", C.c_int32, [_P, C.c_int32, _P])
_sig("gb_ctx_set_class_opts", C.c_int32, [_P, C.c_int32, _P, _P])
_sig("gb_ctx_reach_trace", C.c_int32, [_P, _P, _P, _P, C.c_int32])
_sig("gb_ctx_reach_trace2", C.c_int32, [_P, _P, _P, _P, _P, C.c_int32])
_sig("gb_ctx_block_times", C.c_int32, [_P, _P, C.c_int32])
_sig("gb_graph_from_edges", C.c_int32, [_P, C.c_int32, C.c_int64, _P, _P, C.POINTER(_P)])
_sig("gb_graph_from_csr", C.c_int32, [_P, C.c_int32, C.c_int64, _P, _P, _P, _P, C.POINTER(_P)])
_sig("gb_graph_from_csr32", C.c_int32, [_P, C.c_int32, C.c_uint32, _P, _P, _P, _P, C.POINTER(_P)])
_sig("gb_graph_rmat", C.c_int32, [_P, C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                  C.c_double, C.POINTER(_P)])
_sig("gb_graph_rmat_n", C.c_int32, [_P, C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                    C.c_double, C.POINTER(_P)])
_sig("gb_graph_info", C.c_int32, [_P, _I32P, _I64P, _I32P])
_sig("gb_graph_set_hints", C.c_int32, [_P, _P, C.c_int32])
_sig("gb_graph_has_hints", C.c_int32, [_P, _I32P])
_sig("gb_graph_hints_to_host", C.c_int32, [_P, _P, _P])
_sig("gb_graph_from_file2", C.c_int32, [_P, C.c_char_p, C.c_int32, C.POINTER(_P)])
_sig("gb_write_binary", C.c_int32, [C.c_char_p, C.c_int32, C.c_int64, _P, _P])
_sig("gb_write_text", C.c_int32, [C.c_char_p, C.c_int32, C.c_int64, _P, _P])
_sig("gb_batch_from_edges", C.c_int32, [_P, C.c_int32, _P, C.c_int64, _P, _P, C.POINTER(_P)])
_sig("gb_batch_rmat", C.c_int32, [_P, C.c_int32, _P, _P, _P, C.c_double, C.c_double, C.c_double,
                                  C.POINTER(_P)])
_sig("gb_batch_info", C.c_int32, [_P, _I32P, _I64P, _I64P])
_sig("gb_batch_vbase", C.c_int32, [_P, _P])
_sig("gb_batch_graph", C.c_int32, [_P, C.POINTER(_P)])
for _n in ("gb_batch_scc", "gb_batch_wcc"):
    _sig(_n, C.c_int32, [_P, _P, _P, C.POINTER(Opts), C.POINTER(Stats)])
_sig("gb_batch_scc_async", C.c_int32, [_P, _P, _P, C.POINTER(Opts)])
_sig("gb_batch_destroy", C.c_int32, [_P])
for _n in ("gb_scc_edges", "gb_wcc_edges"):
    _sig(_n, C.c_int32, [_P, C.c_int32, C.c_int64, _P, _P, _P, C.POINTER(Opts)])
_sig("gb_tune", C.c_int32, [_P, _P, C.c_int32, C.c_int32, C.POINTER(Opts), _P])
_sig("gb_tune_batch", C.c_int32, [_P, _P, C.c_int32, C.c_int32, C.POINTER(Opts), _P])


class ServerStats(C.Structure):
    """gb_server_stats."""
    _fields_ = [("completed", C.c_int64), ("batches", C.c_int64), ("mean_batch", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("graphs_per_s", C.c_double)]


_sig("gb_server_create", C.c_int32, [_P, C.c_int64, C.c_int32, C.POINTER(_P)])
_sig("gb_server_start", C.c_int32, [_P])
_sig("gb_server_set_opts", C.c_int32, [_P, C.POINTER(Opts)])
_sig("gb_server_submit", C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int64, _P, _P, _P, C.c_int64,
                                     _I64P])
_sig("gb_server_wait", C.c_int32, [_P, C.c_int64, _I64P])
_sig("gb_server_drain", C.c_int32, [_P])
_sig("gb_server_stats_get", C.c_int32, [_P, C.POINTER(ServerStats)])
_sig("gb_server_destroy", C.c_int32, [_P])
_sig("gb_graph_csr_to_host", C.c_int32, [_P, _P, _P, _P, _P])
_sig("gb_graph_device_csr", C.c_int32, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
                                        C.POINTER(_P)])
_sig("gb_graph_pivot", C.c_int32, [_P, _P, C.c_int32, _I32P, C.POINTER(C.c_double)])
_sig("gb_graph_destroy", C.c_int32, [_P])
for _n in ("gb_scc", "gb_wcc", "gb_cc"):
    _sig(_n, C.c_int32, [_P, _P, _P, C.POINTER(Opts), C.POINTER(Stats)])
for _n in ("gb_scc_async", "gb_wcc_async"):
    _sig(_n, C.c_int32, [_P, _P, _P, C.POINTER(Opts)])
_sig("gb_dropin_set_derive_share", C.c_int32, [C.c_double])
_sig("gb_run_scc", C.c_int32, [C.c_int, C.c_uint, _P, _P, _P, _P, _P, C.c_int, C.c_double, C.c_int])
_sig("gb_run_cc", C.c_int32, [C.c_int, C.c_uint, _P, _P, _P, C.c_int, C.c_double])
_sig("gb_read_edge", C.c_int32, [C.c_char_p, _I32P, _I64P, C.POINTER(_P), C.POINTER(_P)])
_sig("gb_read_edge_pieces", C.c_int32,
     [C.c_char_p, C.c_int32, _I32P, _I64P, C.POINTER(_P), C.POINTER(_P)])
_sig("gb_free_host", None, [_P])
_sig("gb_output_labels", C.c_int32, [C.c_char_p, C.c_int32, _P])
_sig("gb_scc_verify", C.c_int32, [C.c_int32, _P, C.c_char_p, C.c_size_t, _I64P])
_sig("gb_cc_verify", C.c_int32, [C.c_int32, _P, C.c_char_p, C.c_size_t, _I64P])
_sig("gb_canonicalize", C.c_int32, [C.c_int32, _P])
_sig("gb_rmat_edges_host", C.c_int32, [C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                       C.c_double, _I64P, C.POINTER(_P), C.POINTER(_P)])
_sig("gb_rmat_edges_host_n", C.c_int32, [C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                         C.c_double, _I64P, C.POINTER(_P), C.POINTER(_P)])
_sig("gb_grid_edges_host", C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, _I32P, _I64P,
                                       C.POINTER(_P), C.POINTER(_P)])
_sig("gb_batch_sizes", C.c_int32, [C.c_int32, C.c_uint64, C.c_double, C.c_double, C.c_int32,
                                   C.c_int32, C.c_int32, C.c_int32, _P, _P, _P])


def _check(status: int, where: str) -> None:
    if status != GB_OK:
        raise GBError(status, where)


def _ptr(a):
    """Address of a numpy array, or of anything with data_ptr() (a torch
    tensor, host or device)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _take(p: C.c_void_p, count: int, dtype) -> np.ndarray:
    """Copies a library-malloc'd array into numpy and frees it."""
    if count == 0:
        out = np.zeros(0, dtype=dtype)
    else:
        buf = (C.c_byte * (count * np.dtype(dtype).itemsize)).from_address(p.value)
        out = np.frombuffer(buf, dtype=dtype).copy()
    _lib.gb_free_host(p)
    return out


def _optp(o):
    """The options argument: o by reference, or NULL (the context's class
    table, else the defaults)."""
    return C.byref(o) if o is not None else None


def opts(**kw) -> Opts:
    o = Opts()
    _lib.gb_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


# ---------------------------------------------------------------------------
# host utilities
# ---------------------------------------------------------------------------
def write_binary(path: str, n: int, src, dst) -> None:
    """Edge list in the binary graph-file format (gb_write_binary)."""
    s = np.ascontiguousarray(src, np.int32)
    d = np.ascontiguousarray(dst, np.int32)
    _check(_lib.gb_write_binary(str(path).encode(), int(n), s.size, _ptr(s), _ptr(d)),
           "gb_write_binary")


def write_text(path: str, n: int, src, dst) -> None:
    """Edge list in the reference's text format (gb_write_text)."""
    s = np.ascontiguousarray(src, np.int32)
    d = np.ascontiguousarray(dst, np.int32)
    _check(_lib.gb_write_text(str(path).encode(), int(n), s.size, _ptr(s), _ptr(d)),
           "gb_write_text")


def read_edge(path: str, pieces: int = 0) -> tuple[int, np.ndarray, np.ndarray]:
    """read_edge (scc_main.cpp:94-125): returns (n, src, dst).  pieces: how
    many pieces the body is parsed in by host threads (0: automatic)."""
    n, m = C.c_int32(), C.c_int64()
    s, d = C.c_void_p(), C.c_void_p()
    _check(_lib.gb_read_edge_pieces(str(path).encode(), int(pieces), C.byref(n), C.byref(m),
                                    C.byref(s), C.byref(d)), "read_edge")
    return n.value, _take(s, m.value, np.int32), _take(d, m.value, np.int32)


def output_labels(path: str, labels: np.ndarray) -> None:
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    _check(_lib.gb_output_labels(path.encode(), lab.size, _ptr(lab)), "output_labels")


def scc_verify(labels: np.ndarray) -> str:
    """The exact scc_verify line (scc_verify.cpp:73-74), with newline."""
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    buf = C.create_string_buffer(256)
    _check(_lib.gb_scc_verify(lab.size, _ptr(lab), buf, 256, None), "scc_verify")
    return buf.value.decode()


def cc_verify(labels: np.ndarray) -> str:
    """The exact cc_verify line (cc_verify.cpp:70-71), with newline."""
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    buf = C.create_string_buffer(256)
    _check(_lib.gb_cc_verify(lab.size, _ptr(lab), buf, 256, None), "cc_verify")
    return buf.value.decode()


def canonicalize(labels: np.ndarray) -> np.ndarray:
    lab = np.array(labels, dtype=np.int32, copy=True)
    _check(_lib.gb_canonicalize(lab.size, _ptr(lab)), "canonicalize")
    return lab


RMAT_ABC = (0.57, 0.19, 0.19)


def rmat_edges(scale: int, edge_factor: int = 16, seed: int = 1,
               abc: tuple[float, float, float] = RMAT_ABC) -> tuple[int, np.ndarray, np.ndarray]:
    """Seeded R-MAT edge list (host), without self-loops and duplicates,
    sorted by (src, dst).  Returns (n, src, dst)."""
    m = C.c_int64()
    s, d = C.c_void_p(), C.c_void_p()
    _check(_lib.gb_rmat_edges_host(scale, edge_factor, seed, abc[0], abc[1], abc[2], C.byref(m),
                                   C.byref(s), C.byref(d)), "rmat_edges")
    return 1 << scale, _take(s, m.value, np.int32), _take(d, m.value, np.int32)


def rmat_edges_n(n: int, edge_factor: int, seed: int,
                 abc: tuple[float, float, float] = RMAT_ABC) -> tuple[int, np.ndarray, np.ndarray]:
    """R-MAT on any n (the batch rule): edge_factor*n candidates at scale
    ceil(log2 n), ids >= n dropped.  Returns (n, src, dst)."""
    m = C.c_int64()
    s, d = C.c_void_p(), C.c_void_p()
    _check(_lib.gb_rmat_edges_host_n(n, edge_factor, seed, abc[0], abc[1], abc[2], C.byref(m),
                                     C.byref(s), C.byref(d)), "rmat_edges_n")
    return n, _take(s, m.value, np.int32), _take(d, m.value, np.int32)


def grid_edges(side: int, extra: int | None = None, max_chain: int = 64,
               seed: int = 2) -> tuple[int, np.ndarray, np.ndarray]:
    """Oriented side x side lattice plus `extra` chain vertices (default
    side*side // 10).  Returns (n, src, dst)."""
    if extra is None:
        extra = side * side // 10
    n, m = C.c_int32(), C.c_int64()
    s, d = C.c_void_p(), C.c_void_p()
    _check(_lib.gb_grid_edges_host(side, extra, max_chain, seed, C.byref(n), C.byref(m),
                                   C.byref(s), C.byref(d)), "grid_edges")
    return n.value, _take(s, m.value, np.int32), _take(d, m.value, np.int32)


def batch_sizes(count: int, seed: int = 4, median: float = 2000.0, sigma: float = 1.5,
                n_min: int = 64, n_max: int = 500_000, ef_min: int = 4,
                ef_max: int = 32) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    ns = np.zeros(count, np.int32)
    efs = np.zeros(count, np.int32)
    seeds = np.zeros(count, np.uint64)
    _check(_lib.gb_batch_sizes(count, seed, median, sigma, n_min, n_max, ef_min, ef_max,
                               _ptr(ns), _ptr(efs), _ptr(seeds)), "batch_sizes")
    return ns, efs, seeds


def csr_from_edges(n: int, src: np.ndarray, dst: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Host CSR (int64 offsets, int32 adjacency) keyed by src, stable."""
    order = np.argsort(src, kind="stable")
    adj = np.ascontiguousarray(dst[order], dtype=np.int32)
    off = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(src, minlength=n), out=off[1:])
    return off, adj


# ---------------------------------------------------------------------------
# device objects
# ---------------------------------------------------------------------------
class Context:
    """A CUDA stream plus the device workspace of the runs (gb_ctx)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        self.device = device
        _check(_lib.gb_ctx_create(device, C.byref(self._h)), "gb_ctx_create")

    def close(self) -> None:
        if self._h:
            _lib.gb_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_class_opts(self, n_max, option_list) -> None:
        """Options per size class for runs given no options: entry i covers
        graphs of at most n_max[i] vertices (rising); the last covers the
        rest.  Empty lists remove the table."""
        nm = np.ascontiguousarray(n_max, np.int64)
        arr = (Opts * max(1, len(option_list)))(*option_list)
        _check(_lib.gb_ctx_set_class_opts(self._h, nm.size, _ptr(nm) if nm.size else None,
                                          C.cast(arr, C.c_void_p) if option_list else None),
               "gb_ctx_set_class_opts")

    def set_stream(self, stream_handle: int | None) -> None:
        _check(_lib.gb_ctx_set_stream(self._h, C.c_void_p(stream_handle or 0)), "set_stream")

    @property
    def stream(self) -> int:
        return _lib.gb_ctx_stream(self._h) or 0

    def sync(self) -> None:
        _check(_lib.gb_ctx_sync(self._h), "gb_ctx_sync")

    def reach_trace(self, cap: int = 128) -> list[tuple[int, int, int]]:
        """(device ns, vertices appended, mode bits) per reachability step of
        the last completed run."""
        t = np.zeros(cap, np.int64)
        cnt = np.zeros(cap, np.int32)
        mode = np.zeros(cap, np.int32)
        ex = np.zeros(3 * cap, np.int64)
        k = _lib.gb_ctx_reach_trace2(self._h, _ptr(t), _ptr(cnt), _ptr(mode), _ptr(ex), cap)
        return [(int(t[i]), int(cnt[i]), int(mode[i]), int(ex[3 * i]), int(ex[3 * i + 1]),
                 int(ex[3 * i + 2])) for i in range(k)]

    def block_times(self) -> np.ndarray:
        """Per block, device ns at which it finished the thread tier of the
        first pull step of the last run."""
        t = np.zeros(256, np.int64)
        k = _lib.gb_ctx_block_times(self._h, _ptr(t), 256)
        return t[:k]

    def phase_times(self, count: int) -> np.ndarray:
        """(count, 5) ms of the last runs: trim, reach, colour, canon, total."""
        out = np.zeros((count, 5), np.float64)
        _check(_lib.gb_ctx_phase_times(self._h, count, _ptr(out)), "gb_ctx_phase_times")
        return out

    def _run(self, fn, name, g, labels, o: Opts | None, want_stats: bool):
        st = Stats()
        if labels is None:
            labels = np.empty(g.n, np.int32)
        ptr = _ptr(labels) if isinstance(labels, np.ndarray) else C.c_void_p(int(labels))
        _check(fn(self._h, g._h, ptr, _optp(o), C.byref(st)), name)
        return (labels, st) if want_stats else labels

    def scc(self, g: "Graph", labels=None, o: Opts | None = None, stats: bool = False):
        """run_scc: canonical SCC labels (numpy int32, or into a device pointer)."""
        return self._run(_lib.gb_scc, "gb_scc", g, labels, o, stats)

    def wcc(self, g: "Graph", labels=None, o: Opts | None = None, stats: bool = False):
        """run_cc on the mirrored graph: WCC / CC labels."""
        return self._run(_lib.gb_wcc, "gb_wcc", g, labels, o, stats)

    cc = wcc

    def _edges(self, fn, name, n, src, dst, labels, o):
        if labels is None:
            labels = np.empty(n, np.int32)
        if isinstance(src, np.ndarray):
            s = np.ascontiguousarray(src, np.int32)
            d = np.ascontiguousarray(dst, np.int32)
            m, sp, dp = s.size, _ptr(s), _ptr(d)
        else:  # device pointers (ints) and their length as (ptr, m)
            (sp, m), (dp, _) = src, dst
            sp, dp = C.c_void_p(sp), C.c_void_p(dp)
        lp = _ptr(labels) if isinstance(labels, np.ndarray) else C.c_void_p(int(labels))
        _check(fn(self._h, n, m, sp, dp, lp, _optp(o)), name)
        return labels

    def scc_edges(self, n: int, src, dst, labels=None, o: Opts | None = None):
        """SCC labels straight from an edge list (gb_scc_edges)."""
        return self._edges(_lib.gb_scc_edges, "gb_scc_edges", n, src, dst, labels, o)

    def wcc_edges(self, n: int, src, dst, labels=None, o: Opts | None = None):
        """WCC labels straight from an edge list (gb_wcc_edges)."""
        return self._edges(_lib.gb_wcc_edges, "gb_wcc_edges", n, src, dst, labels, o)

    def scc_async(self, g: "Graph", labels_dev: int, o: Opts | None = None) -> None:
        _check(_lib.gb_scc_async(self._h, g._h, C.c_void_p(labels_dev), _optp(o)),
               "gb_scc_async")

    def wcc_async(self, g: "Graph", labels_dev: int, o: Opts | None = None) -> None:
        _check(_lib.gb_wcc_async(self._h, g._h, C.c_void_p(labels_dev), _optp(o)),
               "gb_wcc_async")

    def batch_scc(self, b: "Batch", labels=None, o: Opts | None = None, stats: bool = False):
        """SCC of every graph of a batch: labels (total_n) local to each graph."""
        return self._run(_lib.gb_batch_scc, "gb_batch_scc", b, labels, o, stats)

    def batch_wcc(self, b: "Batch", labels=None, o: Opts | None = None, stats: bool = False):
        return self._run(_lib.gb_batch_wcc, "gb_batch_wcc", b, labels, o, stats)

    def batch_scc_async(self, b: "Batch", labels_dev: int, o: Opts | None = None) -> None:
        _check(_lib.gb_batch_scc_async(self._h, b._h, C.c_void_p(labels_dev), _optp(o)),
               "gb_batch_scc_async")

    def tune(self, target, kind: int = 0, reps: int = 3) -> tuple["Opts", float, float]:
        """Autotuned options for a Graph or a Batch (gb_tune / gb_tune_batch),
        the best device time and the defaults' time, in ms."""
        o, ms = Opts(), (C.c_double * 2)()
        fn = _lib.gb_tune_batch if isinstance(target, Batch) else _lib.gb_tune
        _check(fn(self._h, target._h, int(kind), int(reps), C.byref(o), ms), "gb_tune")
        return o, ms[0], ms[1]

    def pivot(self, g: "Graph", kind: int = 0) -> tuple[int, float]:
        p, a = C.c_int32(), C.c_double()
        _check(_lib.gb_graph_pivot(self._h, g._h, kind, C.byref(p), C.byref(a)), "gb_graph_pivot")
        return p.value, a.value


class Graph:
    """A device-resident graph: out- and in-CSR (gb_graph)."""

    def __init__(self, handle: C.c_void_p, owned: bool = True):
        self._h = handle
        self._owned = owned
        n, m, sym = C.c_int32(), C.c_int64(), C.c_int32()
        _check(_lib.gb_graph_info(handle, C.byref(n), C.byref(m), C.byref(sym)), "gb_graph_info")
        self.n, self.m, self.symmetric = n.value, m.value, bool(sym.value)

    @classmethod
    def from_edges(cls, ctx: Context, n: int, src, dst) -> "Graph":
        """create_csr on the device; src/dst numpy int32 arrays or device
        pointers (ints) with m = len."""
        h = C.c_void_p()
        if isinstance(src, np.ndarray):
            s = np.ascontiguousarray(src, dtype=np.int32)
            d = np.ascontiguousarray(dst, dtype=np.int32)
            _check(_lib.gb_graph_from_edges(ctx._h, n, s.size, _ptr(s), _ptr(d), C.byref(h)),
                   "gb_graph_from_edges")
        else:
            raise TypeError("src/dst must be numpy arrays")
        return cls(h)

    @classmethod
    def from_file(cls, ctx: Context, path: str, chunk: int = 0) -> "Graph":
        """A graph file (the reference's text format or the binary format),
        parsed on the device."""
        h = C.c_void_p()
        _check(_lib.gb_graph_from_file2(ctx._h, str(path).encode(), chunk, C.byref(h)),
               "gb_graph_from_file")
        return cls(h)

    @classmethod
    def from_csr(cls, ctx: Context, n: int, out_off, out_adj, in_off=None, in_adj=None) -> "Graph":
        h = C.c_void_p()
        oo = np.ascontiguousarray(out_off, dtype=np.int64)
        oa = np.ascontiguousarray(out_adj, dtype=np.int32)
        io = None if in_off is None else np.ascontiguousarray(in_off, dtype=np.int64)
        ia = None if in_adj is None else np.ascontiguousarray(in_adj, dtype=np.int32)
        _check(_lib.gb_graph_from_csr(ctx._h, n, oa.size, _ptr(oo), _ptr(oa), _ptr(io), _ptr(ia),
                                      C.byref(h)), "gb_graph_from_csr")
        return cls(h)

    @classmethod
    def from_csr32(cls, ctx: Context, n: int, out_array, out_degree_list, in_array=None,
                   in_degree_list=None) -> "Graph":
        """gb_graph_from_csr32: the reference's 32-bit CSR layout.  With
        in_degree_list given and in_array None, the in-lists are derived on
        the device from the out-CSR.  Arrays are used as given (pinned
        arrays are read by the device directly), so they must already be
        contiguous uint32 offsets and int32 ids."""
        h = C.c_void_p()
        m = int(out_degree_list[n])
        _check(_lib.gb_graph_from_csr32(ctx._h, n, m, _ptr(out_array), _ptr(out_degree_list),
                                        _ptr(in_array), _ptr(in_degree_list), C.byref(h)),
               "gb_graph_from_csr32")
        return cls(h)

    @classmethod
    def rmat(cls, ctx: Context, scale: int, edge_factor: int = 16, seed: int = 1,
             abc: tuple[float, float, float] = RMAT_ABC) -> "Graph":
        h = C.c_void_p()
        _check(_lib.gb_graph_rmat(ctx._h, scale, edge_factor, seed, abc[0], abc[1], abc[2],
                                  C.byref(h)), "gb_graph_rmat")
        return cls(h)

    @classmethod
    def rmat_n(cls, ctx: Context, n: int, edge_factor: int, seed: int,
               abc: tuple[float, float, float] = RMAT_ABC) -> "Graph":
        h = C.c_void_p()
        _check(_lib.gb_graph_rmat_n(ctx._h, n, edge_factor, seed, abc[0], abc[1], abc[2],
                                    C.byref(h)), "gb_graph_rmat_n")
        return cls(h)

    def to_host(self) -> tuple[np.ndarray, np.ndarray, np.ndarray | None, np.ndarray | None]:
        oo = np.empty(self.n + 1, np.int64)
        oa = np.empty(self.m, np.int32)
        io = None if self.symmetric else np.empty(self.n + 1, np.int64)
        ia = None if self.symmetric else np.empty(self.m, np.int32)
        _check(_lib.gb_graph_csr_to_host(self._h, _ptr(oo), _ptr(oa), _ptr(io), _ptr(ia)),
               "gb_graph_csr_to_host")
        return oo, oa, io, ia

    def set_hints(self, ctx: Context, on: bool) -> None:
        """Builds (on) or frees (off) the graph's pull hints."""
        _check(_lib.gb_graph_set_hints(ctx._h, self._h, 1 if on else 0), "gb_graph_set_hints")

    def hints(self) -> tuple[np.ndarray, np.ndarray | None]:
        """The pull hints (out side, in side) on the host."""
        ho = np.empty(self.n, np.int32)
        hi = None if self.symmetric else np.empty(self.n, np.int32)
        _check(_lib.gb_graph_hints_to_host(self._h, _ptr(ho), _ptr(hi)), "gb_graph_hints_to_host")
        return ho, hi

    @property
    def has_hints(self) -> bool:
        v = C.c_int32()
        _check(_lib.gb_graph_has_hints(self._h, C.byref(v)), "gb_graph_has_hints")
        return bool(v.value)

    def device_csr(self) -> tuple[int, int, int, int]:
        ps = [C.c_void_p() for _ in range(4)]
        _check(_lib.gb_graph_device_csr(self._h, *[C.byref(p) for p in ps]), "gb_graph_device_csr")
        return tuple(p.value or 0 for p in ps)

    def close(self) -> None:
        if self._h and self._owned:
            _lib.gb_graph_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent graphs stored as one disjoint union (gb_batch)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        cnt, tn, tm = C.c_int32(), C.c_int64(), C.c_int64()
        _check(_lib.gb_batch_info(handle, C.byref(cnt), C.byref(tn), C.byref(tm)), "gb_batch_info")
        self.count, self.n, self.m = cnt.value, tn.value, tm.value
        self.vbase = np.zeros(self.count + 1, np.int64)
        _check(_lib.gb_batch_vbase(handle, _ptr(self.vbase)), "gb_batch_vbase")

    @classmethod
    def rmat(cls, ctx: Context, ns, efs, seeds,
             abc: tuple[float, float, float] = RMAT_ABC) -> "Batch":
        ns = np.ascontiguousarray(ns, np.int32)
        efs = np.ascontiguousarray(efs, np.int32)
        seeds = np.ascontiguousarray(seeds, np.uint64)
        h = C.c_void_p()
        _check(_lib.gb_batch_rmat(ctx._h, ns.size, _ptr(ns), _ptr(efs), _ptr(seeds), abc[0],
                                  abc[1], abc[2], C.byref(h)), "gb_batch_rmat")
        return cls(h)

    @classmethod
    def from_edges(cls, ctx: Context, vbase, src, dst) -> "Batch":
        vb = np.ascontiguousarray(vbase, np.int64)
        s = np.ascontiguousarray(src, np.int32)
        d = np.ascontiguousarray(dst, np.int32)
        h = C.c_void_p()
        _check(_lib.gb_batch_from_edges(ctx._h, vb.size - 1, _ptr(vb), s.size, _ptr(s), _ptr(d),
                                        C.byref(h)), "gb_batch_from_edges")
        return cls(h)

    def graph(self) -> Graph:
        """The union as a Graph (owned by the batch)."""
        h = C.c_void_p()
        _check(_lib.gb_batch_graph(self._h, C.byref(h)), "gb_batch_graph")
        return Graph(h, owned=False)

    def split(self, labels: np.ndarray) -> list[np.ndarray]:
        return [labels[self.vbase[i]:self.vbase[i + 1]] for i in range(self.count)]

    def close(self) -> None:
        if self._h:
            _lib.gb_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A request loop with continuous batching (gb_server) over one Context.

    submit() takes host edge arrays and returns a request id; the labels
    land in the array returned by result() once wait() has returned.  The
    arrays passed to submit() are kept alive here until the request is done.
    """

    SCC, WCC = 0, 1

    def __init__(self, ctx: Context, budget_bytes: int = 0, max_graphs: int = 4096):
        self.ctx = ctx
        h = C.c_void_p()
        _check(_lib.gb_server_create(ctx._h, int(budget_bytes), int(max_graphs), C.byref(h)),
               "gb_server_create")
        self._h = h
        self._keep: dict[int, tuple] = {}

    def set_opts(self, o: "Opts") -> None:
        """Options of the merged runs (before start)."""
        _check(_lib.gb_server_set_opts(self._h, C.byref(o)), "gb_server_set_opts")

    def start(self) -> None:
        _check(_lib.gb_server_start(self._h), "gb_server_start")

    def submit(self, kind: int, n: int, src, dst, arrival_ns: int = -1,
               out: np.ndarray | None = None) -> int:
        s = np.ascontiguousarray(src, np.int32)
        d = np.ascontiguousarray(dst, np.int32)
        if s.shape != d.shape:
            raise ValueError("src and dst differ in length")
        lab = out if out is not None else np.empty(n, np.int32)
        if lab.dtype != np.int32 or lab.size < n or not lab.flags.c_contiguous:
            raise ValueError("out must be a contiguous int32 array of n entries")
        rid = C.c_int64()
        _check(_lib.gb_server_submit(self._h, int(kind), int(n), s.size, _ptr(s), _ptr(d),
                                     _ptr(lab), int(arrival_ns), C.byref(rid)), "gb_server_submit")
        self._keep[rid.value] = (s, d, lab)
        return rid.value

    def wait(self, rid: int) -> tuple[np.ndarray, float]:
        """Labels and latency (ms) of request rid."""
        lat = C.c_int64()
        st = _lib.gb_server_wait(self._h, int(rid), C.byref(lat))
        keep = self._keep.pop(rid, None)
        _check(st, "gb_server_wait")
        return keep[2], lat.value / 1e6

    def drain(self) -> None:
        _check(_lib.gb_server_drain(self._h), "gb_server_drain")

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(_lib.gb_server_stats_get(self._h, C.byref(s)), "gb_server_stats_get")
        return s

    def close(self) -> None:
        if self._h:
            _lib.gb_server_destroy(self._h)
            self._h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_scc_ref(n: int, out_array, in_array, out_degree_list, in_degree_list,
                max_deg_vert: int = -1, avg_degree: float = 0.0, vert_cutoff: int = 10000,
                scc_maps: np.ndarray | None = None) -> np.ndarray:
    """gb_run_scc: the reference's run_scc signature on host buffers
    (32-bit offsets as in its graph struct)."""
    if scc_maps is None:
        scc_maps = np.empty(n, np.int32)
    m = int(out_degree_list[n])
    _check(_lib.gb_run_scc(n, m, _ptr(out_array), _ptr(in_array), _ptr(out_degree_list),
                           _ptr(in_degree_list), _ptr(scc_maps), max_deg_vert, avg_degree,
                           vert_cutoff), "gb_run_scc")
    return scc_maps


def dropin_set_derive_share(share: float) -> None:
    """gb_dropin_set_derive_share: the share of in-edges whose lists
    gb_run_scc derives on the device from the out-CSR (1: in_array is not
    read; 0: it is copied whole)."""
    _check(_lib.gb_dropin_set_derive_share(float(share)), "gb_dropin_set_derive_share")


def run_cc_ref(n: int, out_array, out_degree_list, max_deg_vert: int = -1,
               avg_degree: float = 0.0, cc_maps: np.ndarray | None = None) -> np.ndarray:
    """gb_run_cc: the reference's run_cc signature on the mirrored host CSR."""
    if cc_maps is None:
        cc_maps = np.empty(n, np.int32)
    m = int(out_degree_list[n])
    _check(_lib.gb_run_cc(n, m, _ptr(out_array), _ptr(out_degree_list), _ptr(cc_maps),
                          max_deg_vert, avg_degree), "gb_run_cc")
    return cc_maps


@dataclass
class Info:
    lib_path: str = LIB_PATH


__all__ = [
    "Context", "Graph", "GBError", "Opts", "Stats", "opts", "read_edge", "output_labels",
    "scc_verify", "cc_verify", "canonicalize", "rmat_edges", "grid_edges", "batch_sizes",
    "csr_from_edges", "run_scc_ref", "run_cc_ref", "LIB_PATH", "Batch", "rmat_edges_n",
    "dropin_set_derive_share",
]
