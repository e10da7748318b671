"""gb_scc_noalloc: the SCC entry point for callers that may not allocate
device memory (its scratch is a fixed static device array inside the
library).  Called through the C ABI on a graph already in device memory, it
must give exactly the labels of gb_scc, on two calls in a row (the second
call starts from the first call's leftover scratch), and the reference's
labels where a golden fixture holds them.  Collected last so that a failure
here comes after every other test has run."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

import connectivity_gb300 as gb

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 18
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fn():
    lib = C.CDLL(gb.LIB_PATH)
    f = lib.gb_scc_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_int32, C.c_int64] + [C.c_void_p] * 6
    return f


def _noalloc(f, torch, g, stream):
    oo, oa, io, ia = g.device_csr()
    out = torch.full((g.n,), -5, dtype=torch.int32, device="cuda:0")
    st = f(g.n, g.m, oo, oa, io, ia, out.data_ptr(), stream)
    assert st == 0, gb._lib.gb_last_error()
    return out.cpu().numpy()


@pytest.mark.parametrize("scale,ef,seed", [(16, 16, 1), (17, 8, 3)])
def test_noalloc_matches_gb_scc_twice(scale, ef, seed):
    torch = pytest.importorskip("torch")
    ctx = gb.Context(0)
    g = gb.Graph.rmat(ctx, scale, ef, seed)
    want = ctx.scc(g)
    f = _fn()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        assert np.array_equal(_noalloc(f, torch, g, stream), want)
    name = f"rmat_s{scale}_ef{ef}_seed{seed}.npz"
    if os.path.exists(os.path.join(GOLDEN, name)):
        # the same graph run by the reference (canonical labels)
        assert np.array_equal(want, np.load(os.path.join(GOLDEN, name))["scc"])
    g.close()
    ctx.close()


def test_noalloc_smaller_after_larger_and_at_capacity():
    """A small graph after a large one (stale scratch past the new n) and a
    graph of exactly the maximum size, each against gb_scc."""
    torch = pytest.importorskip("torch")
    ctx = gb.Context(0)
    f = _fn()
    stream = torch.cuda.current_stream().cuda_stream
    gs = [gb.Graph.rmat(ctx, 18, 8, 5), gb.Graph.rmat(ctx, 10, 16, 1)]
    n, s, d = 3, np.array([0, 1, 0, 1, 0], np.int32), np.array([1, 2, 2, 0, 2], np.int32)
    gs.append(gb.Graph.from_edges(ctx, n, s, d))  # the reference's test.graph
    assert gs[0].n == MAX_VERTICES
    for g in gs:
        want = ctx.scc(g)
        for _ in range(2):
            assert np.array_equal(_noalloc(f, torch, g, stream), want)
    assert list(_noalloc(f, torch, gs[2], stream)) == [0, 0, 2]
    for g in gs:
        g.close()
    ctx.close()


def test_noalloc_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    f = _fn()
    # nothing is queued for a graph larger than the fixed scratch
    assert f(MAX_VERTICES + 1, 0, 1, 1, 1, 1, 1, None) == 9  # GB_ERR_CAPACITY
    # a host array is refused before any kernel runs
    n = 4
    off = np.array([0, 1, 2, 3, 4], np.int64)
    adj = np.array([1, 2, 3, 0], np.int32)
    lab = np.zeros(n, np.int32)
    hp = [a.ctypes.data for a in (off, adj, off, adj, lab)]
    assert f(n, 4, *hp, None) == 1  # GB_ERR_INVALID
    # device arrays of the declared sizes holding an id outside [0, n): the
    # check reads only within them and refuses the CSR
    d_off = torch.from_numpy(off).cuda()
    bad_adj = torch.tensor([1, 2, 7, 0], dtype=torch.int32, device="cuda")
    good_adj = torch.from_numpy(adj).cuda()
    in_adj = torch.tensor([3, 0, 1, 2], dtype=torch.int32, device="cuda")  # the cycle's in-CSR
    d_lab = torch.zeros(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert f(n, 4, d_off.data_ptr(), bad_adj.data_ptr(), d_off.data_ptr(), in_adj.data_ptr(),
             d_lab.data_ptr(), stream) == 1
    # offsets that do not end at m
    short = torch.tensor([0, 1, 2, 3, 3], dtype=torch.int64, device="cuda")
    assert f(n, 4, short.data_ptr(), good_adj.data_ptr(), d_off.data_ptr(),
             in_adj.data_ptr(), d_lab.data_ptr(), stream) == 1
    # and the same call on the good CSR still works: one cycle
    assert f(n, 4, d_off.data_ptr(), good_adj.data_ptr(), d_off.data_ptr(), in_adj.data_ptr(),
             d_lab.data_ptr(), stream) == 0
    assert d_lab.cpu().tolist() == [0, 0, 0, 0]
