"""gb_scc_noalloc: the SCC entry point for callers that may not allocate
device memory (its scratch is a fixed static device array inside the
library).  Called through the C ABI on a graph already in device memory, it
must give exactly the labels of gb_scc, on two calls in a row (the second
call starts from the first call's leftover scratch).  Collected last so that
a failure here comes after every other test has run."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import connectivity_gb300 as gb

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 18


def _fn():
    lib = C.CDLL(gb.LIB_PATH)
    f = lib.gb_scc_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_int32, C.c_int64] + [C.c_void_p] * 6
    return f


@pytest.mark.parametrize("scale,ef,seed", [(16, 16, 1), (17, 8, 3)])
def test_noalloc_matches_gb_scc_twice(scale, ef, seed):
    torch = pytest.importorskip("torch")
    ctx = gb.Context(0)
    g = gb.Graph.rmat(ctx, scale, ef, seed)
    want = ctx.scc(g)
    oo, oa, io, ia = g.device_csr()
    f = _fn()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out = torch.full((g.n,), -5, dtype=torch.int32, device="cuda:0")
        st = f(g.n, g.m, oo, oa, io, ia, out.data_ptr(), stream)
        assert st == 0, gb._lib.gb_last_error()
        assert np.array_equal(out.cpu().numpy(), want)
    g.close()
    ctx.close()


def test_noalloc_rejects_oversize_graph():
    f = _fn()
    # nothing is queued for a graph larger than the fixed scratch
    st = f(MAX_VERTICES + 1, 0, 1, 1, 1, 1, 1, None)
    assert st == 9  # GB_ERR_CAPACITY
