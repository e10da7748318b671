"""The full-size workloads against the reference: the GPU's canonical labels
must hash to the digests of the unmodified reference's labels on the same
edge lists, and its verify lines must equal the reference's
(tests/golden/pins.json, made by tests/golden/make_pins.py)."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

import connectivity_gb300 as gb

pytestmark = pytest.mark.gpu

PINS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                   "pins.json")))


def _lab(x):
    return hashlib.sha256(np.ascontiguousarray(x, "<i4").tobytes()).hexdigest()


def _edges(n, s, d):
    h = hashlib.sha256()
    h.update(np.int64(n).tobytes())
    h.update(np.ascontiguousarray(s, np.int32).tobytes())
    h.update(np.ascontiguousarray(d, np.int32).tobytes())
    return h.hexdigest()


def _check(ctx, g, pin, variants=({},)):
    for o in variants:
        lab = ctx.scc(g, o=gb.opts(**o))
        assert _lab(lab) == pin["scc_labels"], o
        assert gb.scc_verify(lab) == pin["scc_verify"]
    lab = ctx.wcc(g)
    assert _lab(lab) == pin["cc_labels"]
    assert gb.cc_verify(lab) == pin["cc_verify"]


@pytest.mark.parametrize("scale", [20, 22, 24])
def test_rmat_scc_and_wcc_equal_reference(ctx, scale):
    pin = PINS[f"rmat_s{scale}_ef16_seed1"]
    g = gb.Graph.rmat(ctx, scale, 16, 1)
    assert (g.n, g.m) == (pin["n"], pin["m"])
    # the device-built graph holds the pinned edge list: its out-CSR read in
    # order is the generated list (sorted by source, then target)
    oo, oa, _, _ = g.to_host()
    src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(oo))
    assert _edges(g.n, src, oa) == pin["edges"]
    del oo, oa, src
    variants = ({}, {"trim_level": 2}, {"trim_pairs": 1, "fwbw_rounds": 3}) if scale < 24 else ({},)
    _check(ctx, g, pin, variants)
    # and without the pull hints
    g.set_hints(ctx, False)
    assert not g.has_hints
    _check(ctx, g, pin)
    g.set_hints(ctx, True)
    assert g.has_hints
    g.close()


@pytest.mark.parametrize("side", [1024, 2048, 4096])
def test_grid_scc_and_wcc_equal_reference(ctx, side):
    key = f"grid_{side}_seed2"
    if key not in PINS:
        pytest.skip(f"{key} not pinned")
    pin = PINS[key]
    n, s, d = gb.grid_edges(side, side * side // 10, 64, 2)
    assert _edges(n, s, d) == pin["edges"]
    g = gb.Graph.from_edges(ctx, n, s, d)
    _check(ctx, g, pin, ({}, {"trim_level": 2}) if side < 4096 else ({},))
    g.close()
