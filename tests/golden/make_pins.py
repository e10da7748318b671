"""Pins the full-size workloads to the UNMODIFIED reference Multistep code.

    python tests/golden/make_pins.py [case ...]

The label arrays of these graphs are too large to commit, so for each case
this stores, in tests/golden/pins.json:

* the SHA-256 digest of the generated edge list (n, sources, targets; the
  same digest as index.json uses), so a generator change is told apart from
  a labelling change;
* the SHA-256 digest of the reference's labels after canonicalisation to the
  minimum member id of each component, as little-endian int32;
* the reference's own verify lines (scc_verify / cc_verify) and its run
  times on the host that made the pin.

SCC runs run_scc on the directed graph (scc_main.cpp:368-378); CC runs run_cc
on the mirrored graph that cc's reader builds (cc_main.cpp:102-118, timed at
:296-302).  The reference is oracle/_ref (oracle/build_ref.sh).  Without a
case argument every case is (re)made; the grid case needs about half an hour
of 8 host cores for its SCC.
"""
from __future__ import annotations

import hashlib
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import connectivity_gb300 as gb  # noqa: E402
import oracle  # noqa: E402

PINS = os.path.join(HERE, "pins.json")

# name -> generator; the R-MAT cases use a=0.57 b=0.19 c=0.19, the lattices
# n/10 chain vertices of length 1..64.
CASES = {
    "rmat_s20_ef16_seed1": lambda: gb.rmat_edges(20, 16, 1),
    "rmat_s22_ef16_seed1": lambda: gb.rmat_edges(22, 16, 1),
    "rmat_s24_ef16_seed1": lambda: gb.rmat_edges(24, 16, 1),
    "grid_1024_seed2": lambda: gb.grid_edges(1024, 1024 * 1024 // 10, 64, 2),
    "grid_2048_seed2": lambda: gb.grid_edges(2048, 2048 * 2048 // 10, 64, 2),
    "grid_4096_seed2": lambda: gb.grid_edges(4096, 4096 * 4096 // 10, 64, 2),
}


def edge_digest(n, s, d) -> str:
    h = hashlib.sha256()
    h.update(np.int64(n).tobytes())
    h.update(np.ascontiguousarray(s, np.int32).tobytes())
    h.update(np.ascontiguousarray(d, np.int32).tobytes())
    return h.hexdigest()


def label_digest(canonical_labels: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(canonical_labels, "<i4").tobytes()).hexdigest()


def make(name: str) -> dict:
    n, s, d = CASES[name]()
    entry = {"n": int(n), "m": int(s.size), "edges": edge_digest(n, s, d),
             "host": f"{platform.machine()} x {os.cpu_count()} threads"}
    for kind in ("scc", "cc"):
        t0 = time.time()
        raw, line, best = oracle.ref_run(kind, n, s, d)
        lab = oracle.canonical(raw)
        entry[f"{kind}_labels"] = label_digest(lab)
        entry[f"{kind}_verify"] = line
        entry[f"{kind}_ref_seconds"] = best
        print(f"{name} {kind}: {line.strip()} ({best:.3f} s timed, {time.time() - t0:.1f} s wall)",
              flush=True)
    return entry


def main(argv: list[str]) -> None:
    if not oracle.ref_available():
        sys.exit("oracle/_ref is not built (needs the reference tree)")
    names = argv or list(CASES)
    for name in names:
        if name not in CASES:
            sys.exit(f"unknown case {name}; one of {', '.join(CASES)}")
    for name in names:
        entry = make(name)
        pins = {}
        if os.path.exists(PINS):
            with open(PINS) as f:
                pins = json.load(f)
        pins[name] = entry
        with open(PINS, "w") as f:
            json.dump(pins, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:])
