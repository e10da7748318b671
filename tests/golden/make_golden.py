"""Generates the golden fixtures in tests/golden/ from the UNMODIFIED
reference Multistep code (oracle/_ref, built by oracle/build_ref.sh where the
reference tree exists).

    python tests/golden/make_golden.py

For every case it stores the reference's own output, canonicalised to the
minimum member id of each component, its verify lines, and a SHA-256 digest
of the generated edge list (so a test can tell a generator change from a
labelling change).  Graphs come from the seeded generators of libgbconn
(host side) and from tests/graphs.py.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import connectivity_gb300 as gb  # noqa: E402
import oracle  # noqa: E402
from tests import graphs  # noqa: E402

RMAT_CASES = [(10, 16, 1), (12, 16, 1), (14, 16, 1), (16, 16, 1), (12, 4, 2), (16, 32, 3)]
GRID_CASES = [(32, 2), (64, 2), (128, 2)]


def digest(n, s, d) -> str:
    h = hashlib.sha256()
    h.update(np.int64(n).tobytes())
    h.update(np.ascontiguousarray(s, np.int32).tobytes())
    h.update(np.ascontiguousarray(d, np.int32).tobytes())
    return h.hexdigest()


def cases():
    for sc, ef, seed in RMAT_CASES:
        yield f"rmat_s{sc}_ef{ef}_seed{seed}", gb.rmat_edges(sc, ef, seed)
    for side, seed in GRID_CASES:
        yield f"grid_{side}_seed{seed}", gb.grid_edges(side, side * side // 10, 64, seed)
    for name, n, s, d in graphs.edge_cases():
        yield f"edge_{name}", (n, s, d)


def main():
    if not oracle.ref_available():
        sys.exit("oracle/_ref is not built (needs the reference tree)")
    index = {}
    for name, (n, s, d) in cases():
        scc_raw, scc_line, _ = oracle.ref_run("scc", n, s, d)
        cc_raw, cc_line, _ = oracle.ref_run("cc", n, s, d)
        scc = oracle.canonical(scc_raw)
        cc = oracle.canonical(cc_raw)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), scc=scc, cc=cc)
        index[name] = {"n": int(n), "m": int(s.size), "digest": digest(n, s, d),
                       "scc_verify": scc_line, "cc_verify": cc_line}
        print(name, n, s.size, scc_line.strip(), "|", cc_line.strip())
    # the reference's own fixture (multistep/test.graph: the same five edges
    # as graphs.test_graph, duplicate included) through its unchanged main
    tg = os.path.join(HERE, "test_graph.txt")
    n, s, d = graphs.test_graph()
    with open(tg, "w") as f:
        f.write(f"{n} {s.size}\n" + "".join(f"{a} {b}\n" for a, b in zip(s, d)))
    scc_lab, scc_line = oracle.ref_text("scc", tg)
    cc_lab, cc_line = oracle.ref_text("cc", tg)
    index["test_graph_text"] = {"scc": scc_lab.tolist(), "cc": cc_lab.tolist(),
                                "scc_verify": scc_line, "cc_verify": cc_line}
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
