"""Generates the golden vectors in tests/golden/ (run here, where the
reference tree exists; the outputs travel with the repository).

Inputs:
  * the reference's own fixture graphs (test-graphs/small.mtx,
    trivialGraph.mtx, chesapeake.mtx), parsed by the reference's graphio.cpp
    loader compiled in oracle/_ref/libgas_ref.so;
  * small synthetic graphs from this package's generators (R-MAT, lattice),
    whose edge-list hashes are recorded so a generator change is caught.

Outputs, per graph, one compressed .npz holding the edge list and the
results of the reference's compiled CPU engine (GASEngineRef, refgas.h)
for BFS, SSSP, CC and PageRank (FP32 and FP64), plus personalised PageRank
from the oracle restatement (the reference has no PPR program).

    python tests/golden/make_golden.py
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

import oracle  # noqa: E402
from vertexapi2_gb300 import graphs  # noqa: E402
from vertexapi2_gb300.programs import max_outdegree_vertex  # noqa: E402

REF_FIXTURES = ["small.mtx", "trivialGraph.mtx", "chesapeake.mtx"]


def edge_hash(srcs, dsts, w=None) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(srcs, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(dsts, dtype="<i4").tobytes())
    if w is not None:
        h.update(np.ascontiguousarray(w, dtype="<i4").tobytes())
    return h.hexdigest()


def synthetic():
    out = []
    g = graphs.rmat(8, 16, seed=11, symmetrize=True, weights=(1, 255))
    out.append(("rmat8_sym", g))
    g = graphs.rmat(10, 16, seed=12, symmetrize=False, weights=(1, 100))
    out.append(("rmat10_dir", g))
    g = graphs.grid(16, 16, 0.15, seed=13, weights=(1, 100))
    out.append(("grid16", g))
    g = graphs.grid(40, 30, 0.15, seed=14, weights=(1, 100))
    out.append(("grid40x30", g))
    return [(n, g.n_vertices, g.srcs, g.dsts, g.weights) for n, g in out]


def main() -> None:
    ref = oracle.ref()
    if ref is None:
        sys.exit("the reference engine (oracle/_ref) is not available here")
    port = oracle.port()
    ref_dir = oracle._build.ref_dir()
    cases = []
    for fn in REF_FIXTURES:
        nv, s, d, w = ref.load_graph(os.path.join(ref_dir, "test-graphs", fn))
        cases.append((os.path.splitext(fn)[0], nv, s, d, w))
    cases += synthetic()
    index = {}
    for name, nv, s, d, w in cases:
        rec = {"n_vertices": np.int64(nv), "srcs": s.astype(np.int32), "dsts": d.astype(np.int32)}
        src_bfs = max_outdegree_vertex(nv, s) if len(s) else 0
        rec["bfs_source"] = np.int64(src_bfs)
        rec["bfs"], _ = ref.bfs(nv, s, d, src_bfs)
        rec["cc"], _ = ref.cc(nv, s, d)
        rec["pr32"], st = ref.pagerank(nv, s, d)
        rec["pr32_iterations"] = np.int64(st["iterations"])
        rec["pr64"], _ = ref.pagerank(nv, s, d, fp64=True)
        rec["ppr32"], _ = port.ppr(nv, s, d, src_bfs, iters=20)
        rec["ppr64"], _ = port.ppr(nv, s, d, src_bfs, iters=20, fp64=True)
        if w is not None:
            rec["weights"] = w.astype(np.int32)
            rec["sssp"], _ = ref.sssp(nv, s, d, w, 0)
        # per-round frontier counts (restatement), for the GPU round stats
        _, st = port.bfs(nv, s, d, src_bfs, stats_cap=4096)
        rec["bfs_active"] = st["active"]
        _, st = port.cc(nv, s, d, stats_cap=4096)
        rec["cc_active"] = st["active"]
        rec["cc_gathered"] = st["gathered"]
        rec["cc_scattered"] = st["scattered"]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        index[name] = {"n_vertices": int(nv), "n_edges": int(len(s)),
                       "edge_sha256": edge_hash(s, d, w),
                       "weighted": w is not None}
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_golden.py",
                   "engine": "reference GASEngineRef (refgas.h) compiled in place",
                   "graphs": index}, f, indent=1, sort_keys=True)
    print(json.dumps(index, indent=1))


if __name__ == "__main__":
    main()
