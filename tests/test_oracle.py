"""The oracle (CPU restatement of GASEngineRef) against the reference.

* against the golden vectors produced by the reference's own compiled
  engine (tests/golden, make_golden.py) -- runs everywhere;
* against the compiled reference engine itself on fresh random graphs --
  only where oracle/_ref could be built (the reference tree is present).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden

import oracle


def rel_l1(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_golden(port, name):
    g = load_golden(name)
    nv, s, d = int(g["n_vertices"]), g["srcs"], g["dsts"]
    src = int(g["bfs_source"])
    assert np.array_equal(port.bfs(nv, s, d, src)[0], g["bfs"])
    assert np.array_equal(port.cc(nv, s, d)[0], g["cc"])
    if "weights" in g:
        assert np.array_equal(port.sssp(nv, s, d, g["weights"], 0)[0], g["sssp"])
    pr64, _ = port.pagerank(nv, s, d, fp64=True)
    # FP64 sums in a different edge order than std::sort's: rounding only
    assert np.allclose(pr64, g["pr64"], rtol=1e-12, atol=1e-12)
    pr32, st = port.pagerank(nv, s, d)
    # pagerank.cu:154-158 compares ranks with |diff| <= 1e-6; ranks here
    # reach ~20 where one float32 ulp is 2e-6, so the bound is relative
    assert np.allclose(pr32, g["pr32"], rtol=1e-6, atol=1e-6)
    assert rel_l1(pr32, g["pr32"]) < 1e-6
    ppr32, _ = port.ppr(nv, s, d, src, iters=20)
    assert np.array_equal(ppr32, g["ppr32"])
    # per-round frontier counts of the restatement are pinned too
    _, st = port.bfs(nv, s, d, src, stats_cap=4096)
    assert np.array_equal(st["active"], g["bfs_active"])


def test_known_answers_small(port):
    # values of the reference engine on test-graphs/small.mtx (0-based)
    g = load_golden("small")
    nv, s, d, w = int(g["n_vertices"]), g["srcs"], g["dsts"], g["weights"]
    assert port.sssp(nv, s, d, w, 0)[0].tolist() == [0, 1, 4, 1, 2, 2, 2]
    pr, _ = port.pagerank(nv, s, d)
    assert np.allclose(pr, [0.15, 0.247042, 0.1925, 0.1925, 0.414527, 0.286354, 0.827562],
                       atol=1e-6)


def test_fp32_vs_fp64_pagerank_error_small(port):
    for name in golden_names():
        g = load_golden(name)
        assert rel_l1(g["pr32"], g["pr64"]) < 1e-5


def test_oracle_rejects_bad_ids(port):
    with pytest.raises(ValueError):
        port.bfs(3, np.array([0, 5]), np.array([1, 2]), 0)
    with pytest.raises(ValueError):
        port.bfs(3, np.array([0]), np.array([1]), 7)


def test_oracle_edge_cases(port):
    # no edges: only the source is reached, one round
    d, st = port.bfs(4, np.zeros(0, np.int32), np.zeros(0, np.int32), 2, stats_cap=8)
    assert d.tolist() == [-1, -1, 0, -1] and st["iterations"] == 1
    lab, _ = port.cc(4, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert lab.tolist() == [0, 1, 2, 3]
    # unreachable vertices keep gatherZero as their distance
    dist, _ = port.sssp(3, np.array([0]), np.array([1]), np.array([5]), 0)
    assert dist.tolist() == [0, 5, oracle.SSSP_UNREACHED]


@pytest.mark.skipif(oracle.ref() is None, reason="reference tree not present")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_port_matches_reference_engine(port, seed):
    from vertexapi2_gb300 import graphs
    from vertexapi2_gb300.programs import max_outdegree_vertex
    ref = oracle.ref()
    for g in (graphs.rmat(11, 8, seed=seed, symmetrize=True, weights=(1, 255)),
              graphs.rmat(11, 8, seed=seed + 10, weights=(1, 100)),
              graphs.grid(50, 60, 0.2, seed=seed)):
        nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
        src = max_outdegree_vertex(nv, s)
        a, sa = port.bfs(nv, s, d, src)
        b, sb = ref.bfs(nv, s, d, src)
        assert np.array_equal(a, b) and sa["iterations"] == sb["iterations"]
        a, sa = port.sssp(nv, s, d, w, 0)
        b, sb = ref.sssp(nv, s, d, w, 0)
        assert np.array_equal(a, b) and sa["iterations"] == sb["iterations"]
        assert np.array_equal(port.cc(nv, s, d)[0], ref.cc(nv, s, d)[0])
        a, sa = port.pagerank(nv, s, d, max_iters=50, fp64=True)
        b, sb = ref.pagerank(nv, s, d, max_iters=50, fp64=True)
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
        assert sa["iterations"] == sb["iterations"]


def test_scatter_program_port_matches_reference():
    """A Program whose scatter writes its edge (visit count, source
    distance): the restatement calls Program::scatter as refgas.h does."""
    import oracle
    from vertexapi2_gb300 import graphs
    ref = oracle.ref()
    if ref is None:
        pytest.skip("reference engine not built")
    port = oracle.port()
    for seed in range(4):
        g = graphs.rmat(9, 8, seed=70 + seed, weights=(1, 30))
        a = port.sssp_visits(g.n_vertices, g.srcs, g.dsts, g.weights, seed)
        b = ref.sssp_visits(g.n_vertices, g.srcs, g.dsts, g.weights, seed)
        for x, y in zip(a[:3], b[:3]):
            assert np.array_equal(x, y)
        assert a[1].sum() > 0


# The oracle's generators (gas_oracle_gen.c) are a second implementation of
# the benchmark graphs, used where the product library must not be loaded.
GEN_CASES = {
    "rmat8_sym": ("rmat", dict(scale=8, seed=11, symmetrize=True, weights=(1, 255))),
    "rmat10_dir": ("rmat", dict(scale=10, seed=12, symmetrize=False, weights=(1, 100))),
    "grid16": ("grid", (16, 16, 0.15, 13)),
    "grid40x30": ("grid", (40, 30, 0.15, 14)),
}


@pytest.mark.parametrize("name", sorted(GEN_CASES))
def test_oracle_generators_match_golden_hashes(port, name):
    import hashlib
    import json
    import os
    from conftest import GOLDEN
    idx = json.load(open(os.path.join(GOLDEN, "index.json")))["graphs"][name]
    kind, args = GEN_CASES[name]
    nv, s, d, w = port.gen_rmat(**args) if kind == "rmat" else port.gen_grid(*args)
    assert nv == idx["n_vertices"] and len(s) == idx["n_edges"]
    h = hashlib.sha256()  # tests/golden/make_golden.py edge_hash
    for a in (s, d, w):
        h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
    assert h.hexdigest() == idx["edge_sha256"]


@pytest.mark.parametrize("kind,args", [
    ("rmat", dict(scale=16, seed=1, symmetrize=True)),             # BFS benchmark graph
    ("rmat", dict(scale=14, seed=15, symmetrize=True, weights=(1, 255))),
    ("rmat", dict(scale=12, seed=3, symmetrize=False)),
    ("grid", (1024, 1024, 0.15, 1)),                                # SSSP benchmark graph
    ("grid", (7, 300, 0.5, 9)),
])
def test_oracle_generators_match_product(port, gas_lib, kind, args):
    from vertexapi2_gb300 import graphs
    if kind == "rmat":
        nv, s, d, w = port.gen_rmat(**args)
        g = graphs.rmat(**args)
    else:
        nv, s, d, w = port.gen_grid(*args)
        g = graphs.grid(*args)
    assert nv == g.n_vertices
    assert np.array_equal(s, g.srcs) and np.array_equal(d, g.dsts)
    assert (w is None and g.weights is None) or np.array_equal(w, g.weights)
