"""GPU parity: the CUDA engine (through the C ABI) against the oracle.

Bars: BFS depths, SSSP distances and CC labels bit-exact; FP32 PageRank
within 1e-5 relative L1 of the FP64 oracle (and close to the FP32 oracle);
per-round frontier counts equal to the oracle's.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden

import oracle
from vertexapi2_gb300 import GASEngine, graphs
from vertexapi2_gb300 import programs as P
from vertexapi2_gb300._lib import (PROGRAM_BFS, PROGRAM_CC, PROGRAM_PAGERANK, PROGRAM_PPR,
                                   PROGRAM_SSSP)

pytestmark = pytest.mark.gpu

PR_REL_L1 = 1e-5      # FP32 PageRank vs FP64 oracle (relative L1)


def rel_l1(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


def gpu_bfs(nv, s, d, source, stepwise=False):
    vd = P.bfs_init(nv)
    with GASEngine(PROGRAM_BFS) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(source, source + 1)
        if stepwise:  # the reference driver loop, bfs.cu:98-108
            it = 0
            e.set_iteration(it)
            while e.count_active():
                e.gather_apply(False)
                e.scatter_activate(False)
                e.next_iter()
                it += 1
                e.set_iteration(it)
            rounds = it
        else:
            rounds = e.run()
        stats = e.round_stats()
        e.get_results()
    return vd, rounds, stats


def gpu_sssp(nv, s, d, w, source, stepwise=False):
    vd = P.sssp_init(nv, source)
    ed = np.ascontiguousarray(w, dtype=np.int32)
    with GASEngine(PROGRAM_SSSP) as e:
        e.set_graph(nv, vd, s, d, ed)
        e.set_active(0, nv)
        if stepwise:
            rounds = 0
            while e.count_active():
                e.gather_apply()
                e.scatter_activate()
                e.next_iter()
                rounds += 1
        else:
            rounds = e.run()
        stats = e.round_stats()
        e.get_results()
        assert np.array_equal(ed, w)  # edge data comes back in caller order
    return vd, rounds, stats


def gpu_cc(nv, s, d):
    vd = P.cc_init(nv)
    with GASEngine(PROGRAM_CC) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(0, nv)
        rounds = e.run()
        stats = e.round_stats()
        e.get_results()
    return vd, rounds, stats


def gpu_pagerank(nv, s, d, max_iters=0):
    vd = P.pagerank_init(nv, s)
    with GASEngine(PROGRAM_PAGERANK) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(0, nv)
        rounds = e.run(max_iters)
        stats = e.round_stats()
        e.get_results()
    return vd["rank"].copy(), rounds, stats


def gpu_ppr(nv, s, d, source, iters=20):
    vd = P.ppr_init(nv, s, source)
    with GASEngine(PROGRAM_PPR) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(0, nv)
        rounds = e.run(iters)
        e.get_results()
    return vd["rank"].copy(), rounds


@pytest.mark.parametrize("name", golden_names())
def test_matches_golden(gpu, name):
    g = load_golden(name)
    nv, s, d = int(g["n_vertices"]), g["srcs"], g["dsts"]
    src = int(g["bfs_source"])
    depth, rounds, st = gpu_bfs(nv, s, d, src)
    assert np.array_equal(depth, g["bfs"])
    assert np.array_equal(st["active"], g["bfs_active"])
    lab, _, st = gpu_cc(nv, s, d)
    assert np.array_equal(lab, g["cc"])
    assert np.array_equal(st["active"], g["cc_active"])
    assert np.array_equal(st["gathered"], g["cc_gathered"])
    assert np.array_equal(st["scattered"], g["cc_scattered"])
    if "weights" in g:
        dist, _, _ = gpu_sssp(nv, s, d, g["weights"], 0)
        assert np.array_equal(dist, g["sssp"])
    pr, rounds, _ = gpu_pagerank(nv, s, d)
    assert rel_l1(pr, g["pr64"]) <= PR_REL_L1
    assert np.allclose(pr, g["pr32"], rtol=2e-5, atol=2e-6)
    ppr, _ = gpu_ppr(nv, s, d, src)
    assert rel_l1(ppr, g["ppr64"]) <= PR_REL_L1


def test_stepwise_api_matches_run(gpu, port):
    g = graphs.rmat(12, 16, seed=21, symmetrize=True, weights=(1, 255))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    src = P.max_outdegree_vertex(nv, s)
    a, ra, _ = gpu_bfs(nv, s, d, src, stepwise=True)
    b, rb, _ = gpu_bfs(nv, s, d, src)
    ref, st = port.bfs(nv, s, d, src)
    assert np.array_equal(a, ref) and np.array_equal(b, ref)
    assert ra == rb == st["iterations"]
    a, ra, _ = gpu_sssp(nv, s, d, w, 0, stepwise=True)
    ref, st = port.sssp(nv, s, d, w, 0)
    assert np.array_equal(a, ref) and ra == st["iterations"]


@pytest.mark.parametrize("seed", [1, 2])
def test_medium_graphs_vs_oracle(gpu, port, seed):
    gs = graphs.rmat(15, 16, seed=seed, symmetrize=True, weights=(1, 255))
    nv, s, d, w = gs.n_vertices, gs.srcs, gs.dsts, gs.weights
    src = P.max_outdegree_vertex(nv, s)
    ref, st = port.bfs(nv, s, d, src, stats_cap=256)
    got, rounds, gst = gpu_bfs(nv, s, d, src)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert np.array_equal(gst["active"], st["active"])
    assert np.array_equal(gst["scattered"], st["scattered"])
    ref, st = port.sssp(nv, s, d, w, 0, stats_cap=4096)
    got, rounds, gst = gpu_sssp(nv, s, d, w, 0)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert np.array_equal(gst["active"], st["active"])
    assert np.array_equal(gst["gathered"], st["gathered"])
    ref, _ = port.cc(nv, s, d)
    got, _, _ = gpu_cc(nv, s, d)
    assert np.array_equal(got, ref)
    gd = graphs.rmat(15, 16, seed=seed + 100)
    ref64, _ = port.pagerank(gd.n_vertices, gd.srcs, gd.dsts, max_iters=50, fp64=True)
    got, rounds, _ = gpu_pagerank(gd.n_vertices, gd.srcs, gd.dsts, max_iters=50)
    assert rounds == 50 or rounds <= 50
    assert rel_l1(got, ref64) <= PR_REL_L1


def test_grid_sssp_vs_oracle(gpu, port):
    g = graphs.grid(160, 120, 0.15, seed=7)
    ref, st = port.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, 0, stats_cap=8192)
    got, rounds, gst = gpu_sssp(g.n_vertices, g.srcs, g.dsts, g.weights, 0)
    assert np.array_equal(got, ref)
    assert rounds == st["iterations"]
    assert np.array_equal(gst["active"], st["active"])


def test_hub_vertices_span_many_tiles(gpu, port):
    # vertex 0 has 300k in-edges (about 150 gather tiles): its reduction
    # crosses tiles through the look-back; vertex 1 has 5k, others few.
    rng = np.random.default_rng(5)
    nv = 400_000
    hub = np.arange(1, 300_001, dtype=np.int32)
    s = np.concatenate([hub, np.arange(2, 5002, dtype=np.int32),
                        rng.integers(0, nv, 200_000, dtype=np.int32)])
    d = np.concatenate([np.zeros(300_000, np.int32), np.ones(5000, np.int32),
                        rng.integers(0, nv, 200_000, dtype=np.int32)])
    keep = s != d
    s, d = s[keep], d[keep]
    w = rng.integers(1, 100, s.shape[0], dtype=np.int32)
    ref, _ = port.cc(nv, s, d)
    got, _, _ = gpu_cc(nv, s, d)
    assert np.array_equal(got, ref)
    ref, _ = port.sssp(nv, s, d, w, 3)
    got, _, _ = gpu_sssp(nv, s, d, w, 3)
    assert np.array_equal(got, ref)
    ref64, _ = port.pagerank(nv, s, d, max_iters=30, fp64=True)
    got, _, _ = gpu_pagerank(nv, s, d, max_iters=30)
    assert rel_l1(got, ref64) <= PR_REL_L1
    assert abs(got[0] - ref64[0]) / ref64[0] < 1e-5


def test_edge_cases(gpu, port):
    # no edges at all
    z = np.zeros(0, np.int32)
    depth, rounds, _ = gpu_bfs(5, z, z, 3)
    assert depth.tolist() == [-1, -1, -1, 0, -1] and rounds == 1
    lab, rounds, _ = gpu_cc(5, z, z)
    assert lab.tolist() == list(range(5)) and rounds == 1
    # single vertex
    depth, _, _ = gpu_bfs(1, z, z, 0)
    assert depth.tolist() == [0]
    # empty active range: run() does nothing
    vd = P.cc_init(4)
    with GASEngine(PROGRAM_CC) as e:
        e.set_graph(4, vd, np.array([0, 1], np.int32), np.array([1, 2], np.int32))
        e.set_active(2, 2)
        assert e.count_active() == 0
        assert e.run() == 0
        e.get_results()
    assert vd.tolist() == [0, 1, 2, 3]
    # duplicate edges and self-loops (the engine does not dedup, like the
    # reference's setGraph)
    s = np.array([0, 0, 1, 1, 2, 2, 3, 3, 3], np.int32)
    d = np.array([1, 1, 1, 2, 0, 3, 3, 0, 0], np.int32)
    w = np.array([5, 3, 1, 2, 9, 1, 4, 2, 7], np.int32)
    for src in range(4):
        ref, _ = port.sssp(4, s, d, w, src)
        got, _, _ = gpu_sssp(4, s, d, w, src)
        assert np.array_equal(got, ref)
    ref64, _ = port.pagerank(4, s, d, fp64=True)
    got, _, _ = gpu_pagerank(4, s, d)
    assert rel_l1(got, ref64) <= PR_REL_L1
    # active subrange and a vertex with no in-edges
    s = np.array([1, 2, 3], np.int32)
    d = np.array([2, 3, 4], np.int32)
    vd = P.cc_init(6)
    with GASEngine(PROGRAM_CC) as e:
        e.set_graph(6, vd, s, d)
        e.set_active(1, 5)
        e.run()
        e.get_results()
    assert vd.tolist() == [0, 1, 1, 1, 1, 5]


def test_invalid_arguments_are_rejected(gpu):
    from vertexapi2_gb300 import GasError
    vd = P.cc_init(3)
    with GASEngine(PROGRAM_CC) as e:
        with pytest.raises(GasError):
            e.set_graph(3, vd, np.array([0, 7], np.int32), np.array([1, 2], np.int32))
        with pytest.raises(GasError):
            e.set_active(0, 1)  # no graph
        e.set_graph(3, vd, np.array([0], np.int32), np.array([1], np.int32))
        with pytest.raises(GasError):
            e.set_active(2, 9)
        with pytest.raises(GasError):
            e.scatter_activate()  # no gather yet


def test_c1_bfs_rmat16_full_size(gpu, port):
    g = graphs.rmat(16, 16, seed=1, symmetrize=True)
    src = P.max_outdegree_vertex(g.n_vertices, g.srcs)
    ref, st = port.bfs(g.n_vertices, g.srcs, g.dsts, src, stats_cap=64)
    got, rounds, gst = gpu_bfs(g.n_vertices, g.srcs, g.dsts, src)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert np.array_equal(gst["active"], st["active"])


def test_c2_sssp_grid_full_size(gpu, port):
    g = graphs.grid(1024, 1024, 0.15, seed=1)
    ref, st = port.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, 0, stats_cap=8192)
    got, rounds, gst = gpu_sssp(g.n_vertices, g.srcs, g.dsts, g.weights, 0)
    assert np.array_equal(got, ref)
    assert rounds == st["iterations"]
    assert np.array_equal(gst["active"], st["active"])
    assert np.array_equal(gst["gathered"], st["gathered"])


def _run_policy(program, nv, s, d, init, w=None, active=None, alpha=10, max_iters=0):
    vd = init.copy()
    with GASEngine(program) as e:
        e.set_graph(nv, vd, s, d, w)
        e.set_dense_policy(alpha)
        lo, hi = active if active else (0, nv)
        e.set_active(lo, hi)
        rounds = e.run(max_iters)
        st = e.round_stats()
        e.get_results()
    return vd, rounds, st


@pytest.mark.parametrize("alpha", [0, 1, 10, 1000])
def test_dense_policy_does_not_change_results(gpu, port, alpha):
    """Dense (pull) rounds, list (push) rounds and every mix of the two give
    identical results and identical per-round frontier counts.  alpha = 1
    keeps most rounds in list mode, so list rounds whose frontiers hold more
    than E/4 in-edges run as pull passes over the marked vertices."""
    g = graphs.rmat(14, 16, seed=31, symmetrize=True, weights=(1, 255))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    src = P.max_outdegree_vertex(nv, s)
    ref, st = port.bfs(nv, s, d, src, stats_cap=256)
    got, rounds, gst = _run_policy(PROGRAM_BFS, nv, s, d, P.bfs_init(nv), active=(src, src + 1),
                                   alpha=alpha)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    for k in ("active", "gathered", "ret", "scattered"):
        assert np.array_equal(gst[k], st[k]), k
    ref, st = port.cc(nv, s, d, stats_cap=256)
    got, rounds, gst = _run_policy(PROGRAM_CC, nv, s, d, P.cc_init(nv), alpha=alpha)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert np.array_equal(gst["active"], st["active"])
    ref, st = port.sssp(nv, s, d, w, 0, stats_cap=4096)
    got, rounds, gst = _run_policy(PROGRAM_SSSP, nv, s, d, P.sssp_init(nv, 0), w=w, alpha=alpha)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert np.array_equal(gst["gathered"], st["gathered"])
    gd = graphs.rmat(14, 16, seed=32)
    ref64, st = port.pagerank(gd.n_vertices, gd.srcs, gd.dsts, max_iters=50, fp64=True)
    got, rounds, _ = _run_policy(PROGRAM_PAGERANK, gd.n_vertices, gd.srcs, gd.dsts,
                                 P.pagerank_init(gd.n_vertices, gd.srcs), alpha=alpha,
                                 max_iters=50)
    assert rel_l1(got["rank"], ref64) <= PR_REL_L1


def test_dense_rounds_are_deterministic(gpu):
    """With every round dense the FP32 PageRank is bit-identical run to run."""
    gd = graphs.rmat(15, 16, seed=33)
    runs = [_run_policy(PROGRAM_PAGERANK, gd.n_vertices, gd.srcs, gd.dsts,
                        P.pagerank_init(gd.n_vertices, gd.srcs), alpha=1 << 20, max_iters=30)[0]
            for _ in range(2)]
    assert np.array_equal(runs[0]["rank"], runs[1]["rank"])


@pytest.mark.parametrize("nv,ne,seed", [(1, 0, 1), (7, 50, 2), (300, 5000, 3), (70000, 400000, 4)])
def test_device_graph_build_order(gpu, port, nv, ne, seed):
    """setGraph builds CSC/CSR on the device with radix sorts (one to three
    8-bit passes here); in-edges keep edge-list order among equal
    destinations, duplicates included: SSSP distances equal the oracle's and
    edge data comes back in the caller's order."""
    rng = np.random.default_rng(seed)
    s = rng.integers(0, nv, ne).astype(np.int32)
    d = rng.integers(0, nv, ne).astype(np.int32)
    if ne:
        s[: ne // 10] = s[0]  # a hub with duplicate edges
    w = rng.integers(1, 1000, ne).astype(np.int32)
    vd = P.sssp_init(nv, 0)
    with GASEngine(PROGRAM_SSSP) as e:
        ed = w.copy()
        e.set_graph(nv, vd, s, d, ed)
        e.set_active(0, nv)
        e.run()
        e.get_results()
    assert np.array_equal(ed, w)
    assert np.array_equal(vd, port.sssp(nv, s, d, w, 0)[0])


def test_bounded_waits_report_timeouts_and_device_recovers(gpu, port):
    """A grid barrier and a look-back wait whose partners never arrive give
    up at their spin limits with GAS_ERR_TIMEOUT; the next run is normal."""
    import ctypes as C
    b, l, t = C.c_int32(), C.c_int32(), C.c_float()
    assert gpu.gas_selftest_bounded_waits(0, C.byref(b), C.byref(l), C.byref(t)) == 0
    assert b.value == 4 and l.value == 4  # GAS_ERR_TIMEOUT
    assert 0.0 < t.value < 60.0
    g = graphs.rmat(8, 8, seed=9, symmetrize=True)
    depth, _, _ = gpu_bfs(g.n_vertices, g.srcs, g.dsts, 0)
    assert np.array_equal(depth, port.bfs(g.n_vertices, g.srcs, g.dsts, 0)[0])


@pytest.mark.parametrize("program", [PROGRAM_SSSP, PROGRAM_BFS, PROGRAM_CC, PROGRAM_PAGERANK])
def test_fused_rounds_match_two_phase_rounds(gpu, port, program):
    """One-phase rounds with versioned vertex data (every degree <= 8) give
    the two-phase rounds' results and per-round counts exactly."""
    g = graphs.grid(70, 60, 0.15, seed=91, weights=(1, 100))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    out = []
    for fused in (True, False):
        if program == PROGRAM_SSSP:
            vd, act, ed, iters = P.sssp_init(nv, 0), (0, nv), w, 0
        elif program == PROGRAM_BFS:
            vd, act, ed, iters = P.bfs_init(nv), (5, 6), None, 0
        elif program == PROGRAM_CC:
            vd, act, ed, iters = P.cc_init(nv), (0, nv), None, 0
        else:
            vd, act, ed, iters = P.pagerank_init(nv, s), (0, nv), None, 50
        with GASEngine(program) as e:
            e.set_graph(nv, vd, s, d, ed)
            e.set_fused_rounds(fused)
            e.set_active(*act)
            rounds = e.run(iters)
            stats = e.round_stats()
            e.get_results()
        out.append((vd.copy(), rounds, stats))
    (a, ra, sa), (b, rb, sb) = out
    assert ra == rb
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    if program == PROGRAM_PAGERANK:
        assert np.array_equal(a["rank"], b["rank"])
    else:
        assert np.array_equal(a, b)
    if program == PROGRAM_SSSP:
        assert np.array_equal(a, port.sssp(nv, s, d, w, 0)[0])
    if program == PROGRAM_BFS:
        assert np.array_equal(a, port.bfs(nv, s, d, 5)[0])


@pytest.mark.parametrize("program", [PROGRAM_CC, PROGRAM_SSSP, PROGRAM_PAGERANK])
def test_dense_kernel_handover_at_every_round(gpu, program):
    """A run that starts with every vertex active runs its leading dense
    rounds in run_dense_kernel and resumes in the main kernel.  run(k) for
    every k up to the end equals k rounds of the stepwise API (one launch per
    phase, no dense rounds): the hand-over is right whether the dense kernel
    stops at maxIters, at a dense -> list transition or at the end."""
    g = graphs.rmat(13, 16, seed=41, symmetrize=program != PROGRAM_PAGERANK, weights=(1, 255))
    nv, s, d = g.n_vertices, g.srcs, g.dsts
    w = g.weights if program == PROGRAM_SSSP else None
    if program == PROGRAM_CC:
        init = P.cc_init(nv)
    elif program == PROGRAM_SSSP:
        init = P.sssp_init(nv, 0)
    else:
        init = P.pagerank_init(nv, s)
    _, total, _ = _run_policy(program, nv, s, d, init, w=w, max_iters=12)
    for k in range(1, total + 1):
        vd = init.copy()
        with GASEngine(program) as e:
            e.set_graph(nv, vd, s, d, w)
            e.set_active(0, nv)
            for _ in range(k):
                if not e.count_active():
                    break
                e.gather_apply()
                e.scatter_activate()
                e.next_iter()
            e.get_results()
        got, rounds, _ = _run_policy(program, nv, s, d, init, w=w, max_iters=k)
        assert rounds == k
        if program == PROGRAM_PAGERANK:
            assert rel_l1(got["rank"], vd["rank"]) <= PR_REL_L1, k
        else:
            assert np.array_equal(got, vd), k


@pytest.mark.parametrize("k", [1, 2, 3])
def test_run_resumes_across_calls(gpu, port, k):
    """run(k) called repeatedly continues where the last call stopped --
    also when a call stops before a dense round, whose frontier exists only
    as round stamps until the next call turns it into a list (k = 1 stops
    before every dense round).  The dense-rounds kernel only leads a run
    that starts with every vertex active."""
    g = graphs.rmat(13, 16, seed=43, symmetrize=True, weights=(1, 255))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    for program in (PROGRAM_SSSP, PROGRAM_CC):
        if program == PROGRAM_SSSP:
            ref, st = port.sssp(nv, s, d, w, 0)
            vd, ed = P.sssp_init(nv, 0), w
        else:
            ref, st = port.cc(nv, s, d)
            vd, ed = P.cc_init(nv), None
        with GASEngine(program) as e:
            e.set_graph(nv, vd, s, d, ed)
            e.set_active(0, nv)
            done = 0
            while True:
                r = e.run(k)
                done += r
                if r < k:
                    break
            e.get_results()
        assert np.array_equal(vd, ref) and done == st["iterations"], program


def test_stepwise_after_run_stopped_before_dense_round(gpu, port):
    """The stepwise API picks up a frontier a run left as round stamps."""
    g = graphs.rmat(13, 16, seed=44, symmetrize=True, weights=(1, 255))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    ref, st = port.sssp(nv, s, d, w, 0)
    for k in range(1, st["iterations"]):
        vd = P.sssp_init(nv, 0)
        with GASEngine(PROGRAM_SSSP) as e:
            e.set_graph(nv, vd, s, d, w)
            e.set_active(0, nv)
            done = e.run(k)
            while e.count_active():
                e.gather_apply()
                e.scatter_activate()
                e.next_iter()
                done += 1
            e.get_results()
        assert np.array_equal(vd, ref) and done == st["iterations"], k


@pytest.mark.parametrize("alpha", [0, 10, 5000])
def test_fused_bitmap_rounds_match_oracle(gpu, port, alpha):
    """Lattices run fused rounds whose frontier is a bitmap.  Results and
    per-round counts equal the oracle's for SSSP (every vertex active at the
    start: a dense first round, then fused rounds) and BFS (a one-vertex
    range, then fused rounds); alpha = 5000 turns many fused rounds' successors
    into dense rounds that take their active set from the fused round's
    bitmap."""
    g = graphs.grid(70, 55, 0.15, seed=95, weights=(1, 100))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    ref, st = port.sssp(nv, s, d, w, 0, stats_cap=4096)
    got, rounds, gst = _run_policy(PROGRAM_SSSP, nv, s, d, P.sssp_init(nv, 0), w=w, alpha=alpha)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    for k in ("active", "gathered", "ret", "scattered"):
        assert np.array_equal(gst[k][:rounds], st[k]), k
    ref, st = port.bfs(nv, s, d, 5, stats_cap=4096)
    got, rounds, gst = _run_policy(PROGRAM_BFS, nv, s, d, P.bfs_init(nv), active=(5, 6), alpha=alpha)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    for k in ("active", "gathered", "ret", "scattered"):
        assert np.array_equal(gst[k][:rounds], st[k]), k


@pytest.mark.parametrize("k", [1, 2, 5])
def test_fused_run_resumes_across_calls(gpu, port, k):
    """run(k) on a lattice stops with the next frontier in a bitmap; the run
    turns it into a list before it returns, and the next call (or the
    stepwise API) continues from that list."""
    g = graphs.grid(40, 37, 0.15, seed=96, weights=(1, 100))
    nv, s, d, w = g.n_vertices, g.srcs, g.dsts, g.weights
    ref, st = port.sssp(nv, s, d, w, 0)
    for alpha in (10, 5000):
        vd = P.sssp_init(nv, 0)
        with GASEngine(PROGRAM_SSSP) as e:
            e.set_graph(nv, vd, s, d, w)
            e.set_dense_policy(alpha)
            e.set_active(0, nv)
            done = 0
            while True:
                r = e.run(k)
                done += r
                if r < k:
                    break
            e.get_results()
        assert np.array_equal(vd, ref) and done == st["iterations"], alpha
    ref, st = port.bfs(nv, s, d, 0)
    vd = P.bfs_init(nv)
    with GASEngine(PROGRAM_BFS) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(0, 1)
        done = e.run(k + 3)
        e.set_iteration(done)
        while e.count_active():  # stepwise from the list the capped run left
            e.gather_apply(False)
            e.scatter_activate(False)
            e.next_iter()
            done += 1
            e.set_iteration(done)  # the driver sets the round, as bfs.cu:98-108 does
        e.get_results()
    assert np.array_equal(vd, ref) and done == st["iterations"]
