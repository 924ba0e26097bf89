"""Batched multi-source BFS / SSSP: every query equals its single-source
oracle result bit for bit, across batch sizes, work-unit chunkings (hub
vertices split over many warps) and with or without CUDA-graph replay."""
from __future__ import annotations

import numpy as np
import pytest

from vertexapi2_gb300 import GASBatch, graphs
from vertexapi2_gb300._lib import PROGRAM_BFS, PROGRAM_SSSP

pytestmark = pytest.mark.gpu


def check_queries(port, g, program, sources, got):
    for q, s in enumerate(sources):
        if program == PROGRAM_BFS:
            ref, _ = port.bfs(g.n_vertices, g.srcs, g.dsts, int(s))
        else:
            ref, _ = port.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, int(s))
        assert np.array_equal(got[q], ref), f"query {q} (source {s})"


@pytest.mark.parametrize("nq", [1, 7, 40, 256, 300])
def test_batch_matches_single_source_rmat(gpu, port, nq):
    g = graphs.rmat(12, 16, seed=41, symmetrize=True, weights=(1, 255))
    rng = np.random.default_rng(nq)
    sources = rng.integers(0, g.n_vertices, nq).astype(np.int32)
    with GASBatch() as b:
        b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
        for program in (PROGRAM_BFS, PROGRAM_SSSP):
            got, rounds = b.run(program, sources)
            assert rounds > 0
            check_queries(port, g, program, sources[: min(nq, 64)], got)


@pytest.mark.parametrize("chunk,graphs_on,alpha", [(1, True, 10), (32, False, 0),
                                                   (2048, True, 1 << 20), (128, True, 2)])
def test_batch_configs_directed_and_grid(gpu, port, chunk, graphs_on, alpha):
    for g in (graphs.rmat(11, 16, seed=42, weights=(1, 100)),
              graphs.grid(48, 40, 0.15, seed=43)):
        rng = np.random.default_rng(chunk)
        sources = rng.integers(0, g.n_vertices, 33).astype(np.int32)
        sources[5] = sources[6]  # two queries from the same source
        with GASBatch() as b:
            b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
            b.set_config(chunk, 0, graphs_on)
            b.set_policy(alpha)
            for program in (PROGRAM_BFS, PROGRAM_SSSP):
                got, _ = b.run(program, sources)
                again, _ = b.run(program, sources)  # graph replay / reuse
                assert np.array_equal(got, again)
                check_queries(port, g, program, sources, got)


def test_batch_autotune_and_errors(gpu):
    from vertexapi2_gb300 import GasError
    g = graphs.rmat(10, 8, seed=44, symmetrize=True, weights=(1, 9))
    with GASBatch() as b:
        b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
        chunk, blocks = b.autotune(PROGRAM_SSSP, 64)
        assert chunk in (32, 128, 512, 2048) and blocks in (0, 1, 2, 4)
        with pytest.raises(GasError):
            b.run(PROGRAM_SSSP, np.array([g.n_vertices], np.int32))
        with pytest.raises(GasError):
            b.run(3, np.array([0], np.int32))  # CC is not batched
    with GASBatch() as b:
        b.set_graph(g.n_vertices, g.srcs, g.dsts)  # no weights
        with pytest.raises(GasError):
            b.run(PROGRAM_SSSP, np.array([0], np.int32))


@pytest.mark.parametrize("delta", [1, 16, 100, 5000])
def test_batch_sssp_buckets_match_single_source(gpu, port, delta):
    """Delta-stepping order (distances relaxed a bucket at a time, far pairs
    deferred) gives the same distances as Bellman-Ford rounds."""
    for g in (graphs.grid(40, 36, 0.15, seed=47, weights=(1, 100)),
              graphs.rmat(11, 16, seed=48, symmetrize=True, weights=(1, 255)),
              graphs.rmat(10, 8, seed=49, weights=(1, 9))):
        rng = np.random.default_rng(delta)
        sources = rng.integers(0, g.n_vertices, 70).astype(np.int32)
        with GASBatch() as b:
            b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
            b.set_delta(delta)
            assert b.get_delta() == delta
            got, _ = b.run(PROGRAM_SSSP, sources)
            b.set_delta(0)
            base, _ = b.run(PROGRAM_SSSP, sources)
        assert np.array_equal(got, base)
        check_queries(port, g, PROGRAM_SSSP, sources[::7], got[::7])


@pytest.mark.parametrize("delta", [0, 50])
def test_batch_pair_frontier_matches_masks(gpu, port, delta):
    """(vertex, query) pair frontier (small out-degree graphs) = vertex-mask
    frontier = single-source oracle, for BFS and SSSP."""
    g = graphs.grid(64, 50, 0.15, seed=51, weights=(1, 100))
    rng = np.random.default_rng(52 + delta)
    for nq in (5, 33, 256):
        sources = rng.integers(0, g.n_vertices, nq).astype(np.int32)
        with GASBatch() as b:
            b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
            b.set_delta(delta)
            for program in (PROGRAM_BFS, PROGRAM_SSSP):
                out = []
                for mode in (1, 0):
                    b.set_frontier(mode)
                    got, rounds = b.run(program, sources)
                    out.append(got)
                assert np.array_equal(out[0], out[1])
                check_queries(port, g, program, sources[::11], out[0][::11])


PPR_REL_L1 = 1e-5  # FP32 vs the FP64 oracle, relative L1


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


@pytest.mark.parametrize("nq", [1, 6, 33, 256])
def test_batch_ppr_matches_oracle(gpu, port, nq):
    """Batched personalised PageRank (one persistent launch for all 20
    rounds): every query bit for bit the FP32 oracle's single-source run
    (every in-degree here is <= 4096), within 1e-5 of the FP64 oracle."""
    from vertexapi2_gb300._lib import PROGRAM_PPR
    for g in (graphs.rmat(12, 16, seed=71, symmetrize=True),
              graphs.rmat(10, 8, seed=72),             # directed: dangling vertices
              graphs.grid(40, 30, 0.15, seed=73)):
        rng = np.random.default_rng(nq)
        sources = rng.integers(0, g.n_vertices, nq).astype(np.int32)
        with GASBatch() as b:
            b.set_graph(g.n_vertices, g.srcs, g.dsts)
            got, rounds = b.run(PROGRAM_PPR, sources)
            again, _ = b.run(PROGRAM_PPR, sources)   # graph replay
        assert rounds == 20 and got.dtype == np.float32
        assert np.array_equal(got, again)
        for q in range(0, nq, max(1, nq // 8)):
            ref32, _ = port.ppr(g.n_vertices, g.srcs, g.dsts, int(sources[q]), iters=20)
            ref64, _ = port.ppr(g.n_vertices, g.srcs, g.dsts, int(sources[q]), iters=20, fp64=True)
            assert np.array_equal(got[q], ref32), f"query {q}"
            assert rel_l1(got[q], ref64) <= PPR_REL_L1


def test_batch_ppr_hubs_equal_served(gpu, port):
    """A graph with in-degrees above 4096 (hub vertices summed in 4096-edge
    chunks): batched ranks equal the served queries' bit for bit, and stay
    within 1e-5 of the FP64 oracle."""
    from vertexapi2_gb300 import GASServer
    from vertexapi2_gb300._lib import PROGRAM_PPR
    g = graphs.rmat(16, 16, seed=74, symmetrize=True)
    assert np.bincount(g.dsts).max() > 4096
    sources = np.array([0, 1, 77, 4242, 65535], np.int32)
    with GASBatch() as b:
        b.set_graph(g.n_vertices, g.srcs, g.dsts)
        b.autotune(PROGRAM_PPR, len(sources))
        t = b.tuning()
        assert t["blocks_per_sm"] in (0, 1, 2, 4)
        got, _ = b.run(PROGRAM_PPR, sources)
    with GASServer(lanes=2) as srv:
        gid = srv.add_graph(g.n_vertices, g.srcs, g.dsts)
        for q, s in enumerate(sources):
            res, info = srv.wait(srv.submit(gid, PROGRAM_PPR, int(s)), gid, PROGRAM_PPR)
            assert info["status"] == 0 and np.array_equal(got[q], res)
    ref64, _ = port.ppr(g.n_vertices, g.srcs, g.dsts, int(sources[2]), iters=20, fp64=True)
    assert rel_l1(got[2], ref64) <= PPR_REL_L1


def test_batch_autotune_reports_tuple(gpu):
    """The autotuner searches the frontier form and the push/pull switch as
    well as the work-unit chunk and CTAs per SM; results do not change."""
    g = graphs.rmat(12, 16, seed=75, symmetrize=True, weights=(1, 255))
    rng = np.random.default_rng(76)
    sources = rng.integers(0, g.n_vertices, 40).astype(np.int32)
    with GASBatch() as b:
        b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
        base, _ = b.run(PROGRAM_SSSP, sources)
        b.autotune(PROGRAM_SSSP, 40)
        t = b.tuning()
        assert t["alpha"] in (2, 10, 50) and t["frontier"] in (-1, 0)
        assert t["delta"] in (0, 128, 512, 2048) and t["chunk"] in (32, 128, 512, 2048)
        got, _ = b.run(PROGRAM_SSSP, sources)
        b.set_tuning(t)
        assert b.tuning() == t
    assert np.array_equal(got, base)
