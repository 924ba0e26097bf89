"""Serving loop: resident graphs, continuous batching over lanes, admission
by free device memory.  Every served result equals the query's
single-source result (BFS / SSSP bit for bit against the oracle, PPR bit
for bit against the oracle's FP32 run and within 1e-5 relative L1 of its
FP64 run), and is the same when the query runs alone and in a mix."""
from __future__ import annotations

import threading

import numpy as np
import pytest

from vertexapi2_gb300 import GASServer, GasError, graphs
from vertexapi2_gb300._lib import (PROGRAM_BFS, PROGRAM_CC, PROGRAM_PPR, PROGRAM_SSSP,
                                   STATUS_NAMES)

pytestmark = pytest.mark.gpu

PPR_REL_L1 = 1e-5  # FP32 vs FP64, relative L1


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


def make_graphs():
    return [graphs.rmat(11, 16, seed=61, symmetrize=True, weights=(1, 255)),
            graphs.grid(40, 30, 0.15, seed=62),
            graphs.rmat(10, 8, seed=63, weights=(1, 100))]  # directed


def oracle_result(port, g, program, source):
    if program == PROGRAM_BFS:
        return port.bfs(g.n_vertices, g.srcs, g.dsts, source)[0]
    if program == PROGRAM_SSSP:
        return port.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, source)[0]
    return port.ppr(g.n_vertices, g.srcs, g.dsts, source, iters=20)[0]


def mix(gs, n, seed):
    rng = np.random.default_rng(seed)
    progs = rng.choice([PROGRAM_BFS, PROGRAM_SSSP, PROGRAM_PPR], size=n, p=[0.5, 0.3, 0.2])
    gids = rng.integers(0, len(gs), n)
    srcs = [int(rng.integers(0, gs[k].n_vertices)) for k in gids]
    return list(zip(gids.tolist(), progs.tolist(), srcs))


def test_mix_matches_oracle_and_alone(gpu, port):
    gs = make_graphs()
    queries = mix(gs, 160, seed=7)
    with GASServer(lanes=4) as srv:
        ids = [srv.add_graph(g.n_vertices, g.srcs, g.dsts, g.weights) for g in gs]
        tickets = [srv.submit(ids[k], p, s) for k, p, s in queries]
        mixed = [srv.wait(t, ids[k], p) for t, (k, p, s) in zip(tickets, queries)]
        st = srv.stats()
        assert st["completed"] == len(queries) and st["failed"] == 0
        assert st["batches"] < len(queries)  # queries were batched
        assert max(info["batchSize"] for _, info in mixed) > 1
        # each query alone (a batch of one)
        alone = []
        for k, p, s in queries[:40]:
            alone.append(srv.wait(srv.submit(ids[k], p, s), ids[k], p))
    for (k, p, s), (res, info) in zip(queries, mixed):
        assert info["status"] == 0
        ref = oracle_result(port, gs[k], p, s)
        assert np.array_equal(res, ref), f"graph {k} program {p} source {s}"
        if p == PROGRAM_PPR:
            ref64 = port.ppr(gs[k].n_vertices, gs[k].srcs, gs[k].dsts, s, iters=20,
                             fp64=True)[0]
            assert rel_l1(res, ref64) <= PPR_REL_L1
    for (k, p, s), (res, info), (res1, info1) in zip(queries, mixed, alone):
        assert info1["batchSize"] == 1
        assert np.array_equal(res, res1), f"alone != mix: graph {k} program {p} source {s}"


def test_large_batches_and_lanes(gpu, port):
    g = graphs.rmat(12, 16, seed=64, symmetrize=True, weights=(1, 255))
    rng = np.random.default_rng(3)
    sources = rng.integers(0, g.n_vertices, 300).astype(np.int32)
    with GASServer(lanes=2, max_batch=128) as srv:
        gid = srv.add_graph(g.n_vertices, g.srcs, g.dsts, g.weights)
        ts = [srv.submit(gid, PROGRAM_SSSP, int(s)) for s in sources]
        out = [srv.wait(t, gid, PROGRAM_SSSP) for t in ts]
        assert max(i["batchSize"] for _, i in out) <= 128
        assert {i["lane"] for _, i in out} <= {0, 1}
    for q in range(0, 300, 37):
        assert np.array_equal(out[q][0], oracle_result(port, g, PROGRAM_SSSP, int(sources[q])))
    for (r, i), s in zip(out, sources):
        assert r[s] == 0 and i["submitNs"] <= i["admitNs"] <= i["doneNs"]


def test_concurrent_clients(gpu, port):
    """Several client threads submit and wait at once."""
    gs = make_graphs()[:2]
    with GASServer(lanes=3) as srv:
        ids = [srv.add_graph(g.n_vertices, g.srcs, g.dsts, g.weights) for g in gs]
        results, errors = {}, []

        def client(c):
            try:
                for k, p, s in mix(gs, 20, seed=100 + c):
                    r, info = srv.wait(srv.submit(ids[k], p, s), ids[k], p)
                    results[(c, k, p, s)] = r
            except Exception as e:  # reported below
                errors.append(e)

        th = [threading.Thread(target=client, args=(c,)) for c in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    assert not errors, errors
    for (c, k, p, s), r in list(results.items())[::5]:
        assert np.array_equal(r, oracle_result(port, gs[k], p, s))


def test_admission_shrinks_batches_under_memory_limit(gpu, port):
    import torch
    g = graphs.rmat(16, 16, seed=65, symmetrize=True, weights=(1, 255))
    V = g.n_vertices
    # device bytes the resident graph takes, measured
    free0 = torch.cuda.mem_get_info(0)[0]
    with GASServer(lanes=1, reserve_bytes=0) as probe:
        probe.add_graph(V, g.srcs, g.dsts, g.weights)
        graph_bytes = free0 - torch.cuda.mem_get_info(0)[0]
    free = torch.cuda.mem_get_info(0)[0]
    # room for the graph and a batch of 32 BFS queries (~20 MB), not 64 (~38 MB)
    batch32 = V * 32 * 4 * 2 + V * 16 + 24 * (V + g.n_edges // 512) + 4 * V
    room = graph_bytes + batch32 + (8 << 20)
    with GASServer(lanes=1, reserve_bytes=max(free - room, 0)) as srv:
        gid = srv.add_graph(V, g.srcs, g.dsts, g.weights)
        rng = np.random.default_rng(5)
        sources = rng.integers(0, V, 100)
        ts = [srv.submit(gid, PROGRAM_BFS, int(s)) for s in sources]
        out = [srv.wait(t, gid, PROGRAM_BFS) for t in ts]
        st = srv.stats()
    assert st["memoryWaits"] > 0
    assert max(i["batchSize"] for _, i in out) < 64
    for q in (0, 57, 99):
        assert np.array_equal(out[q][0], oracle_result(port, g, PROGRAM_BFS, int(sources[q])))


def test_graph_admission_and_errors(gpu):
    import torch
    g = graphs.rmat(9, 8, seed=66, symmetrize=True)  # no weights
    total = torch.cuda.mem_get_info(0)[1]
    with GASServer(reserve_bytes=total) as srv:  # nothing fits
        with pytest.raises(GasError) as ei:
            srv.add_graph(g.n_vertices, g.srcs, g.dsts)
        assert STATUS_NAMES[ei.value.status] == "GAS_ERR_OOM"
    with GASServer() as srv:
        gid = srv.add_graph(g.n_vertices, g.srcs, g.dsts)
        for bad in [(gid + 1, PROGRAM_BFS, 0), (gid, PROGRAM_BFS, g.n_vertices),
                    (gid, PROGRAM_BFS, -1), (gid, PROGRAM_SSSP, 0), (gid, PROGRAM_CC, 0)]:
            with pytest.raises(GasError):
                srv.submit(*bad)
        with pytest.raises(GasError):
            srv.wait(12345, gid, PROGRAM_BFS)
        t = srv.submit(gid, PROGRAM_BFS, 1)
        with pytest.raises(GasError):  # result buffer too small
            srv.wait(t, out=np.empty(3, np.int32))
        r, info = srv.wait(srv.submit(gid, PROGRAM_PPR, 2), gid, PROGRAM_PPR)
        assert info["status"] == 0 and r.dtype == np.float32 and r[2] > 0
    with pytest.raises(GasError):
        GASServer(lanes=0)


def test_ppr_hub_chunks_and_directed_levels(gpu, port):
    """A vertex of in-degree > 4096 (its sum is split into chunks: within
    1e-5 relative L1 of FP64, identical alone and in a mix) and a directed
    chain feeding a cycle (active sets that shrink round by round: bit for
    bit with the FP32 oracle)."""
    rng = np.random.default_rng(9)
    n = 9000
    leaves = np.arange(1, n, dtype=np.int32)
    hub = np.zeros(n - 1, np.int32)
    extra_s = rng.integers(1, n, 20000).astype(np.int32)
    extra_d = rng.integers(1, n, 20000).astype(np.int32)
    keep = extra_s != extra_d
    s = np.concatenate([leaves, hub, extra_s[keep]])
    d = np.concatenate([hub, leaves, extra_d[keep]])
    # directed: 0..29 a chain into a 5-cycle 30..34, plus a tail out of it
    cs = np.array(list(range(29)) + [29, 30, 31, 32, 33, 34, 34], np.int32)
    cd = np.array(list(range(1, 30)) + [30, 31, 32, 33, 34, 30, 35], np.int32)
    with GASServer(lanes=3) as srv:
        gh = srv.add_graph(n, s, d)
        gc = srv.add_graph(36, cs, cd)
        srcs = [0, 1, 4500, 8999]
        ts = [srv.submit(gh, PROGRAM_PPR, x) for x in srcs] + \
             [srv.submit(gc, PROGRAM_PPR, x) for x in (0, 29, 34)]
        mixed = [srv.wait(t, gh if i < 4 else gc, PROGRAM_PPR)[0] for i, t in enumerate(ts)]
        alone = [srv.wait(srv.submit(gh, PROGRAM_PPR, x), gh, PROGRAM_PPR)[0] for x in srcs]
    for x, m, a in zip(srcs, mixed, alone):
        assert np.array_equal(m, a)
        ref64 = port.ppr(n, s, d, x, iters=20, fp64=True)[0]
        assert rel_l1(m, ref64) <= PPR_REL_L1
    for x, m in zip((0, 29, 34), mixed[4:]):
        assert np.array_equal(m, port.ppr(36, cs, cd, x, iters=20)[0]), f"chain source {x}"
