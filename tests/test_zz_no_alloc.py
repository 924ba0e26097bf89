"""gas_bfs_noalloc: the BFS entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc (device memory already
owned by another allocator, or serving threads that must not take
cudaMalloc's device synchronisation): they pass a CSR graph and the output
array in device memory they already own, and the search uses a fixed
scratch array inside the library.  Its results are checked against the
oracle (the CPU restatement of the reference engine) and against the
allocating entry point, gas_engine_* with the built-in BFS.  This file is
collected last so a failure here leaves every other test already run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vertexapi2_gb300 import GASEngine, graphs
from vertexapi2_gb300 import programs as P
from vertexapi2_gb300._lib import PROGRAM_BFS

pytestmark = pytest.mark.gpu


def engine_bfs(nv, s, d, source):
    """The existing entry point: gas_engine_* with the built-in BFS."""
    vd = P.bfs_init(nv)
    with GASEngine(PROGRAM_BFS) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(source, source + 1)
        rounds = e.run()
        e.get_results()
    return vd, rounds


def device_csr(torch, nv, s, d):
    """CSR of the edge list in device memory: (offsets, destinations)."""
    order = np.argsort(s, kind="stable")
    offs = np.zeros(nv + 1, np.int32)
    offs[1:] = np.cumsum(np.bincount(s, minlength=nv))
    dev = torch.device("cuda:0")
    t_off = torch.from_numpy(offs).to(dev)
    t_dst = torch.from_numpy(np.ascontiguousarray(d[order]).astype(np.int32)).to(dev)
    return t_off, t_dst


def noalloc_bfs(lib, torch, nv, ne, t_off, t_dst, src, t_depth):
    stream = torch.cuda.current_stream(t_depth.device).cuda_stream
    rounds = C.c_int32(-1)
    st = lib.gas_bfs_noalloc(nv, ne, C.c_void_p(t_off.data_ptr()),
                             C.c_void_p(t_dst.data_ptr()) if ne else None, src,
                             C.c_void_p(t_depth.data_ptr()), C.c_void_p(stream),
                             C.byref(rounds))
    assert st == 0, lib.gas_last_error()
    return t_depth.cpu().numpy(), rounds.value


def test_bfs_noalloc_matches_oracle_and_engine_twice(gpu, port):
    torch = pytest.importorskip("torch")
    lib = gpu
    g = graphs.rmat(16, 16, seed=1, symmetrize=True)  # 65,536 vertices: the limit
    nv, s, d = g.n_vertices, g.srcs, g.dsts
    t_off, t_dst = device_csr(torch, nv, s, d)
    t_depth = torch.empty(nv, dtype=torch.int32, device="cuda:0")
    sources = [P.max_outdegree_vertex(nv, s), 12345]
    for src in sources:  # two calls in a row share the scratch array
        got, rounds = noalloc_bfs(lib, torch, nv, len(s), t_off, t_dst, src, t_depth)
        ref, st = port.bfs(nv, s, d, src)
        assert np.array_equal(got, ref)  # integer depths: bit-exact
        assert rounds == st["iterations"]
        want, want_rounds = engine_bfs(nv, s, d, src)
        assert np.array_equal(got, want) and rounds == want_rounds


def test_bfs_noalloc_source_without_out_edges(gpu, port):
    torch = pytest.importorskip("torch")
    lib = gpu
    g = graphs.rmat(12, 16, seed=5)  # directed: some vertices have no out-edges
    nv, s, d = g.n_vertices, g.srcs, g.dsts
    outdeg = np.bincount(s, minlength=nv)
    sink = int(np.flatnonzero(outdeg == 0)[0])
    t_off, t_dst = device_csr(torch, nv, s, d)
    t_depth = torch.empty(nv, dtype=torch.int32, device="cuda:0")
    for src in (sink, int(np.argmax(outdeg))):  # a dead end, then a full search
        got, rounds = noalloc_bfs(lib, torch, nv, len(s), t_off, t_dst, src, t_depth)
        ref, st = port.bfs(nv, s, d, src)
        assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert (got >= 0).sum() > 1


def test_bfs_noalloc_graph_without_edges(gpu, port):
    torch = pytest.importorskip("torch")
    lib = gpu
    nv = 100
    s = d = np.zeros(0, np.int32)
    t_off = torch.zeros(nv + 1, dtype=torch.int32, device="cuda:0")
    t_depth = torch.empty(nv, dtype=torch.int32, device="cuda:0")
    got, rounds = noalloc_bfs(lib, torch, nv, 0, t_off, None, 7, t_depth)
    ref, st = port.bfs(nv, s, d, 7)
    assert np.array_equal(got, ref) and rounds == st["iterations"]
    assert got[7] == 0 and (got == -1).sum() == nv - 1


def test_bfs_noalloc_rejects_oversize(gpu):
    lib = gpu
    too_many = 65536 + 1
    st = lib.gas_bfs_noalloc(too_many, 0, C.c_void_p(16), None, 0, C.c_void_p(16), None, None)
    assert st == 1
    assert b"limit" in lib.gas_last_error()
