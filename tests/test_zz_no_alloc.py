"""gas_bfs_noalloc: the BFS entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc (device memory already
owned by another allocator, or serving threads that must not take
cudaMalloc's device synchronisation): they pass a CSR graph and the output
array in device memory they already own, and the search uses a fixed
scratch array inside the library.  This file is collected last so a failure
here leaves every other test already run.
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


def test_bfs_noalloc_matches_engine_twice(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu
    g = graphs.rmat(16, 16, seed=1, symmetrize=True)  # 65,536 vertices: the limit
    nv, s, d = g.n_vertices, g.srcs, g.dsts
    order = np.argsort(s, kind="stable")
    offs = np.zeros(nv + 1, np.int32)
    offs[1:] = np.cumsum(np.bincount(s, minlength=nv))
    dev = torch.device("cuda:0")
    t_off = torch.from_numpy(offs).to(dev)
    t_dst = torch.from_numpy(np.ascontiguousarray(d[order])).to(dev)
    t_depth = torch.empty(nv, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    sources = [P.max_outdegree_vertex(nv, s), 12345]
    for src in sources:  # two calls in a row share the scratch array
        rounds = C.c_int32(-1)
        st = lib.gas_bfs_noalloc(nv, len(s), C.c_void_p(t_off.data_ptr()),
                                 C.c_void_p(t_dst.data_ptr()), src,
                                 C.c_void_p(t_depth.data_ptr()), C.c_void_p(stream),
                                 C.byref(rounds))
        assert st == 0, lib.gas_last_error()
        got = t_depth.cpu().numpy()
        want, want_rounds = engine_bfs(nv, s, d, src)
        assert np.array_equal(got, want)  # integer depths: bit-exact
        assert rounds.value == want_rounds


def test_bfs_noalloc_rejects_oversize(gpu):
    lib = gpu
    too_many = 65536 + 1
    st = lib.gas_bfs_noalloc(too_many, 0, C.c_void_p(16), None, 0, C.c_void_p(16), None, None)
    assert st == 1
    assert b"limit" in lib.gas_last_error()
