"""Python mirror of vertexAPI2's GASEngineGPU over the C ABI.

Method names and meaning follow gpugas.h:212-772 (setGraph, getResults,
setActive, countActive, gatherApply, scatterActivate, nextIter, run) for
the built-in programs; every call goes through libgas_gb300.so's
gas_engine_* entry points and raises GasError on a non-zero status.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import PROGRAM_PPR, check, load
from .programs import EDGE_DTYPES, VERTEX_DTYPES


def _i32ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class GASEngine:
    def __init__(self, program: int, device: int = 0, stream: int | None = None):
        self.program = program
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.gas_engine_create(program, device, C.c_void_p(stream or 0), C.byref(h)),
              "gas_engine_create")
        self._h = h
        self._keep: list = []
        self.vertex_data: np.ndarray | None = None
        self.edge_data: np.ndarray | None = None

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gas_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # gpugas.h:212-322.  vertex_data / edge_data are borrowed (kept alive
    # here) and written back by get_results, as in the reference.
    def set_graph(self, n_vertices: int, vertex_data: np.ndarray | None, srcs: np.ndarray,
                  dsts: np.ndarray, edge_data: np.ndarray | None = None) -> None:
        srcs = np.ascontiguousarray(srcs, dtype=np.int32)
        dsts = np.ascontiguousarray(dsts, dtype=np.int32)
        if vertex_data is not None:
            want = VERTEX_DTYPES[self.program]
            if vertex_data.dtype != want or not vertex_data.flags.c_contiguous:
                raise TypeError(f"vertex data must be contiguous {want}")
        if edge_data is not None:
            want = EDGE_DTYPES.get(self.program)
            if want is None:
                edge_data = None
            elif edge_data.dtype != want or not edge_data.flags.c_contiguous:
                raise TypeError(f"edge data must be contiguous {want}")
        self.vertex_data, self.edge_data = vertex_data, edge_data
        self._keep = [srcs, dsts]
        vd = vertex_data.ctypes.data_as(C.c_void_p) if vertex_data is not None else None
        ed = edge_data.ctypes.data_as(C.c_void_p) if edge_data is not None else None
        check(self._lib.gas_engine_set_graph(self._h, n_vertices, vd, int(srcs.shape[0]), ed,
                                             _i32ptr(srcs), _i32ptr(dsts)), "gas_engine_set_graph")

    def set_vertex_data(self, host: np.ndarray) -> None:
        check(self._lib.gas_engine_set_vertex_data(self._h, host.ctypes.data_as(C.c_void_p)),
              "gas_engine_set_vertex_data")

    def get_results(self) -> None:
        check(self._lib.gas_engine_get_results(self._h), "gas_engine_get_results")

    def set_active(self, start: int, end: int) -> None:
        check(self._lib.gas_engine_set_active(self._h, start, end), "gas_engine_set_active")

    def count_active(self) -> int:
        n = C.c_int32()
        check(self._lib.gas_engine_count_active(self._h, C.byref(n)), "gas_engine_count_active")
        return n.value

    def gather_apply(self, have_gather: bool = True) -> None:
        check(self._lib.gas_engine_gather_apply(self._h, int(have_gather)), "gas_engine_gather_apply")

    def scatter_activate(self, have_scatter: bool = True) -> None:
        check(self._lib.gas_engine_scatter_activate(self._h, int(have_scatter)),
              "gas_engine_scatter_activate")

    def next_iter(self, wait: bool = True) -> int | None:
        n = C.c_int32()
        check(self._lib.gas_engine_next_iter(self._h, C.byref(n) if wait else None),
              "gas_engine_next_iter")
        return n.value if wait else None

    def run(self, max_iters: int = 0) -> int:
        it = C.c_int32()
        check(self._lib.gas_engine_run(self._h, max_iters, C.byref(it)), "gas_engine_run")
        return it.value

    def set_iteration(self, iteration: int) -> None:
        check(self._lib.gas_engine_set_iteration(self._h, iteration), "gas_engine_set_iteration")

    def round_stats(self, capacity: int = 1 << 16) -> dict[str, np.ndarray]:
        arrs = {k: np.zeros(capacity, dtype=np.int64)
                for k in ("active", "gathered", "ret", "scattered")}
        rounds = C.c_int32()
        p = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
        check(self._lib.gas_engine_round_stats(self._h, capacity, p(arrs["active"]),
                                               p(arrs["gathered"]), p(arrs["ret"]),
                                               p(arrs["scattered"]), C.byref(rounds)),
              "gas_engine_round_stats")
        r = min(rounds.value, capacity)
        return {k: v[:r] for k, v in arrs.items()}

    def save_vertex_data(self) -> None:
        check(self._lib.gas_engine_save_vertex_data(self._h), "gas_engine_save_vertex_data")

    def restore_vertex_data(self) -> None:
        check(self._lib.gas_engine_restore_vertex_data(self._h), "gas_engine_restore_vertex_data")

    def set_launch_config(self, persistent: bool = True, run_blocks_per_sm: int = 0) -> None:
        check(self._lib.gas_engine_set_launch_config(self._h, int(persistent), run_blocks_per_sm),
              "gas_engine_set_launch_config")

    def set_dense_policy(self, alpha: int) -> None:
        check(self._lib.gas_engine_set_dense_policy(self._h, alpha), "gas_engine_set_dense_policy")

    def set_fused_rounds(self, on: bool) -> None:
        check(self._lib.gas_engine_set_fused_rounds(self._h, int(on)), "gas_engine_set_fused_rounds")

    def set_profiling(self, enabled: bool) -> None:
        check(self._lib.gas_engine_set_profiling(self._h, int(enabled)), "gas_engine_set_profiling")

    def kernel_times(self) -> dict:
        g, s = C.c_float(), C.c_float()
        gl, sl = C.c_int32(), C.c_int32()
        check(self._lib.gas_engine_kernel_times(self._h, C.byref(g), C.byref(s), C.byref(gl),
                                                C.byref(sl)), "gas_engine_kernel_times")
        return {"gather_ms": g.value, "scatter_ms": s.value, "gather_launches": gl.value,
                "scatter_launches": sl.value}

    def last_run_ms(self) -> float:
        ms = C.c_float()
        check(self._lib.gas_engine_last_run_ms(self._h, C.byref(ms)), "gas_engine_last_run_ms")
        return float(ms.value)


def device_supported(device: int = 0) -> bool:
    return bool(load().gas_device_supported(device))


class GASBatch:
    """Batched multi-source BFS / SSSP / personalised PageRank on one resident
    graph (gas_batch_*)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.gas_batch_create(device, C.c_void_p(stream or 0), C.byref(h)),
              "gas_batch_create")
        self._h = h
        self.n_vertices = 0

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gas_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_graph(self, n_vertices: int, srcs, dsts, weights=None) -> None:
        s = np.ascontiguousarray(srcs, dtype=np.int32)
        d = np.ascontiguousarray(dsts, dtype=np.int32)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.int32)
        check(self._lib.gas_batch_set_graph(self._h, n_vertices, int(s.shape[0]), _i32ptr(s),
                                            _i32ptr(d), _i32ptr(w) if w is not None else None),
              "gas_batch_set_graph")
        self.n_vertices = n_vertices

    def run(self, program: int, sources, want_results: bool = True):
        """(results[nQueries][nVertices] or None, rounds): int32 depths or
        distances, float32 PPR ranks."""
        src = np.ascontiguousarray(sources, dtype=np.int32)
        out = np.empty((src.shape[0], self.n_vertices), dtype=np.int32) if want_results else None
        rounds = C.c_int32()
        check(self._lib.gas_batch_run(self._h, program, int(src.shape[0]), _i32ptr(src),
                                      _i32ptr(out) if out is not None else None, C.byref(rounds)),
              "gas_batch_run")
        if out is not None and program == PROGRAM_PPR:
            out = out.view(np.float32)
        return out, rounds.value

    def set_config(self, chunk_edges: int = 256, blocks_per_sm: int = 0, use_graphs: bool = True):
        check(self._lib.gas_batch_set_config(self._h, chunk_edges, blocks_per_sm, int(use_graphs)),
              "gas_batch_set_config")

    def set_policy(self, alpha: int) -> None:
        check(self._lib.gas_batch_set_policy(self._h, alpha), "gas_batch_set_policy")

    def set_frontier(self, mode: int) -> None:
        check(self._lib.gas_batch_set_frontier(self._h, mode), "gas_batch_set_frontier")

    def set_delta(self, delta: int) -> None:
        check(self._lib.gas_batch_set_delta(self._h, delta), "gas_batch_set_delta")

    def get_delta(self) -> int:
        d = C.c_int32()
        check(self._lib.gas_batch_get_delta(self._h, C.byref(d)), "gas_batch_get_delta")
        return d.value

    def autotune(self, program: int, n_queries: int) -> tuple[int, int]:
        c, b = C.c_int32(), C.c_int32()
        check(self._lib.gas_batch_autotune(self._h, program, n_queries, C.byref(c), C.byref(b)),
              "gas_batch_autotune")
        return c.value, b.value

    def tuning(self) -> dict:
        """The current settings (after autotune: the chosen ones)."""
        v = [C.c_int32() for _ in range(5)]
        check(self._lib.gas_batch_get_tuning(self._h, *[C.byref(x) for x in v]),
              "gas_batch_get_tuning")
        return dict(zip(("chunk", "blocks_per_sm", "alpha", "frontier", "delta"),
                        (x.value for x in v)))

    def set_tuning(self, t: dict) -> None:
        """Restores settings read with tuning()."""
        self.set_delta(t["delta"])
        self.set_frontier(t["frontier"])
        self.set_policy(t["alpha"])
        self.set_config(t["chunk"], t["blocks_per_sm"], True)

    def last_ms(self) -> float:
        ms = C.c_float()
        check(self._lib.gas_batch_last_ms(self._h, C.byref(ms)), "gas_batch_last_ms")
        return float(ms.value)


class GASServer:
    """Serving loop over resident graphs (gas_server_*): submit BFS / SSSP /
    PPR queries from any thread, wait for their results.

    Results: int32 BFS depth / SSSP distance, float32 PPR rank, one value
    per vertex.
    """

    def __init__(self, device: int = 0, lanes: int = 4, max_batch: int = 256,
                 reserve_bytes: int = 1 << 30):
        from ._lib import ServerConfig
        self._lib = load()
        cfg = ServerConfig(lanes, max_batch, reserve_bytes)
        h = C.c_void_p()
        check(self._lib.gas_server_create(device, C.byref(cfg), C.byref(h)), "gas_server_create")
        self._h = h
        self.n_vertices: dict[int, int] = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gas_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_graph(self, n_vertices: int, srcs, dsts, weights=None) -> int:
        s = np.ascontiguousarray(srcs, dtype=np.int32)
        d = np.ascontiguousarray(dsts, dtype=np.int32)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.int32)
        gid = C.c_int32()
        check(self._lib.gas_server_add_graph(self._h, n_vertices, int(s.shape[0]), _i32ptr(s),
                                             _i32ptr(d), _i32ptr(w) if w is not None else None,
                                             C.byref(gid)), "gas_server_add_graph")
        self.n_vertices[gid.value] = n_vertices
        return gid.value

    def submit(self, graph: int, program: int, source: int) -> int:
        t = C.c_uint64()
        check(self._lib.gas_server_submit(self._h, graph, program, source, C.byref(t)),
              "gas_server_submit")
        return t.value

    def poll(self, ticket: int) -> bool:
        d = C.c_int32()
        check(self._lib.gas_server_poll(self._h, ticket, C.byref(d)), "gas_server_poll")
        return bool(d.value)

    def wait(self, ticket: int, graph: int | None = None, program: int | None = None,
             timeout_ms: int = -1, out: np.ndarray | None = None, want_result: bool = True):
        """Returns (result array or None, info dict).  `out` may be a
        preallocated (pinned) array of the graph's vertex count."""
        from ._lib import PROGRAM_PPR, QueryInfo
        info = QueryInfo()
        res = out
        if res is None and want_result:
            if graph is None or program is None:
                raise ValueError("graph and program are needed to size the result")
            res = np.empty(self.n_vertices[graph],
                           dtype=np.float32 if program == PROGRAM_PPR else np.int32)
        ptr = res.ctypes.data_as(C.c_void_p) if res is not None else None
        nbytes = res.nbytes if res is not None else 0
        check(self._lib.gas_server_wait(self._h, ticket, timeout_ms, ptr, nbytes, C.byref(info)),
              "gas_server_wait")
        d = {f: getattr(info, f) for f, _ in QueryInfo._fields_ if f != "pad"}
        return res, d

    def stats(self) -> dict:
        from ._lib import ServerStats
        st = ServerStats()
        check(self._lib.gas_server_get_stats(self._h, C.byref(st)), "gas_server_get_stats")
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}
