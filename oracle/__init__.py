"""TEST INFRASTRUCTURE ONLY -- Python access to the oracle.

Two interchangeable CPU engines with identical entry points:

* ``port()`` -- the C restatement of the reference's GASEngineRef
  (oracle/gas_oracle.c), built anywhere by oracle/build.py;
* ``ref()``  -- the reference's own refgas.h compiled in place
  (oracle/_ref/libgas_ref.so), only where the reference tree exists.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
SSSP_UNREACHED = 2**31 - 1 - 100000


class OraStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("capacity", C.c_int32),
                ("active", C.POINTER(C.c_int64)), ("edges_gathered", C.POINTER(C.c_int64)),
                ("ret", C.POINTER(C.c_int64)), ("edges_scattered", C.POINTER(C.c_int64)),
                ("run_ns", C.c_int64)]


class OraGraph(C.Structure):
    _fields_ = [("nVertices", C.c_int32), ("nEdges", C.c_int64), ("srcs", C.POINTER(C.c_int32)),
                ("dsts", C.POINTER(C.c_int32)), ("weights", C.POINTER(C.c_int32))]


_PI = C.POINTER(C.c_int32)
_PS = C.POINTER(OraStats)
_SIGS = {
    "run_bfs": [C.c_int32, C.c_int32, _PI, _PI, C.c_int32, _PI, _PS],
    "run_sssp": [C.c_int32, C.c_int32, _PI, _PI, _PI, C.c_int32, _PI, _PS],
    "run_cc": [C.c_int32, C.c_int32, _PI, _PI, _PI, _PS],
    "run_pagerank_f32": [C.c_int32, C.c_int32, _PI, _PI, C.c_int32, C.POINTER(C.c_float), _PS],
    "run_pagerank_f64": [C.c_int32, C.c_int32, _PI, _PI, C.c_int32, C.POINTER(C.c_double), _PS],
    "run_sssp_visits": [C.c_int32, C.c_int32, _PI, _PI, _PI, C.c_int32, _PI, _PI, _PI, _PS],
    "run_ppr_f32": [C.c_int32, C.c_int32, _PI, _PI, C.c_int32, C.c_float, C.c_int32,
                    C.POINTER(C.c_float), _PS],
    "run_ppr_f64": [C.c_int32, C.c_int32, _PI, _PI, C.c_int32, C.c_double, C.c_int32,
                    C.POINTER(C.c_double), _PS],
}


class Engine:
    """One of the two CPU engines; every run returns (result, stats dict)."""

    def __init__(self, path: str, prefix: str):
        self.lib = C.CDLL(path)
        self.prefix = prefix
        self.kind = "port" if prefix == "ora_" else "reference"
        self.path = path
        for name, args in _SIGS.items():
            fn = getattr(self.lib, prefix + name, None)
            if fn is None:
                continue
            fn.restype = C.c_int
            fn.argtypes = args
        if prefix == "ora_":
            self.lib.ora_gen_rmat.restype = C.c_int
            self.lib.ora_gen_rmat.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double,
                                              C.c_double, C.c_uint64, C.c_int32, C.c_int32,
                                              C.c_int32, C.POINTER(OraGraph)]
            self.lib.ora_gen_grid.restype = C.c_int
            self.lib.ora_gen_grid.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_uint64,
                                              C.c_int32, C.c_int32, C.POINTER(OraGraph)]
            self.lib.ora_graph_free.argtypes = [C.POINTER(OraGraph)]
        if prefix == "ref_":
            self.lib.ref_load_graph.restype = C.c_int
            self.lib.ref_load_graph.argtypes = [C.c_char_p, _PI, _PI, C.POINTER(_PI),
                                                C.POINTER(_PI), C.POINTER(_PI)]
            self.lib.ref_free.argtypes = [C.c_void_p]

    def has(self, name: str) -> bool:
        return hasattr(self.lib, self.prefix + name)

    @staticmethod
    def _stats(cap: int):
        arrs = [np.zeros(max(cap, 1), dtype=np.int64) for _ in range(4)]
        st = OraStats()
        st.capacity = cap
        p = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
        st.active, st.edges_gathered, st.ret, st.edges_scattered = (p(a) for a in arrs)
        return st, arrs

    @staticmethod
    def _out(st, arrs):
        n = min(st.iterations, st.capacity)
        keys = ("active", "gathered", "ret", "scattered")
        d = {k: a[:n].copy() for k, a in zip(keys, arrs)}
        d["iterations"] = int(st.iterations)
        d["run_ns"] = int(st.run_ns)
        return d

    def _call(self, name, *args, cap=0):
        st, arrs = self._stats(cap)
        rc = getattr(self.lib, self.prefix + name)(*args, C.byref(st))
        if rc != 0:
            raise ValueError(f"{self.prefix}{name} rejected its arguments")
        return self._out(st, arrs)

    @staticmethod
    def _edges(srcs, dsts):
        s = np.ascontiguousarray(srcs, dtype=np.int32)
        d = np.ascontiguousarray(dsts, dtype=np.int32)
        return s, d, s.ctypes.data_as(_PI), d.ctypes.data_as(_PI)

    def bfs(self, n, srcs, dsts, source, stats_cap=0):
        s, d, ps, pd = self._edges(srcs, dsts)
        out = np.zeros(max(n, 1), dtype=np.int32)
        st = self._call("run_bfs", n, len(s), ps, pd, source, out.ctypes.data_as(_PI), cap=stats_cap)
        return out[:n], st

    def sssp(self, n, srcs, dsts, weights, source, stats_cap=0):
        s, d, ps, pd = self._edges(srcs, dsts)
        w = np.ascontiguousarray(weights, dtype=np.int32)
        out = np.zeros(max(n, 1), dtype=np.int32)
        st = self._call("run_sssp", n, len(s), ps, pd, w.ctypes.data_as(_PI), source,
                        out.ctypes.data_as(_PI), cap=stats_cap)
        return out[:n], st

    def sssp_visits(self, n, srcs, dsts, weights, source, stats_cap=0):
        """SSSP whose Program::scatter counts visits per edge and records the
        source distance: (dist, visits, last), edge arrays in edge order."""
        s, d, ps, pd = self._edges(srcs, dsts)
        w = np.ascontiguousarray(weights, dtype=np.int32)
        dist = np.zeros(max(n, 1), dtype=np.int32)
        vis = np.zeros(max(len(s), 1), dtype=np.int32)
        last = np.zeros(max(len(s), 1), dtype=np.int32)
        p = lambda a: a.ctypes.data_as(_PI)
        st = self._call("run_sssp_visits", n, len(s), ps, pd, p(w), source, p(dist), p(vis), p(last),
                        cap=stats_cap)
        return dist[:n], vis[:len(s)], last[:len(s)], st

    def cc(self, n, srcs, dsts, stats_cap=0):
        s, d, ps, pd = self._edges(srcs, dsts)
        out = np.zeros(max(n, 1), dtype=np.int32)
        st = self._call("run_cc", n, len(s), ps, pd, out.ctypes.data_as(_PI), cap=stats_cap)
        return out[:n], st

    def pagerank(self, n, srcs, dsts, max_iters=0, fp64=False, stats_cap=0):
        s, d, ps, pd = self._edges(srcs, dsts)
        dt, ct = (np.float64, C.c_double) if fp64 else (np.float32, C.c_float)
        out = np.zeros(max(n, 1), dtype=dt)
        st = self._call("run_pagerank_f64" if fp64 else "run_pagerank_f32", n, len(s), ps, pd,
                        max_iters, out.ctypes.data_as(C.POINTER(ct)), cap=stats_cap)
        return out[:n], st

    def ppr(self, n, srcs, dsts, source, alpha=np.float32(0.15), iters=20, fp64=False,
            stats_cap=0):
        s, d, ps, pd = self._edges(srcs, dsts)
        dt, ct = (np.float64, C.c_double) if fp64 else (np.float32, C.c_float)
        out = np.zeros(max(n, 1), dtype=dt)
        a = float(np.float32(alpha))
        st = self._call("run_ppr_f64" if fp64 else "run_ppr_f32", n, len(s), ps, pd, source, a,
                        iters, out.ctypes.data_as(C.POINTER(ct)), cap=stats_cap)
        return out[:n], st

    def _take_graph(self, g: OraGraph):
        m = int(g.nEdges)
        take = lambda p: np.ctypeslib.as_array(p, shape=(max(m, 1),))[:m].copy()
        out = (int(g.nVertices), take(g.srcs), take(g.dsts), take(g.weights) if g.weights else None)
        self.lib.ora_graph_free(C.byref(g))
        return out

    def gen_rmat(self, scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1,
                 symmetrize=False, weights=None):
        """The benchmark's seeded R-MAT graph (restatement only):
        (n_vertices, srcs, dsts, weights or None)."""
        g = OraGraph()
        lo, hi = weights if weights else (0, -1)
        if self.lib.ora_gen_rmat(scale, edge_factor, a, b, c, seed, int(symmetrize), lo, hi,
                                 C.byref(g)) != 0:
            raise ValueError("ora_gen_rmat rejected its arguments")
        return self._take_graph(g)

    def gen_grid(self, rows, cols, p_delete=0.15, seed=1, weights=(1, 100)):
        """The benchmark's seeded lattice (restatement only)."""
        g = OraGraph()
        lo, hi = weights if weights else (0, -1)
        if self.lib.ora_gen_grid(rows, cols, p_delete, seed, lo, hi, C.byref(g)) != 0:
            raise ValueError("ora_gen_grid rejected its arguments")
        return self._take_graph(g)

    def load_graph(self, path: str):
        """graphio.cpp loadGraph (reference engine only)."""
        nv, ne = C.c_int32(), C.c_int32()
        ps, pd, pw = _PI(), _PI(), _PI()
        nw = self.lib.ref_load_graph(path.encode(), C.byref(nv), C.byref(ne), C.byref(ps),
                                     C.byref(pd), C.byref(pw))
        m = ne.value
        take = lambda p, k: np.ctypeslib.as_array(p, shape=(max(k, 1),))[:k].copy()
        s, d = take(ps, m), take(pd, m)
        w = take(pw, nw) if nw > 0 else None
        for p in (ps, pd, pw):
            self.lib.ref_free(C.cast(p, C.c_void_p))
        return nv.value, s, d, w


_port = None
_ref = None


def port() -> Engine:
    global _port
    if _port is None:
        _port = Engine(_build.build_port(), "ora_")
    return _port


def ref() -> Engine | None:
    """The compiled reference engine, or None where it cannot be built."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_ref()
            except Exception:
                path = None
        if not path or not os.path.exists(path):
            return None
        try:
            _ref = Engine(path, "ref_")
        except OSError:  # e.g. a library built for another architecture
            return None
    return _ref
