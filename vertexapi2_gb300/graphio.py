"""Graph files over the C ABI: the reference's loaders and writers
(graphio.cpp), its format converters (mtx2gr.cpp, gr2mtx.cpp) and the
drivers' "vid value" result files.

    python -m vertexapi2_gb300.graphio mtx2gr input.mtx output.gr
    python -m vertexapi2_gb300.graphio gr2mtx input.gr output.mtx
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from ._lib import EdgeList, check, load
from .graphs import Graph, _take


def _i32(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None


def load_graph(path: str, values: bool = False) -> Graph:
    """loadGraph (graphio.cpp:441-473): format from the extension."""
    el = EdgeList()
    check(load().gas_load_graph(str(path).encode(), int(values), C.byref(el)), "gas_load_graph")
    return _take(el)


def write_mtx(path: str, g: Graph) -> None:
    """writeGraph_mtx (graphio.cpp:416-438)."""
    s = np.ascontiguousarray(g.srcs, np.int32)
    d = np.ascontiguousarray(g.dsts, np.int32)
    w = None if g.weights is None else np.ascontiguousarray(g.weights, np.int32)
    check(load().gas_write_graph_mtx(str(path).encode(), g.n_vertices, len(s), _i32(s), _i32(d),
                                     _i32(w)), "gas_write_graph_mtx")


def csr(g: Graph):
    """Offsets, destinations and values in CSR order, stable in edge-list
    order (the engine's CSR)."""
    order = np.argsort(g.srcs, kind="stable")
    off = np.zeros(g.n_vertices + 1, np.int64)
    np.add.at(off, g.srcs.astype(np.int64) + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    w = None if g.weights is None else np.ascontiguousarray(g.weights[order], np.int32)
    return off, np.ascontiguousarray(g.dsts[order], np.int32), w


def write_gr(path: str, g: Graph) -> None:
    """writeGraph_binaryCSR (graphio.cpp:365-413) of the graph's CSR."""
    off, dst, w = csr(g)
    check(load().gas_write_graph_gr(str(path).encode(), g.n_vertices, len(dst), _i32(off),
                                    _i32(dst), _i32(w)), "gas_write_graph_gr")


def write_vertex_values(path: str, values: np.ndarray, field: str | None = None) -> None:
    """The drivers' result file: "vid value" per vertex (bfs.cu:115-119,
    sssp.cu:85-89: "%d %d"; pagerank.cu:77-81: "%d %f").  `values` is an
    int32/float32 array, or a structured vertex-data array with `field`."""
    a = values if field is None else values[field]
    base = values
    if field is None:
        base = np.ascontiguousarray(values)
        a = base
    if a.dtype not in (np.int32, np.float32):
        raise TypeError("values must be int32 or float32")
    stride = base.strides[0] if base.ndim else 4
    offset = base.dtype.fields[field][1] if field is not None else 0
    ptr = C.c_void_p(base.ctypes.data + offset)
    check(load().gas_write_vertex_values(str(path).encode(), len(a), ptr,
                                         int(a.dtype == np.float32), int(stride)),
          "gas_write_vertex_values")


def mtx2gr(src: str, dst: str) -> None:
    """mtx2gr.cpp: load with edge values, write the CSR as .gr."""
    write_gr(dst, load_graph(src, values=True))


def gr2mtx(src: str, dst: str) -> None:
    """gr2mtx.cpp: load a .gr with its values, write MatrixMarket."""
    write_mtx(dst, load_graph(src, values=True))


def main(argv: list[str]) -> int:
    if len(argv) != 3 or argv[0] not in ("mtx2gr", "gr2mtx"):
        print("usage: python -m vertexapi2_gb300.graphio {mtx2gr|gr2mtx} input output")
        return 1
    (mtx2gr if argv[0] == "mtx2gr" else gr2mtx)(argv[1], argv[2])
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
