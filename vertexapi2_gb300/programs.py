"""Vertex-data layouts and initial states of the built-in vertex programs.

Each dtype matches the program's VertexData struct in
include/gas_gb300/programs.cuh; the init helpers set vertex data the way the
reference's example drivers do (bfs.cu:143-145, sssp.cu:139-144,
connected_component.cu:110-114, pagerank.cu:120-132 and :82).
"""
from __future__ import annotations

import numpy as np

from ._lib import PROGRAM_BFS, PROGRAM_CC, PROGRAM_PAGERANK, PROGRAM_PPR, PROGRAM_SSSP

SSSP_UNREACHED = 2**31 - 1 - 100000  # sssp.cu:32-33 gatherZero, also the init distance

VERTEX_DTYPES = {
    PROGRAM_BFS: np.dtype(np.int32),
    PROGRAM_SSSP: np.dtype(np.int32),
    PROGRAM_CC: np.dtype(np.int32),
    PROGRAM_PAGERANK: np.dtype([("rank", np.float32), ("numOutEdges", np.int32)]),
    PROGRAM_PPR: np.dtype([("rank", np.float32), ("numOutEdges", np.int32),
                           ("teleport", np.float32)]),
}
EDGE_DTYPES = {PROGRAM_SSSP: np.dtype(np.int32)}
PPR_ALPHA = np.float32(0.15)


def out_degrees(n_vertices: int, srcs: np.ndarray) -> np.ndarray:
    return np.bincount(srcs, minlength=n_vertices).astype(np.int32)


def bfs_init(n_vertices: int) -> np.ndarray:
    return np.full(n_vertices, -1, dtype=np.int32)


def sssp_init(n_vertices: int, source: int) -> np.ndarray:
    d = np.full(n_vertices, SSSP_UNREACHED, dtype=np.int32)
    d[source] = 0
    return d


def cc_init(n_vertices: int) -> np.ndarray:
    return np.arange(n_vertices, dtype=np.int32)


def pagerank_init(n_vertices: int, srcs: np.ndarray) -> np.ndarray:
    vd = np.zeros(n_vertices, dtype=VERTEX_DTYPES[PROGRAM_PAGERANK])
    vd["rank"] = np.float32(0.15)
    vd["numOutEdges"] = out_degrees(n_vertices, srcs)
    return vd


def ppr_init(n_vertices: int, srcs: np.ndarray, source: int) -> np.ndarray:
    vd = np.zeros(n_vertices, dtype=VERTEX_DTYPES[PROGRAM_PPR])
    vd["numOutEdges"] = out_degrees(n_vertices, srcs)
    vd["rank"][source] = 1.0
    vd["teleport"][source] = PPR_ALPHA
    return vd


def max_outdegree_vertex(n_vertices: int, srcs: np.ndarray) -> int:
    """bfs.cu:148-166: first vertex with the strictly largest out-degree."""
    return int(np.argmax(out_degrees(n_vertices, srcs)))
