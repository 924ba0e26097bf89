"""Synthetic graph generators (R-MAT, lattice) over the C ABI."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import EdgeList, check, load


@dataclass
class Graph:
    n_vertices: int
    srcs: np.ndarray
    dsts: np.ndarray
    weights: np.ndarray | None = None

    @property
    def n_edges(self) -> int:
        return int(self.srcs.shape[0])


def _copy_i32(ptr, m: int) -> np.ndarray:
    if m == 0:
        return np.zeros(0, dtype=np.int32)
    addr = C.cast(ptr, C.c_void_p).value
    return np.frombuffer((C.c_int32 * m).from_address(addr), dtype=np.int32).copy()


def _take(el: EdgeList) -> Graph:
    m = int(el.nEdges)
    srcs = _copy_i32(el.srcs, m)
    dsts = _copy_i32(el.dsts, m)
    w = _copy_i32(el.weights, m) if el.weights else None
    g = Graph(int(el.nVertices), srcs, dsts, w)
    load().gas_edge_list_free(C.byref(el))
    return g


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1, symmetrize: bool = False, weights: tuple[int, int] | None = None) -> Graph:
    el = EdgeList()
    lo, hi = weights if weights else (0, -1)
    check(load().gas_gen_rmat(scale, edge_factor, a, b, c, seed, int(symmetrize), lo, hi,
                              C.byref(el)), "gas_gen_rmat")
    return _take(el)


def grid(rows: int, cols: int, p_delete: float = 0.15, seed: int = 1,
         weights: tuple[int, int] | None = (1, 100)) -> Graph:
    el = EdgeList()
    lo, hi = weights if weights else (0, -1)
    check(load().gas_gen_grid(rows, cols, p_delete, seed, lo, hi, C.byref(el)), "gas_gen_grid")
    return _take(el)
