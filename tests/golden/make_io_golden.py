"""Writes the graph-file fixtures in tests/golden/io/ and records what the
reference's own loader (graphio.cpp, compiled in place into
oracle/_ref/libgas_ref.so) reads from each: run here, where the reference
tree exists; the fixtures and the recorded edge lists travel with the
repository.

The fixture contents are this project's own: each exercises one rule of the
reference loaders (comments, blank lines, the MatrixMarket size line and
1-based ids, symmetric / skew-symmetric / hermitian expansion, pattern
files, self-loops with and without values, float values truncated to int,
gzip, SNAP '#' comments, the Lonestar binary layout with odd edge counts,
and a line longer than the 1023-byte read buffer).

    python tests/golden/make_io_golden.py
"""
from __future__ import annotations

import gzip
import os
import struct
import sys

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io")
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

TEXT = {
    "general_int.mtx": (
        "%%MatrixMarket matrix coordinate integer general\n"
        "% a comment\n"
        "\n"
        "6 6 9\n"
        "1 2 5\n"
        "2 3 7.9\n"
        "3 3 4\n"            # self-loop with a value: dropped, not counted
        "   4   1   -2.5\n"
        "\t\n"
        "5 6 100\n"
        "6 5 3\n"
        "1 2 8\n"            # duplicate edge kept
        "6 1 0.4\n"),
    "sym_pattern.mtx": (
        "%%MatrixMarket matrix coordinate pattern symmetric\n"
        "%\n"
        "9 9 5\n"
        "2 1\n"
        "3 1\n"
        "9 9\n"              # self-loop without values: dropped, still counted
        "4 2\n"
        "5 3\n"),
    "skew_real.mtx": (
        "%%MatrixMarket matrix coordinate real skew-symmetric\n"
        "4 4 3\n"
        "2 1 1.5\n"
        "3 2 -2.75\n"
        "4 1 10\n"),
    "hermitian_pattern.mtx": (
        "%%MatrixMarket matrix coordinate pattern hermitian\n"
        "3 3 2\n"
        "2 1\n"
        "3 2\n"),
    "snap.edge": (
        "# SNAP-style edge list\n"
        "# FromNodeId ToNodeId\n"
        "0 1\n"
        "1 2\n"
        "2 2\n"
        "\n"
        "2 0\n"
        "7 3\n"),
    "long_comment.mtx": (
        "%%MatrixMarket matrix coordinate integer general\n"
        "%" + "x" * 1022 + " 7 8 2\n"   # the tail past 1023 bytes reads as a data line
        "8 8 2\n"
        "1 2 3\n"),
}
GZ = {
    "sym_real.mtx.gz": (
        "%%MatrixMarket matrix coordinate real symmetric\n"
        "5 5 4\n"
        "2 1 0.5\n"
        "3 1 2.5\n"
        "5 4 -1.5\n"
        "4 4 9\n"),
}


def write_gr(path, n, offsets_end, dsts, values, width=4):
    with open(path, "wb") as f:
        f.write(struct.pack("<4Q", 1, width, n, len(dsts)))
        f.write(struct.pack(f"<{n}Q", *offsets_end))
        f.write(struct.pack(f"<{len(dsts)}I", *dsts))
        if len(dsts) % 2:
            f.write(struct.pack("<I", 0))
        if values is not None:
            f.write(struct.pack(f"<{len(values)}i", *values))


def main() -> None:
    os.makedirs(HERE, exist_ok=True)
    for name, body in TEXT.items():
        with open(os.path.join(HERE, name), "w") as f:
            f.write(body)
    for name, body in GZ.items():
        with gzip.open(os.path.join(HERE, name), "wt") as f:
            f.write(body)
    # 5 vertices, 7 edges (odd: padded), values
    write_gr(os.path.join(HERE, "csr_vals.gr"), 5, [2, 2, 5, 6, 7],
             [1, 4, 0, 2, 3, 4, 1], [3, -1, 7, 8, 9, 10, 11])
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("the reference engine (oracle/_ref) is not built")
    out = {}
    names = sorted(list(TEXT) + list(GZ) + ["csr_vals.gr"])
    for name in names:
        for values in (0, 1):
            if name == "hermitian_pattern.mtx" and values:
                continue
            nv, s, d, w = ref.load_graph(os.path.join(HERE, name)) if values else \
                ref_load_no_values(ref, os.path.join(HERE, name))
            key = f"{name}|{values}"
            out[key + "|nv"] = np.array([nv], np.int32)
            out[key + "|s"] = s.astype(np.int32)
            out[key + "|d"] = d.astype(np.int32)
            out[key + "|w"] = (w if w is not None else np.zeros(0)).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "expected.npz"), **out)
    print(f"{len(names)} fixtures, {len(out) // 4} loads recorded")


def ref_load_no_values(ref, path):
    """loadGraph without an edge-value vector (the drivers' BFS/CC call)."""
    import ctypes as C
    nv, ne = C.c_int32(), C.c_int32()
    PI = C.POINTER(C.c_int32)
    ps, pd = PI(), PI()
    ref.lib.ref_load_graph(path.encode(), C.byref(nv), C.byref(ne), C.byref(ps), C.byref(pd),
                           None)
    m = ne.value
    take = lambda p: np.ctypeslib.as_array(p, shape=(max(m, 1),))[:m].copy()
    s, d = take(ps), take(pd)
    for p in (ps, pd):
        ref.lib.ref_free(C.cast(p, C.c_void_p))
    return nv.value, s, d, None


if __name__ == "__main__":
    main()
