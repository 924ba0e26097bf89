"""Graph files: the library's loaders read the fixtures in tests/golden/io
exactly as the reference's graphio.cpp does (edge lists recorded by
tests/golden/make_io_golden.py from the reference loader compiled in place),
and the writers round-trip."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GOLDEN

IO = os.path.join(GOLDEN, "io")


def expected():
    with np.load(os.path.join(IO, "expected.npz")) as z:
        return {k: z[k] for k in z.files}


def cases():
    keys = sorted({k.rsplit("|", 2)[0] + "|" + k.rsplit("|", 2)[1] for k in expected()})
    return [(k.split("|")[0], int(k.split("|")[1])) for k in keys]


@pytest.mark.parametrize("name,values", cases())
def test_loader_matches_reference(gas_lib, name, values):
    from vertexapi2_gb300 import graphio
    from vertexapi2_gb300.build import zlib_available
    if name.endswith(".gz") and not zlib_available():
        pytest.skip("library built without zlib")
    exp = expected()
    key = f"{name}|{values}"
    g = graphio.load_graph(os.path.join(IO, name), values=bool(values))
    assert g.n_vertices == int(exp[key + "|nv"][0])
    assert np.array_equal(g.srcs, exp[key + "|s"])
    assert np.array_equal(g.dsts, exp[key + "|d"])
    w = exp[key + "|w"]
    if values and len(w):
        assert g.weights is not None and np.array_equal(g.weights, w)
    else:
        assert g.weights is None


def test_loader_errors(gas_lib, tmp_path):
    from vertexapi2_gb300 import GasError, graphio
    bad = {
        "a.txt": "1 2\n",
        "b.mtx": "%%MatrixMarket matrix array real general\n2 2\n1\n",
        "c.mtx": "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 2 1 1\n",
        "d.mtx": "%%MatrixMarket matrix coordinate real general\n2 2 1\nx y\n",
        "e.mtx": "%%MatrixMarket matrix coordinate real hermitian\n2 2 1\n1 2 3\n",
    }
    for name, body in bad.items():
        p = tmp_path / name
        p.write_text(body)
        with pytest.raises(GasError):
            graphio.load_graph(str(p), values=True)
    with pytest.raises(GasError):
        graphio.load_graph(str(tmp_path / "missing.mtx"))
    short = tmp_path / "short.gr"
    short.write_bytes(b"\x01\x00")
    with pytest.raises(GasError):
        graphio.load_graph(str(short))


def test_missing_value_reads_as_zero(gas_lib, tmp_path):
    """A value line without its value: 0 (the reference reads an
    uninitialised float there)."""
    from vertexapi2_gb300 import graphio
    p = tmp_path / "m.mtx"
    p.write_text("%%MatrixMarket matrix coordinate integer general\n3 3 2\n1 2 7\n2 3\n")
    g = graphio.load_graph(str(p), values=True)
    assert list(g.weights) == [7, 0]


def test_writers_round_trip(gas_lib, tmp_path):
    from vertexapi2_gb300 import graphio, graphs
    g = graphs.rmat(8, 8, seed=5, weights=(1, 50))
    graphio.write_mtx(str(tmp_path / "g.mtx"), g)
    h = graphio.load_graph(str(tmp_path / "g.mtx"), values=True)
    assert np.array_equal(h.srcs, g.srcs) and np.array_equal(h.dsts, g.dsts)
    assert np.array_equal(h.weights, g.weights)
    assert h.n_vertices == int(max(g.srcs.max(), g.dsts.max())) + 1
    # .gr holds the CSR (stable in edge-list order); n_vertices is kept
    graphio.mtx2gr(str(tmp_path / "g.mtx"), str(tmp_path / "g.gr"))
    r = graphio.load_graph(str(tmp_path / "g.gr"), values=True)
    order = np.argsort(h.srcs, kind="stable")
    assert np.array_equal(r.srcs, h.srcs[order]) and np.array_equal(r.dsts, h.dsts[order])
    assert np.array_equal(r.weights, h.weights[order])
    graphio.gr2mtx(str(tmp_path / "g.gr"), str(tmp_path / "back.mtx"))
    b = graphio.load_graph(str(tmp_path / "back.mtx"), values=True)
    assert np.array_equal(b.srcs, r.srcs) and np.array_equal(b.weights, r.weights)


def test_write_vertex_values(gas_lib, tmp_path):
    from vertexapi2_gb300 import graphio
    from vertexapi2_gb300 import programs as P
    depth = np.array([0, 1, -1, 2], np.int32)
    graphio.write_vertex_values(str(tmp_path / "bfs.txt"), depth)
    assert (tmp_path / "bfs.txt").read_text() == "0 0\n1 1\n2 -1\n3 2\n"
    vd = P.pagerank_init(3, np.array([0, 1], np.int32))
    vd["rank"] = [0.15, 0.5, 1.25]
    graphio.write_vertex_values(str(tmp_path / "pr.txt"), vd, field="rank")
    assert (tmp_path / "pr.txt").read_text() == "0 0.150000\n1 0.500000\n2 1.250000\n"
