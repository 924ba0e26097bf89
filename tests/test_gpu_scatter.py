"""Program::scatter through the C++ engine template: a user Program that
opts in (scatterEdges) gets scatter(src, dst, edge) on every out-edge of
each round's apply-returned-true vertices, as the reference's CPU engine
calls it (refgas.h:171-197); distances, per-edge visit counts and the
recorded source distances equal the oracle's, stepwise and in run()."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
EXE = os.path.join(HERE, "cpp", "_build", "edge_scatter")


@pytest.fixture(scope="module")
def driver(gpu):
    src = os.path.join(HERE, "cpp", "edge_scatter.cu")
    lib = os.path.join(ROOT, "vertexapi2_gb300", "_build")
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(src):
        cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
               "-I", os.path.join(ROOT, "include"), src, "-L", lib, "-lgas_gb300",
               "-Xlinker", f"-rpath={lib}", "-o", EXE]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
    return EXE


def run_driver(exe, tmp_path, g, source, mode):
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    head = np.array([g.n_vertices, g.n_edges, source, mode], np.int32)
    with open(inp, "wb") as f:
        for a in (head, g.srcs, g.dsts, g.weights):
            f.write(np.ascontiguousarray(a, np.int32).tobytes())
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    data = np.fromfile(out, np.int32)
    assert r.returncode == 0 and data[0] == 0, (r.returncode, data[:2], r.stderr[-500:])
    nv, ne = g.n_vertices, g.n_edges
    return data[1], data[2:2 + nv], data[2 + nv:2 + nv + ne], data[2 + nv + ne:2 + nv + 2 * ne]


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_program_scatter_matches_oracle(driver, port, tmp_path, mode):
    from vertexapi2_gb300 import graphs
    for g, source in ((graphs.rmat(10, 8, seed=81, weights=(1, 30)), 3),
                      (graphs.grid(30, 20, 0.15, seed=82), 0)):
        rounds, dist, visits, last = run_driver(driver, tmp_path, g, source, mode)
        rd, rv, rl, st = port.sssp_visits(g.n_vertices, g.srcs, g.dsts, g.weights, source)
        assert np.array_equal(dist, rd)
        assert np.array_equal(visits, rv)
        assert np.array_equal(last, rl)
        assert rounds == st["iterations"]
