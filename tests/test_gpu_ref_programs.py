"""Drop-in check: the reference's own example Programs, compiled against the
C++ engine template and driven as the reference's drivers drive them.

* BFS (bfs.cu:24-112): apply(vertex, gatherResult) reads the round from a
  `__device__ __constant__` variable that the host loop sets with
  cudaMemcpyToSymbol between stepwise countActive / gatherApply(false) /
  scatterActivate(false) / nextIter calls.  Depths and rounds must equal
  the oracle's bit for bit.
* PageRank (pagerank.cu:27-101, constants made constexpr): every vertex
  active, run() until none is.  Ranks within 1e-5 relative L1 of the FP64
  oracle.  Per vertex, the FP32 oracle is matched to within the program's
  activation threshold (tol = 0.01, pagerank.cu:30): a vertex stops
  updating once its change falls below tol, so where two FP32 summation
  orders put a vertex's last update in different rounds its final values
  differ by up to tol (pagerank.cu:154-158's 1e-6 check assumes identical
  rounds).
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
EXE = os.path.join(HERE, "cpp", "_build", "ref_programs")


@pytest.fixture(scope="module")
def driver(gpu):
    src = os.path.join(HERE, "cpp", "ref_programs.cu")
    lib = os.path.join(ROOT, "vertexapi2_gb300", "_build")
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(src):
        cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
               "-I", os.path.join(ROOT, "include"), src, "-L", lib, "-lgas_gb300",
               "-Xlinker", f"-rpath={lib}", "-o", EXE]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
    return EXE


def run_driver(exe, tmp_path, nv, s, d, source, which):
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    head = np.array([nv, len(s), source, which], np.int32)
    with open(inp, "wb") as f:
        for a in (head, s, d):
            f.write(np.ascontiguousarray(a, np.int32).tobytes())
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    data = np.fromfile(out, np.int32)
    assert r.returncode == 0 and data[0] == 0, (r.returncode, data[:2], r.stderr[-500:])
    vals = data[2:2 + nv]
    return int(data[1]), (vals if which == 0 else vals.view(np.float32))


def cases():
    from vertexapi2_gb300 import graphs
    out = []
    for name in ("chesapeake", "rmat10_dir"):
        g = load_golden(name)
        out.append((name, int(g["n_vertices"]), g["srcs"], g["dsts"]))
    g = graphs.rmat(14, 16, seed=91, symmetrize=True)
    out.append(("rmat14_sym", g.n_vertices, g.srcs, g.dsts))
    g = graphs.grid(64, 48, 0.15, seed=92)
    out.append(("grid64x48", g.n_vertices, g.srcs, g.dsts))
    return out


@pytest.mark.parametrize("case", cases(), ids=lambda c: c[0])
def test_reference_bfs_program_stepwise(driver, port, tmp_path, case):
    from vertexapi2_gb300.programs import max_outdegree_vertex
    _, nv, s, d = case
    src = max_outdegree_vertex(nv, s)  # bfs.cu:148-166
    rounds, depth = run_driver(driver, tmp_path, nv, s, d, src, 0)
    ref, st = port.bfs(nv, s, d, src)
    assert np.array_equal(depth, ref)
    assert rounds == st["iterations"]


@pytest.mark.parametrize("case", cases(), ids=lambda c: c[0])
def test_reference_pagerank_program_run(driver, port, tmp_path, case):
    _, nv, s, d = case
    _, rank = run_driver(driver, tmp_path, nv, s, d, 0, 1)
    ref32, _ = port.pagerank(nv, s, d)
    ref64, _ = port.pagerank(nv, s, d, fp64=True)
    a = rank.astype(np.float64)
    assert np.abs(a - ref64).sum() <= 1e-5 * np.abs(ref64).sum()
    assert np.abs(a - ref32).max() <= 0.01 + 1e-4 * np.abs(ref32).max()
