"""The reference's regression checks (checkDist.py, checkPageRank.py,
report.py) restated in vertexapi2_gb300.regress, and the engine's results
written as the drivers' "vid value" files passing them against the
oracle's."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden


def test_check_dist_rules():
    from vertexapi2_gb300.regress import check_dist
    gold = [(0, 0), (2, 5), (3, 10000000)]
    assert check_dist([(0, 0), (1, 9), (2, 5), (3, 2147383647)], gold)[0]  # extra vertex, unreachable
    assert not check_dist([(0, 0), (2, 6), (3, 10000000)], gold)[0]
    ok, msg = check_dist([(0, 0), (3, 10000000)], gold)
    assert not ok and "vertex 2" in msg
    assert not check_dist([(0, 0), (2, 5)], gold)[0]  # test ends early


def test_check_pagerank_bands():
    from vertexapi2_gb300.regress import check_pagerank, pagerank_histogram
    n = 100000
    gold = {i: 1.0 for i in range(n)}
    test = dict(gold)
    assert check_pagerank(test, gold)[0]
    for i in range(900):        # 0.9 % in [1e-4, 1e-3): allowed (1 %)
        test[i] = 1.0005
    assert check_pagerank(test, gold)[0]
    test[n - 1] = 1.5           # one vertex (1e-5) in [0.1, 1): allowed up to 5e-5
    assert check_pagerank(test, gold)[0]
    test[n - 2] = 12.0          # beyond 10: none allowed
    ok, h = check_pagerank(test, gold)
    assert not ok and h[-1] == 1.0 / n
    h = pagerank_histogram({0: 1.0, 7: 2.0}, {0: 1.00005})
    assert h == [0.5, 0, 0, 0, 0, 0, 0]  # vertex 7 only counts in the total


def test_report_and_cli(tmp_path, capsys):
    from vertexapi2_gb300 import regress
    (tmp_path / "ak2010.bfs.timing").write_text("120.0")
    (tmp_path / "ak2010.bfs.timing_gpu").write_text("3.0")
    (tmp_path / "ak2010.sssp.timing").write_text("bad")
    cpu, gpu = regress.read_timings(str(tmp_path))
    out = regress.summary(cpu, gpu)
    assert "Algorithm: bfs" in out and "40.0x" in out and "-1.0" in out
    (tmp_path / "t.txt").write_text("0 0\n1 3\n")
    (tmp_path / "g.txt").write_text("0 0\n1 3\n")
    assert regress.main(["checkdist", str(tmp_path / "t.txt"), str(tmp_path / "g.txt")]) == 0
    assert "No differences found" in capsys.readouterr().out
    (tmp_path / "p.txt").write_text("0 0.150000\n1 0.300000\n")
    assert regress.main(["checkpagerank", str(tmp_path / "p.txt"), str(tmp_path / "p.txt")]) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_engine_results_pass_regression_checks(gpu, port, tmp_path, name):
    """GPU results written as result files pass checkDist (BFS depths, SSSP
    distances) and checkPageRank against the oracle's files."""
    from vertexapi2_gb300 import GASEngine, graphio
    from vertexapi2_gb300 import programs as P
    from vertexapi2_gb300._lib import PROGRAM_BFS, PROGRAM_PAGERANK, PROGRAM_SSSP
    from vertexapi2_gb300.regress import check_dist, check_pagerank, read_values
    g = load_golden(name)
    nv, s, d = int(g["n_vertices"]), g["srcs"], g["dsts"]
    w = g["weights"] if "weights" in g else np.ones(len(s), np.int32)
    src = int(g["bfs_source"])
    runs = [(PROGRAM_BFS, P.bfs_init(nv), (src, src + 1), None, port.bfs(nv, s, d, src)[0]),
            (PROGRAM_SSSP, P.sssp_init(nv, 0), (0, nv), w, port.sssp(nv, s, d, w, 0)[0])]
    for prog, vd, act, ed, ref in runs:
        with GASEngine(prog) as e:
            e.set_graph(nv, vd, s, d, ed)
            e.set_active(*act)
            e.run()
            e.get_results()
        graphio.write_vertex_values(str(tmp_path / "test.txt"), vd)
        graphio.write_vertex_values(str(tmp_path / "gold.txt"), ref.astype(np.int32))
        ok, msg = check_dist(read_values(str(tmp_path / "test.txt")),
                             read_values(str(tmp_path / "gold.txt")))
        assert ok, msg
    vd = P.pagerank_init(nv, s)
    with GASEngine(PROGRAM_PAGERANK) as e:
        e.set_graph(nv, vd, s, d)
        e.set_active(0, nv)
        e.run(50)
        e.get_results()
    graphio.write_vertex_values(str(tmp_path / "pr.txt"), vd, field="rank")
    graphio.write_vertex_values(str(tmp_path / "prgold.txt"),
                                port.pagerank(nv, s, d, max_iters=50, fp64=True)[0].astype(np.float32))
    ok, h = check_pagerank(dict(read_values(str(tmp_path / "pr.txt"), float)),
                           dict(read_values(str(tmp_path / "prgold.txt"), float)))
    assert ok, h
