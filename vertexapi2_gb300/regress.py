"""Regression-harness checks of the reference (regressions/checkDist.py,
checkPageRank.py, report.py), restated over "vid value" result files (the
format gas_write_vertex_values writes and the reference drivers print).

    python -m vertexapi2_gb300.regress checkdist test.txt gold.txt
    python -m vertexapi2_gb300.regress checkpagerank test.txt gold.txt
    python -m vertexapi2_gb300.regress report [directory]
"""
from __future__ import annotations

import glob
import math
import os
import sys

# A gold distance of PowerGraph's "unreachable" matches the engine's SSSP
# gatherZero (checkDist.py:43-44; sssp.cu:32-33).
GOLD_UNREACHABLE = 10000000
TEST_UNREACHABLE = 2147383647

# checkPageRank.py:74-80: |gold - test| bins [0,1e-4), [1e-4,1e-3), ...,
# [10, inf) and the largest share of vertices allowed in each.
PR_BOUNDS = (1e-4, 1e-3, 1e-2, 1e-1, 1.0, 10.0)
PR_ALLOWED = (1.0, 1e-2, 5e-3, 5e-4, 5e-5, 5e-6, 0.0)


def read_values(path: str, cast=int) -> list[tuple[int, float]]:
    """(vid, value) pairs of a result file, in file order."""
    out = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if parts:
                out.append((int(parts[0]), cast(parts[1])))
    return out


def check_dist(test: list[tuple[int, int]], gold: list[tuple[int, int]]) -> tuple[bool, str]:
    """checkDist.py:31-47: both lists sorted by vid; every gold vertex must be
    in the test list with the same integer value (gold 10000000 accepts
    2147383647).  Extra test vertices are allowed."""
    i = 0
    for vid, g in gold:
        while i < len(test) and test[i][0] < vid:
            i += 1
        if i >= len(test) or test[i][0] != vid:
            return False, f"vertex {vid} is in gold but not in test"
        t = test[i][1]
        if t != g and not (g == GOLD_UNREACHABLE and t == TEST_UNREACHABLE):
            return False, f"{vid} gold={g} ref={t}"
        i += 1
    return True, "No differences found"


def pagerank_histogram(test: dict[int, float], gold: dict[int, float]) -> list[float]:
    """Share of test vertices per |gold - test| bin (checkPageRank.py:40-59);
    vertices absent from gold count in the total only."""
    counts = [0] * (len(PR_BOUNDS) + 1)
    for vid, val in test.items():
        if vid not in gold:
            continue
        diff = math.fabs(gold[vid] - val)
        pos = len(PR_BOUNDS) - 1
        while pos >= 0 and diff < PR_BOUNDS[pos]:
            pos -= 1
        counts[pos + 1] += 1
    total = float(len(test)) or 1.0
    return [c / total for c in counts]


def check_pagerank(test: dict[int, float], gold: dict[int, float]) -> tuple[bool, list[float]]:
    """checkPageRank.py:62-65: every bin's share within its allowance."""
    h = pagerank_histogram(test, gold)
    return all(x <= a for x, a in zip(h, PR_ALLOWED)), h


def summary(cpu: dict[str, dict[str, float]], gpu: dict[str, dict[str, float]]) -> str:
    """report.py:34-44: per algorithm, one line per graph with the CPU and
    GPU times and their ratio."""
    lines = []
    for algo in sorted(set(cpu) | set(gpu)):
        lines.append("-" * 51)
        lines.append(f"Algorithm: {algo}")
        lines.append("-" * 51)
        graphs = sorted(set(cpu.get(algo, {})) | set(gpu.get(algo, {})))
        for g in graphs:
            c = cpu.get(algo, {}).get(g, -1.0)
            t = gpu.get(algo, {}).get(g, -1.0)
            ratio = c / t if t else float("inf")
            lines.append(f"{g[:20]:<20}  {c:8.1f}  {t:8.1f}  {ratio:8.1f}x")
        lines.append("-" * 51)
    return "\n".join(lines)


def read_timings(directory: str = "."):
    """report.py:24-31, 47-55: <graph>.<algo>.timing (CPU) and
    .timing_gpu files holding one number; unreadable files count -1."""
    cpu: dict[str, dict[str, float]] = {}
    gpu: dict[str, dict[str, float]] = {}
    for ext, table in (("timing", cpu), ("timing_gpu", gpu)):
        for path in glob.glob(os.path.join(directory, f"*.{ext}")):
            graph, algo = os.path.basename(path).split(".")[:2]
            try:
                val = float(open(path).read())
            except (OSError, ValueError):
                val = -1.0
            table.setdefault(algo, {})[graph] = val
    for a, b in ((cpu, gpu), (gpu, cpu)):  # every (algo, graph) in both tables
        for algo, row in a.items():
            for graph in row:
                b.setdefault(algo, {}).setdefault(graph, -1.0)
    return cpu, gpu


def main(argv: list[str]) -> int:
    if len(argv) == 3 and argv[0] == "checkdist":
        ok, msg = check_dist(read_values(argv[1]), read_values(argv[2]))
        print(msg)
        return 0 if ok else 1
    if len(argv) == 3 and argv[0] == "checkpagerank":
        ok, h = check_pagerank(dict(read_values(argv[1], float)), dict(read_values(argv[2], float)))
        if not ok:
            print("Share too high:", ", ".join(f"{x:.2e}/{a:.0e}" for x, a in zip(h, PR_ALLOWED)))
        return 0 if ok else 1
    if argv and argv[0] == "report":
        print(summary(*read_timings(argv[1] if len(argv) > 1 else ".")))
        return 0
    print("usage: python -m vertexapi2_gb300.regress "
          "{checkdist test gold | checkpagerank test gold | report [dir]}")
    return 1


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
