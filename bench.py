"""Benchmark of the GB300 GAS engine (one JSON line on stdout).

Headline workload: SSSP on the 1024x1024 4-neighbour lattice with 15% of
its edges deleted (largest component kept, relabelled row-major), int32
weights uniform in [1, 100], source 0, every vertex active at start -- the
configuration the reference's GTEPS metric is quoted on for one GPU.
A step is one full run(): rounds of gather/apply + scatter/activate until no
vertex is active, from the driver's initial vertex data (sssp.cu:67-82).

  value   GTEPS = edges traversed (in-edges gathered + out-edges scattered,
          summed over rounds) / device time, inputs resident in HBM
  e2e     the same through the C ABI with host buffers: vertex data H2D
          from pinned memory, run(), results D2H, every step
  roofline  the run's kernels: algorithmic bytes / their CUDA-event time
  cpu_baseline  the oracle (CPU restatement of the reference engine) on
          the same graph, one run on one core
  parity  the run's result against the oracle's on the same graph

per_algo (default run on one GPU): the same record for every other
workload of the metric -- BFS on R-MAT-16, PageRank FP32 and connected
components on R-MAT-22, the batched queries (256 BFS + 256 SSSP per graph)
and the serving loop over 8 resident graphs -- each with its own value,
e2e, roofline or latency figures, CPU baseline and oracle parity.

--impl reference times the reference's CPU engine (oracle/_ref where it
was built, else the oracle restatement) with every host core running one
instance of the headline workload; its graphs come from the oracle's own
generators, so that process never loads the product library.

Multi-GPU: replicas only (every rank runs the workload on its own GPU; the
path has no exchange step); value sums the ranks' edges over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 512 << 20   # > 129 MB L2
SEED = 1

WORKLOADS = {
    "sssp-grid1024": dict(desc="SSSP, 1024x1024 lattice, 15% edges deleted, LCC, w in [1,100], source 0"),
    "bfs-rmat16": dict(desc="BFS, R-MAT scale 16 ef 16 (0.57/0.19/0.19), symmetrised, source = max out-degree"),
    "pagerank-rmat22": dict(desc="PageRank FP32 (0.85, tol 0.01, <=50 rounds), R-MAT scale 22 ef 16, directed"),
    "cc-rmat22": dict(desc="connected components, R-MAT scale 22 ef 16, symmetrised"),
    "batch-c4": dict(desc="256 BFS + 256 SSSP queries, uniform random sources, on R-MAT scale 21 "
                          "ef 16 symmetrised (w in [1,255]) and on the 1024x1024 lattice; batched "
                          "engine vs one-at-a-time plain runs"),
    "serve-c5": dict(desc="serving loop over 8 resident graphs (R-MAT scales 12,14,16,18,20,21,22 "
                          "ef 16 symmetrised, w in [1,255]; the 1024x1024 lattice, w in [1,100]); "
                          "Poisson arrivals of a 50/30/20 BFS/SSSP/PPR (FP32, alpha 0.15, 20 "
                          "rounds) mix on uniform random graph and source; served vs "
                          "one-at-a-time plain engine"),
}
HEADLINE = "sssp-grid1024"
PER_ALGO = ("bfs-rmat16", "pagerank-rmat22", "cc-rmat22", "batch-c4", "serve-c5")
RMAT_SCALE = {"pagerank-rmat22": 22, "cc-rmat22": 22}
PROGRAM_NAMES = {1: "bfs", 2: "sssp", 3: "cc", 4: "pagerank", 5: "ppr"}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per run (the
# run's kernels) from ncu captures of the same command (profiles/): the
# lattice run's two kernels directly (main kernel 71.7 + 4.0 MB, one-round
# dense kernel 41.1 + 0.4 MB, L2 flushed before the step); PageRank's two kernels on
# R-MAT-20 (2.381 GB per run, 16.09 M edges) scaled by edges, its traffic
# being per-edge gathers and the CSC stream; CC the same way; BFS on R-MAT-16
# directly.  None where no capture exists.
TRAFFIC_PER_LAUNCH = {
    "sssp-grid1024": 71.680512e6 + 4.024320e6 + 41.136896e6 + 0.366080e6,
    "pagerank-rmat22": (2.094825e9 + 0.218918e9 + 0.063529e9 + 0.003429e9) * (65244320 / 16086703),
    # CC's two kernels on R-MAT-20 symmetric (31,406,204 edges), scaled by edges
    "cc-rmat22": (424.575488e6 + 15.346176e6 + 37.384960e6 + 0.033024e6) * (128308912 / 31406204),
    # BFS on R-MAT-16 captured at full size
    "bfs-rmat16": 8.890368e6,
}


class Graph:
    """An edge list (srcs -> dsts, optional int32 weights)."""

    def __init__(self, n_vertices, srcs, dsts, weights=None):
        self.n_vertices = int(n_vertices)
        self.srcs, self.dsts, self.weights = srcs, dsts, weights

    @property
    def n_edges(self) -> int:
        return int(self.srcs.shape[0])


def gen_rmat(scale, seed, symmetrize=False, weights=None, source="product"):
    """The seeded R-MAT graph: from the product's generator, or ("oracle")
    from the oracle's independent one (identical edge lists; the reference
    arm uses it so that its process never loads the product library)."""
    if source == "oracle":
        import oracle
        return Graph(*oracle.port().gen_rmat(scale, 16, seed=seed, symmetrize=symmetrize,
                                             weights=weights))
    from vertexapi2_gb300 import graphs
    g = graphs.rmat(scale, 16, seed=seed, symmetrize=symmetrize, weights=weights)
    return Graph(g.n_vertices, g.srcs, g.dsts, g.weights)


def gen_grid(side, seed, weights=(1, 100), source="product"):
    if source == "oracle":
        import oracle
        return Graph(*oracle.port().gen_grid(side, side, 0.15, seed=seed, weights=weights))
    from vertexapi2_gb300 import graphs
    g = graphs.grid(side, side, 0.15, seed=seed, weights=weights)
    return Graph(g.n_vertices, g.srcs, g.dsts, g.weights)


def max_outdegree_vertex(n, srcs) -> int:
    """bfs.cu:148-166: the first vertex with the largest out-degree."""
    return int(np.argmax(np.bincount(srcs, minlength=n)))


def make_workload(name: str, source: str = "product"):
    """Graph, program and initial state of a plain-engine workload (program
    ids and initial vertex data as include/gas_gb300.h and the reference
    drivers define them)."""
    unreached = 2**31 - 1 - 100000   # sssp.cu:32-33
    if name == "sssp-grid1024":
        g = gen_grid(1024, SEED, source=source)
        init = np.full(g.n_vertices, unreached, np.int32)
        init[0] = 0
        return dict(program=2, g=g, source=0, init=init,
                    active=(0, g.n_vertices), max_iters=0, vd_bytes=4, ed_bytes=4, gather=True)
    if name == "bfs-rmat16":
        g = gen_rmat(16, SEED, symmetrize=True, source=source)
        s = max_outdegree_vertex(g.n_vertices, g.srcs)
        return dict(program=1, g=g, source=s, init=np.full(g.n_vertices, -1, np.int32),
                    active=(s, s + 1), max_iters=0, vd_bytes=4, ed_bytes=0, gather=False)
    if name == "pagerank-rmat22":
        g = gen_rmat(RMAT_SCALE[name], SEED, source=source)
        init = np.zeros(g.n_vertices, dtype=[("rank", np.float32), ("numOutEdges", np.int32)])
        init["rank"] = np.float32(0.15)
        init["numOutEdges"] = np.bincount(g.srcs, minlength=g.n_vertices)
        return dict(program=4, g=g, source=0, init=init,
                    active=(0, g.n_vertices), max_iters=50, vd_bytes=8, ed_bytes=0, gather=True)
    if name == "cc-rmat22":
        g = gen_rmat(RMAT_SCALE[name], SEED, symmetrize=True, source=source)
        return dict(program=3, g=g, source=0, init=np.arange(g.n_vertices, dtype=np.int32),
                    active=(0, g.n_vertices), max_iters=0, vd_bytes=4, ed_bytes=0, gather=True)
    raise SystemExit(f"unknown workload {name}")


def workload_config(name: str, g=None) -> dict:
    """The `config` object of a workload: identical in both arms."""
    cfg = {"workload": name, "desc": WORKLOADS[name]["desc"], "seed": SEED}
    if g is not None:
        cfg.update(n_vertices=g.n_vertices, n_edges=g.n_edges)
        if name in RMAT_SCALE:
            cfg["rmat_scale"] = RMAT_SCALE[name]
    return cfg


def round_bytes(st: dict, vd: int, ed: int, gather: bool):
    """Algorithmic (compulsory) bytes per round, gather+apply and scatter.

    gather+apply: |A|*(4 id + 8 offset pair + 2*VD read/write + 1 ret)
                  + |E_in|*(4 source id + ED + VD of the source)
    apply only:   |A|*(4 id + 2*VD + 1 ret)
    scatter:      |R|*8 offset pair + |E_out|*4 destination id
                  + 4 per vertex appended to the next frontier
    """
    a, ein, r, eout = (st[k].astype(np.float64) for k in ("active", "gathered", "ret", "scattered"))
    if gather:
        g = a * (4 + 8 + 2 * vd + 1) + ein * (4 + ed + vd)
    else:
        g = a * (4 + 2 * vd + 1)
    nxt = np.concatenate([a[1:], [0.0]])
    s = r * 8 + eout * 4 + nxt * 4
    return g, s


def measured_peak() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def mapped_libraries() -> list[str]:
    """Shared libraries of this repository mapped into this process."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                p = line.split()[-1] if line.strip() else ""
                if p.startswith(ROOT) and ".so" in p:
                    out.add(os.path.relpath(p, ROOT))
    except OSError:
        pass
    return sorted(out)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.path or not os.path.exists(self.path):
            return None
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxs.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sms:
            return None
        return {"sm_mhz": float(np.median(sms)), "sm_max_mhz": float(max(maxs)),
                "reasons": sorted(reasons), "samples": len(sms)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_run(engine, w, name, fp64=False):
    """One oracle run of a plain workload: (result, stats)."""
    g = w["g"]
    if name == "sssp-grid1024":
        return engine.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, w["source"], stats_cap=1 << 14)
    if name == "bfs-rmat16":
        return engine.bfs(g.n_vertices, g.srcs, g.dsts, w["source"], stats_cap=1 << 14)
    if name == "pagerank-rmat22":
        return engine.pagerank(g.n_vertices, g.srcs, g.dsts, max_iters=50, fp64=fp64,
                               stats_cap=1 << 14)
    return engine.cc(g.n_vertices, g.srcs, g.dsts, stats_cap=1 << 14)


def in_threads(*fns):
    """Runs the callables at once on host threads (ctypes calls drop the
    GIL) and returns their results in order."""
    out = [None] * len(fns)

    def run(i, f):
        out[i] = f()
    ts = [threading.Thread(target=run, args=(i, f)) for i, f in enumerate(fns)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out


def pr_error(got: np.ndarray, ref64: np.ndarray) -> dict:
    """FP32 PageRank against the FP64 oracle: relative L1 and the largest
    per-vertex relative error."""
    a, b = got.astype(np.float64), ref64.astype(np.float64)
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    return {"rel_l1_vs_fp64": float(np.abs(a - b).sum() / np.abs(b).sum()),
            "max_rel_err_vs_fp64": float(rel.max()), "bound_rel_l1": 1e-5}


# ---------------------------------------------------------------- C5 / C4 --
C5_GRAPHS = [("rmat12", 12), ("rmat14", 14), ("rmat16", 16), ("rmat18", 18), ("rmat20", 20),
             ("rmat21", 21), ("rmat22", 22), ("grid1024", None)]
C5_MIX = (0.5, 0.3, 0.2)      # BFS / SSSP / PPR
C5_QUERIES = 1024             # queries per timed step
C5_SWEEP = (0.25, 0.5, 0.75)  # offered load, as fractions of the measured capacity
C5_SWEEP_QUERIES = 512
C5_LANES = 8                  # batches in flight at once


def c5_graphs(only=None, source="product"):
    out = []
    for name, sc in C5_GRAPHS:
        if only and name not in only:
            continue
        if sc is None:
            g = gen_grid(1024, SEED, source=source)
        else:
            g = gen_rmat(sc, SEED + sc, symmetrize=True, weights=(1, 255), source=source)
        out.append((name, g))
    return out


def c4_graphs(scale=21, side=1024, source="product"):
    return [(f"rmat{scale}", gen_rmat(scale, SEED, symmetrize=True, weights=(1, 255), source=source)),
            (f"grid{side}", gen_grid(side, SEED, source=source))]


def query_mix(gs, n, seed, mix=C5_MIX):
    """n (graph index, program, source) triples: programs drawn from `mix`
    (BFS/SSSP/PPR), graph and source uniform."""
    rng = np.random.default_rng(seed)
    progs = rng.choice([1, 2, 5], size=n, p=list(mix))
    gids = rng.integers(0, len(gs), n)
    srcs = [int(rng.integers(0, gs[k][1].n_vertices)) for k in gids]
    return list(zip(gids.tolist(), progs.tolist(), srcs))


def cpu_cells(gs, cells, threads, per_cell=1, seed=SEED + 11):
    """CPU engines' throughput on a query mix, stratified by cell.

    `cells` maps (graph index, program) to the cell's share of the mix.
    Each cell runs `per_cell` seeded random sources; all of them run at
    once on `threads` host threads (ctypes calls drop the GIL), largest
    graphs first.  BFS/SSSP use oracle/_ref (the reference engine built in
    place) when it was built, else the restatement; PPR (not a reference
    program) the restatement.  run() is timed inside the engine (graph
    construction excluded, as bfs.cu:100-111 times it).  Throughput =
    threads / (sum over cells of share x mean run time): `threads` engines
    each answering queries of the mix back to back.
    Returns (queries/s, queries run, wall s, engine kind)."""
    import queue
    import oracle
    port = oracle.port()
    eng = oracle.ref() or port
    rng = np.random.default_rng(seed)
    work = queue.Queue()
    order = sorted(cells, key=lambda c: -gs[c[0]][1].n_edges)
    for k, p in order:
        for s0 in rng.integers(0, gs[k][1].n_vertices, per_cell):
            work.put((k, p, int(s0)))
    times = {c: [] for c in cells}
    lock = threading.Lock()

    def worker():
        while True:
            try:
                k, p, s0 = work.get_nowait()
            except queue.Empty:
                return
            g = gs[k][1]
            if p == 1:
                _, st = eng.bfs(g.n_vertices, g.srcs, g.dsts, s0)
            elif p == 2:
                _, st = eng.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, s0)
            else:
                _, st = port.ppr(g.n_vertices, g.srcs, g.dsts, s0, iters=20)
            with lock:
                times[(k, p)].append(st["run_ns"] / 1e9)

    t0 = time.perf_counter()
    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    wall = time.perf_counter() - t0
    expected = sum(share * float(np.mean(times[c])) for c, share in cells.items())
    return threads / expected, per_cell * len(cells), wall, eng.kind


def c5_cells(gs):
    progs = dict(zip((1, 2, 5), C5_MIX))
    return {(k, p): w / len(gs) for k in range(len(gs)) for p, w in progs.items()}


def c4_cells(gs):
    return {(k, p): 1.0 / (2 * len(gs)) for k in range(len(gs)) for p in (1, 2)}


# --------------------------------------------------------- reference arm --
def run_reference(args):
    """The reference's CPU engine on every host core (rank 0 only), on the
    headline workload (or the one --workload names).  Graphs come from the
    oracle's generators: the product library is never loaded here."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    import oracle
    cores = os.cpu_count() or 1
    port = oracle.port()
    eng = oracle.ref() or port
    if args.workload in ("batch-c4", "serve-c5"):
        if args.workload == "batch-c4":
            gs = c4_graphs(source="oracle")
            cells = c4_cells(gs)
            metric = "batched queries/s (vs one-at-a-time plain engine)"
        else:
            gs = c5_graphs(source="oracle")
            cells = c5_cells(gs)
            metric = "served queries/s, p50/p99 latency (vs one-at-a-time plain engine)"
        per_cell = max(1, -(-cores // len(cells)))
        value, n, wall, kind = cpu_cells(gs, cells, cores, per_cell)
        sample = (f"one step (of the {args.steps} asked; a cell of the largest graph runs for "
                  f"minutes on one core): {per_cell} random source(s) per (graph, program) cell, "
                  f"{n} queries on {cores} threads in {wall:.0f} s; value = {cores} / (mix-weighted "
                  f"mean run() time); BFS/SSSP on the {kind} engine, PPR on the restatement")
        line = {"metric": metric, "value": value, "unit": "queries/s", "steps": 1, "warmup": 0,
                "ms_per_step": 1e3 * wall, "config": workload_config(args.workload),
                "cpu_baseline": {"value": value, "unit": "queries/s", "cores": cores,
                                 "kind": kind, "sample": sample}}
    else:
        w = make_workload(args.workload, source="oracle")
        # traversed edges per run (from the restatement's instrumented counts)
        _, st = cpu_run(port, w, args.workload)
        edges = float(st["gathered"].sum() + st["scattered"].sum())

        def one_step():
            t0 = time.perf_counter()
            in_threads(*[lambda: cpu_run(eng, w, args.workload)] * cores)
            return time.perf_counter() - t0

        for _ in range(args.warmup):
            one_step()
        times = [one_step() for _ in range(args.steps)]
        total = sum(times)
        value = cores * edges * args.steps / total / 1e9
        line = {"metric": "GTEPS & %HBM roofline per algo", "value": value, "unit": "GTEPS",
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
                "config": workload_config(args.workload, w["g"]),
                "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": cores, "kind": eng.kind,
                                 "sample": f"{cores} concurrent full runs of the workload per step "
                                           f"({st['iterations']} rounds each)"}}
    libs = mapped_libraries()
    if any("libgas_gb300" in p for p in libs):
        raise SystemExit(f"reference arm mapped the product library: {libs}")
    unit = line["unit"]
    line.update({
        "impl": "reference", "n_gpus": args.gpus, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "e2e": {"value": line["value"], "unit": unit, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "native_libraries": libs,
    })
    print(json.dumps(line))


# ------------------------------------------------------- plain workloads --
def run_rounds(e, w, stepwise):
    """One run() of a plain workload, or (stepwise) the same rounds through
    countActive / gatherApply / scatterActivate / nextIter, the loop of the
    reference's drivers (bfs.cu:98-108)."""
    if not stepwise:
        return e.run(w["max_iters"])
    it = 0
    e.set_iteration(0)
    while (w["max_iters"] == 0 or it < w["max_iters"]) and e.count_active():
        e.gather_apply(w["gather"])
        e.scatter_activate(w["gather"])
        e.next_iter()
        it += 1
        e.set_iteration(it)
    return it


def measure_plain(name, steps, warmup, world, rank, local, with_cpu=True, stepwise=False):
    """One plain-engine workload: device-timed GTEPS, e2e through the C ABI,
    roofline of the run's kernels, CPU baseline and oracle parity.  With
    stepwise, every round is driven from the host (one gather/apply and one
    scatter/activate launch per round) instead of run()'s persistent kernel."""
    import torch
    import vertexapi2_gb300 as gas
    w = make_workload(name)
    g = w["g"]
    stream = torch.cuda.current_stream()
    eng = gas.GASEngine(w["program"], device=local, stream=stream.cuda_stream)
    init = w["init"].copy()
    ed = g.weights if w["ed_bytes"] else None
    t_sg = time.perf_counter()
    eng.set_graph(g.n_vertices, init, g.srcs, g.dsts, ed)
    set_graph_ms = 1e3 * (time.perf_counter() - t_sg)
    eng.save_vertex_data()
    lo, hi = w["active"]

    def device_step():
        eng.restore_vertex_data()
        eng.set_active(lo, hi)
        return run_rounds(eng, w, stepwise)

    for _ in range(max(warmup, 1)):
        rounds = device_step()
    stats = eng.round_stats()
    edges_per_run = float(stats["gathered"].sum() + stats["scattered"].sum())
    # per-kernel CUDA-event profile (separate, untimed pass)
    eng.set_profiling(True)
    device_step()
    kt = eng.kernel_times()
    eng.set_profiling(False)
    gbytes, sbytes = round_bytes(stats, w["vd_bytes"], w["ed_bytes"], w["gather"])

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=f"cuda:{local}")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    barrier(world)
    torch.cuda.synchronize()
    run_kernel_ms = 0.0
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for k in range(steps):
            flush.fill_(k)                      # L2 flush between timed steps
            eng.restore_vertex_data()
            ev[k][0].record(stream)
            eng.set_active(lo, hi)
            run_rounds(eng, w, stepwise)
            ev[k][1].record(stream)
            if not stepwise:
                run_kernel_ms += eng.last_run_ms()  # the run kernels' own events
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    if stepwise:  # the rounds' kernels and the host round trips between them
        run_kernel_ms = float(sum(step_ms))
    total_ms = allreduce_max(world, float(sum(step_ms)))
    all_edges = allreduce_sum(world, edges_per_run * steps)
    value = all_edges / (total_ms / 1e3) / 1e9

    # end to end through the C ABI with host buffers: initial vertex data
    # H2D from pinned memory, run(), results D2H into the borrowed array
    host_in = torch.from_numpy(init.view(np.uint8).copy()).pin_memory().numpy().view(init.dtype)
    result = torch.empty(init.nbytes, dtype=torch.uint8).pin_memory().numpy().view(init.dtype)
    e2e_eng = gas.GASEngine(w["program"], device=local, stream=stream.cuda_stream)
    e2e_eng.set_graph(g.n_vertices, result, g.srcs, g.dsts, ed)
    for _ in range(max(1, warmup)):
        e2e_eng.set_vertex_data(host_in)
        e2e_eng.set_active(lo, hi)
        run_rounds(e2e_eng, w, stepwise)
        e2e_eng.get_results()
    barrier(world)
    torch.cuda.synchronize()
    e2e_local = 0.0
    for k in range(steps):
        flush.fill_(k)  # L2 flushed before each step, as for the device-timed steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_eng.set_vertex_data(host_in)
        e2e_eng.set_active(lo, hi)
        run_rounds(e2e_eng, w, stepwise)
        e2e_eng.get_results()
        torch.cuda.synchronize()
        e2e_local += time.perf_counter() - t0
    e2e_s = allreduce_max(world, e2e_local)
    e2e_value = all_edges / e2e_s / 1e9
    eng.get_results()  # device-resident run's result, into `init`
    e2e_eng.close()
    eng.close()
    del flush
    nbytes = init.nbytes
    # per-step device times (min and median of the timed steps), and for BFS
    # the Graph500 count: edges within the reached component / 2 per second
    step_stats = {"min": float(np.min(step_ms)), "median": float(np.median(step_ms)),
                  "n": len(step_ms)}
    graph500 = None
    if w["program"] == 1:
        reached = init != -1
        outdeg = np.bincount(g.srcs, minlength=g.n_vertices)
        comp_edges = float(outdeg[reached].sum()) / 2.0
        graph500 = {"gteps": comp_edges / (step_stats["median"] / 1e3) / 1e9,
                    "edges_in_component": comp_edges, "at": "median step"}

    peak, peak_kind = measured_peak()
    run_bytes = float(gbytes.sum() + sbytes.sum())
    kernel_ms = run_kernel_ms / steps
    achieved = run_bytes / (kernel_ms / 1e3) / 1e9 if kernel_ms > 0 else 0.0
    # set_active's range split, run()'s zeroing of its counters and round-0
    # bitmaps, the leading dense-rounds kernel when every vertex starts
    # active, the persistent run
    dense_first = (lo, hi) == (0, g.n_vertices)
    launches_per_step = 3 + (1 if dense_first else 0)
    kernel_label = ("run_dense_kernel + run_persistent_kernel" if dense_first
                    else "run_persistent_kernel")
    if stepwise:
        launches_per_step = 1 + 2 * rounds
        kernel_label = "gather_apply_kernel + scatter_activate_kernel (stepwise)"

    # CPU baseline (one core, the restatement) and parity with the oracle
    cpu, parity = None, None
    if rank == 0 and with_cpu:
        import oracle
        port = oracle.port()
        t0 = time.perf_counter()
        if w["program"] == 4:  # FP32 baseline and the FP64 oracle side by side
            (ref, st), (ref64, _) = in_threads(lambda: cpu_run(port, w, name),
                                               lambda: cpu_run(port, w, name, fp64=True))
        else:
            ref, st = cpu_run(port, w, name)
        cpu_s = time.perf_counter() - t0
        cpu_edges = float(st["gathered"].sum() + st["scattered"].sum())
        cpu = {"value": cpu_edges / (st["run_ns"] / 1e9) / 1e9, "unit": "GTEPS", "cores": 1,
               "kind": "port",
               "sample": f"one full run of the workload ({st['iterations']} rounds, "
                         f"{cpu_s:.1f} s wall), run()+getResults() timed as bfs.cu:100-111"}
        same_rounds = st["iterations"] == rounds
        if w["program"] == 4:
            parity = dict(pr_error(init["rank"], ref64), vs="oracle FP64 PageRank (same graph)",
                          e2e_rel_l1_vs_fp64=pr_error(result["rank"], ref64)["rel_l1_vs_fp64"],
                          rounds_equal=bool(same_rounds))
            parity["ok"] = bool(parity["rel_l1_vs_fp64"] <= 1e-5 and
                                parity["e2e_rel_l1_vs_fp64"] <= 1e-5)
        else:
            ok = bool(np.array_equal(init, ref) and np.array_equal(result, ref))
            parity = {"vs": "oracle (same graph)", "bit_exact": ok, "rounds_equal": bool(same_rounds),
                      "ok": ok and bool(same_rounds)}
    return {
        "metric": "GTEPS & %HBM roofline per algo", "value": value, "unit": "GTEPS",
        "n_gpus": world, "steps": steps, "warmup": warmup,
        "ms_per_step": total_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if w["program"] == 4 else "int32",
        "data": "synthetic",
        "config": workload_config(name, g),
        "run": {"rounds": rounds, "edges_traversed_per_run": edges_per_run,
                "driver": "stepwise (host loop per round)" if stepwise else "run() (persistent)",
                "l2": "flushed before every timed step, device-timed and end-to-end (512 MB write)",
                "parallelism": f"replicas x{world}", "set_graph_ms": set_graph_ms,
                "step_ms": step_stats},
        "roofline": {"bound": "hbm", "kernel": kernel_label, "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": (TRAFFIC_PER_LAUNCH.get(name)
                                 if RMAT_SCALE.get(name, 22) == 22 else None),
                     "kernel_ms_per_launch": kernel_ms,
                     "algorithmic_bytes_per_launch": run_bytes,
                     "phase_profile_per_launch_kernels": {
                         "gather_apply_ms": kt["gather_ms"], "scatter_activate_ms": kt["scatter_ms"],
                         "gather_apply_bytes": float(gbytes.sum()),
                         "scatter_activate_bytes": float(sbytes.sum())}},
        "cpu_baseline": cpu,
        "parity": parity,
        "e2e": {"value": e2e_value, "unit": "GTEPS", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "ms_per_step": 1e3 * e2e_s / steps},
        "gpu_launches": launches_per_step * steps,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
        **({"graph500": graph500} if graph500 else {}),
    }


# ------------------------------------------------------------------- C4 --
def measure_batch_c4(args, steps, warmup, world, rank, local, with_cpu=True):
    """Batched multi-source queries (queries/s) vs one-at-a-time plain runs,
    with a sample of every set checked against the oracle.  value counts
    the 256 BFS + 256 SSSP queries per graph; a batched personalised
    PageRank set (256 sources on the R-MAT graph) is reported beside it."""
    import torch
    import vertexapi2_gb300 as gas
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(SEED)
    nq = 256
    gs = c4_graphs(args.rmat_scale or 21, args.grid_side)
    only = set(args.c4_sets.split(",")) if args.c4_sets else None
    sets = []
    progs = {gs[0][0]: (1, 2, 5), gs[1][0]: (1, 2)}
    for name, g in gs:
        for prog in progs[name]:
            src = rng.integers(0, g.n_vertices, nq).astype(np.int32)
            key = f"{name}-{PROGRAM_NAMES[prog]}"
            if only is not None and key not in only:
                continue
            # one batch object per set: its tuned settings and captured
            # CUDA graph stay in place from step to step
            b = gas.GASBatch(device=local, stream=stream.cuda_stream)
            b.set_graph(g.n_vertices, g.srcs, g.dsts, g.weights if prog == 2 else None)
            if args.no_autotune:
                b.set_config(256, args.c4_blocks, True)
                b.set_delta(args.c4_delta if prog == 2 else 0)
            else:
                b.autotune(prog, nq)
            sets.append((key, g, b, prog, src, b.tuning()))
    per_set_ms = [0.0] * len(sets)
    per_set_rounds = [0] * len(sets)

    def batched_step():
        for i, (key, g, b, prog, src, t) in enumerate(sets):
            _, per_set_rounds[i] = b.run(prog, src, want_results=False)
            per_set_ms[i] += b.last_ms()
    for _ in range(warmup):
        batched_step()
    barrier(world)
    torch.cuda.synchronize()
    per_set_ms[:] = [0.0] * len(sets)
    with ClockSampler(local) as clk:
        for _ in range(steps):
            batched_step()
    head = [i for i, x in enumerate(sets) if x[3] != 5]   # BFS + SSSP: the metric's queries
    if not head:  # a subset of PPR sets only (--c4-sets): report those
        head = list(range(len(sets)))
    total_ms = allreduce_max(world, float(sum(per_set_ms[i] for i in head)))
    queries = allreduce_sum(world, float(len(head) * nq * steps))
    value = queries / (total_ms / 1e3)
    # end to end: sources up and every query's result copied to host memory
    outs = [None] * len(sets)
    e2e_s = 0.0
    for i, (key, g, b, prog, src, t) in enumerate(sets):
        t0 = time.perf_counter()
        outs[i] = b.run(prog, src, want_results=True)[0]
        if i in head:
            e2e_s += time.perf_counter() - t0
    e2e_value = len(head) * nq / e2e_s
    d2h = sum(nq * sets[i][1].n_vertices * 4 for i in head)
    # one-at-a-time plain engine on a sample of the same queries
    from vertexapi2_gb300 import programs as P
    sample = 8
    single_ms, single_n = 0.0, 0
    parity, ppr_plain_err = True, 0.0
    per_set = {}
    for i, (key, g, b, prog, src, t) in enumerate(sets):
        s_ms = 0.0
        e = gas.GASEngine(prog, device=local, stream=stream.cuda_stream)
        for q, s0 in enumerate(src[:sample]):
            s0 = int(s0)
            if prog == 1:
                vd, act = P.bfs_init(g.n_vertices), (s0, s0 + 1)
            elif prog == 2:
                vd, act = P.sssp_init(g.n_vertices, s0), (0, g.n_vertices)
            else:
                vd, act = P.ppr_init(g.n_vertices, g.srcs, s0), (0, g.n_vertices)
            e.set_graph(g.n_vertices, vd, g.srcs, g.dsts, g.weights if prog == 2 else None) \
                if q == 0 else e.set_vertex_data(vd)
            e.set_active(*act)
            e.run(20 if prog == 5 else 0)
            s_ms += e.last_run_ms()
            e.get_results()  # into the array borrowed by set_graph
            if prog == 5:
                ppr_plain_err = max(ppr_plain_err, pr_error(outs[i][q], e.vertex_data["rank"])["rel_l1_vs_fp64"])
            else:
                parity &= bool(np.array_equal(e.vertex_data, outs[i][q]))
        e.close()
        if i in head:
            single_ms += s_ms
            single_n += sample
        per_set[key] = {"batched_ms_per_256": per_set_ms[i] / steps,
                        "batched_rounds": per_set_rounds[i],
                        "single_ms": s_ms / sample,
                        "speedup": (s_ms / sample * nq) / (per_set_ms[i] / steps),
                        "tuning": t}
    for x in sets:
        x[2].close()
    single_qps = single_n / (single_ms / 1e3)
    # oracle parity on a sample of every set (two queries per set, at once)
    oracle_ok, oracle_n, ppr_err, cpu = None, 0, 0.0, None
    if rank == 0 and with_cpu:
        import oracle
        port = oracle.port()
        jobs = []
        for i, (key, g, b, prog, src, t) in enumerate(sets):
            for q in (0, nq - 1):
                x = int(src[q])
                if prog == 1:
                    f = lambda g=g, x=x: port.bfs(g.n_vertices, g.srcs, g.dsts, x)[0]
                elif prog == 2:
                    f = lambda g=g, x=x: port.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, x)[0]
                else:
                    f = lambda g=g, x=x: port.ppr(g.n_vertices, g.srcs, g.dsts, x, iters=20, fp64=True)[0]
                jobs.append((i, q, f))
        res = in_threads(*[f for _, _, f in jobs])
        oracle_ok = True
        for (i, q, _), r in zip(jobs, res):
            if sets[i][3] == 5:
                ppr_err = max(ppr_err, pr_error(outs[i][q], r)["rel_l1_vs_fp64"])
            else:
                oracle_ok &= bool(np.array_equal(r, outs[i][q]))
        oracle_n = len(jobs)
        cores = os.cpu_count() or 1
        cells = c4_cells(gs)
        v, n, wall, kind = cpu_cells(gs, cells, cores, max(1, -(-cores // len(cells))))
        cpu = {"value": v, "unit": "queries/s", "cores": cores, "kind": kind,
               "sample": f"{n} random sources spread over the (graph, program) cells on {cores} "
                         f"threads in {wall:.0f} s; value = {cores} / (mean run() time per query "
                         f"of the mix)"}
    return {
        "metric": "batched queries/s (vs one-at-a-time plain engine)", "value": value,
        "unit": "queries/s", "n_gpus": world, "steps": steps, "warmup": warmup,
        "ms_per_step": total_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config("batch-c4"),
        "run": {"queries_per_step": len(head) * nq,
                "l2": "inputs (R-MAT-21 CSC/CSR, 2 GB query state) larger than L2",
                "sets": "one persistent launch per set of 256 queries (BFS and SSSP launched "
                        "separately), each replayed from its captured CUDA graph"},
        "one_at_a_time": {"value": single_qps, "unit": "queries/s", "sample_queries": single_n,
                          "speedup": value / single_qps, "results_identical": parity,
                          "ppr_max_rel_l1_vs_plain": ppr_plain_err},
        "per_set": per_set,
        "parity": {"vs": "oracle BFS/SSSP (bit-exact) and FP64 PPR on the first and last source "
                         "of every set", "queries": oracle_n, "bit_exact": oracle_ok,
                   "ppr_max_rel_l1_vs_fp64": ppr_err,
                   "ok": bool(oracle_ok and parity and ppr_err <= 1e-5) if oracle_ok is not None else None},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": 4 * nq * len(head),
                "d2h_bytes_per_step": d2h},
        "gpu_launches": 5 * len(sets) * steps,
        "clocks": clk.summary(),
    }


# ------------------------------------------------------------------- C5 --
def serve_pass(srv, ids, gs, queries, rate, bufs, seed, keep=None):
    """Submits `queries` with Poisson arrivals at `rate` queries/s (inf: all
    at once) from a submitter thread while this thread waits for each result
    in submission order and copies it into the graph's pinned buffer (and a
    copy of it into `keep[i]` for the indices `keep` holds).
    Returns per-query infos and the wall time from the first submission to
    the last result in host memory."""
    import queue
    n = len(queries)
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n)) if np.isfinite(rate) else np.zeros(n)
    arrivals -= arrivals[0]
    handoff = queue.Queue()
    t0 = time.perf_counter()

    def submitter():
        for i, (k, p, src) in enumerate(queries):
            target = t0 + arrivals[i]
            while True:
                d = target - time.perf_counter()
                if d <= 0:
                    break
                time.sleep(d if d > 2e-3 else 0)
            handoff.put((i, srv.submit(ids[k], p, src)))

    th = threading.Thread(target=submitter)
    th.start()
    infos = [None] * n
    for _ in range(n):
        i, t = handoff.get()
        k, p, _ = queries[i]
        out = bufs[k][1 if p == 5 else 0]
        _, infos[i] = srv.wait(t, out=out)
        if keep is not None and i in keep:
            keep[i] = out.copy()
    wall = time.perf_counter() - t0
    th.join()
    bad = [x for x in infos if x["status"] != 0]
    if bad:
        raise SystemExit(f"{len(bad)} served queries failed (status {bad[0]['status']})")
    return infos, wall


def serve_summary(infos, gs=None):
    lat = np.array([(x["doneNs"] - x["submitNs"]) / 1e6 for x in infos])
    span = (max(x["doneNs"] for x in infos) - min(x["submitNs"] for x in infos)) / 1e9
    out = {"qps": len(infos) / span, "p50_ms": float(np.percentile(lat, 50)),
           "p99_ms": float(np.percentile(lat, 99)), "span_s": span,
           "mean_batch": float(np.mean([x["batchSize"] for x in infos]))}
    if gs is not None:  # p50 latency and rounds per graph and program
        cells, batches = {}, {}
        for x, l in zip(infos, lat):
            key = f"{gs[x['graph']][0]}-{PROGRAM_NAMES[x['program']]}"
            cells.setdefault(key, []).append((l, x["rounds"], (x["doneNs"] - x["admitNs"]) / 1e6))
            batches.setdefault(key, {})[(x["lane"], x["admitNs"])] = (x["doneNs"] - x["admitNs"]) / 1e6
        # lane_ms: the cell's batches' run times summed (lane time it held)
        out["cells"] = {k: {"n": len(v), "p50_ms": float(np.median([a for a, _, _ in v])),
                            "run_ms": float(np.median([c for _, _, c in v])),
                            "rounds": int(np.median([b for _, b, _ in v])),
                            "batches": len(batches[k]), "lane_ms": float(sum(batches[k].values()))}
                        for k, v in sorted(cells.items())}
    return out


def pinned_like(a):
    """A page-locked copy of the numpy array `a` (same dtype and shape)."""
    import torch
    buf = torch.empty(max(a.nbytes, 1), dtype=torch.uint8).pin_memory().numpy()
    out = buf[:a.nbytes].view(a.dtype).reshape(a.shape)
    out[...] = a
    return out


def plain_one_at_a_time(gs, local, stream, per_cell=4):
    """Mean run()+getResults() time of the plain engine per (graph, program)
    on `per_cell` seeded sources, the result of each, and the mix's
    queries/s (1 / expected time per query).  Initial values go up from, and
    results come back into, page-locked host buffers, as the served queries'
    results do."""
    import vertexapi2_gb300 as gas
    from vertexapi2_gb300 import programs as P
    rng = np.random.default_rng(SEED + 3)
    cells, results = {}, []
    for k, (name, g) in enumerate(gs):
        for prog in (1, 2, 5):
            srcs = [int(x) for x in rng.integers(0, g.n_vertices, per_cell)]
            e = gas.GASEngine(prog, device=local, stream=stream)
            times = []
            for q, s0 in enumerate(srcs):
                if prog == 1:
                    vd, act = P.bfs_init(g.n_vertices), (s0, s0 + 1)
                elif prog == 2:
                    vd, act = P.sssp_init(g.n_vertices, s0), (0, g.n_vertices)
                else:
                    vd, act = P.ppr_init(g.n_vertices, g.srcs, s0), (0, g.n_vertices)
                vd = pinned_like(vd)
                if q == 0:  # the engine borrows a page-locked result array
                    e.set_graph(g.n_vertices, pinned_like(vd), g.srcs, g.dsts,
                                g.weights if prog == 2 else None)
                else:
                    e.set_vertex_data(vd)
                e.set_active(*act)
                e.run(20 if prog == 5 else 0)   # warm
                e.set_vertex_data(vd)
                t0 = time.perf_counter()
                e.set_active(*act)
                e.run(20 if prog == 5 else 0)
                e.get_results()
                times.append(time.perf_counter() - t0)
                res = e.vertex_data["rank"].copy() if prog == 5 else e.vertex_data.copy()
                results.append((k, prog, s0, res))
            e.close()
            cells[(k, prog)] = float(np.mean(times))
    mix = dict(zip((1, 2, 5), C5_MIX))
    expected = sum(cells[(k, p)] * mix[p] / len(gs) for (k, p) in cells)
    return 1.0 / expected, cells, results


def c5_oracle_check(gs, queries, kept):
    """Served results of a sample of the mix against the oracle, at once on
    host threads: BFS/SSSP bit for bit; PPR within 1e-5 relative L1 of the
    FP64 oracle, and bit for bit with the FP32 oracle on graphs whose
    in-degrees are all <= 4096 (the served sums follow its order there)."""
    import oracle
    port = oracle.port()
    jobs = []
    for i in sorted(kept):
        k, p, s0 = queries[i]
        g = gs[k][1]
        if p == 1:
            jobs.append(lambda g=g, s0=s0: port.bfs(g.n_vertices, g.srcs, g.dsts, s0)[0])
        elif p == 2:
            jobs.append(lambda g=g, s0=s0: port.sssp(g.n_vertices, g.srcs, g.dsts, g.weights, s0)[0])
        else:
            jobs.append(lambda g=g, s0=s0: (port.ppr(g.n_vertices, g.srcs, g.dsts, s0, iters=20)[0],
                                            port.ppr(g.n_vertices, g.srcs, g.dsts, s0, iters=20,
                                                     fp64=True)[0]))
    res = in_threads(*jobs)
    exact, ppr_err = True, 0.0
    for i, r in zip(sorted(kept), res):
        if queries[i][1] == 5:
            g = gs[queries[i][0]][1]
            if np.bincount(g.dsts, minlength=g.n_vertices).max() <= 4096:
                exact &= bool(np.array_equal(kept[i], r[0]))
            ppr_err = max(ppr_err, pr_error(kept[i], r[1])["rel_l1_vs_fp64"])
        else:
            exact &= bool(np.array_equal(kept[i], r))
    return exact, ppr_err, len(jobs)


def c5_sample(queries, gs, per_cell=1, cap_edges=None):
    """Indices of the first query of every (graph, program) cell."""
    seen, out = {}, []
    for i, (k, p, _) in enumerate(queries):
        if cap_edges is not None and gs[k][1].n_edges > cap_edges:
            continue
        if seen.get((k, p), 0) < per_cell:
            seen[(k, p)] = seen.get((k, p), 0) + 1
            out.append(i)
    return out


def measure_serve_c5(args, steps, warmup, world, rank, local, with_cpu=True):
    """Serving loop (queries/s, p50/p99) vs one-at-a-time plain runs."""
    import torch
    import vertexapi2_gb300 as gas
    stream = torch.cuda.current_stream()
    gs = c5_graphs(set(args.c5_graphs.split(",")) if args.c5_graphs else None)
    srv = gas.GASServer(device=local, lanes=args.c5_lanes)
    ids = [srv.add_graph(g.n_vertices, g.srcs, g.dsts, g.weights) for _, g in gs]
    bufs = [(torch.empty(g.n_vertices, dtype=torch.int32).pin_memory().numpy(),
             torch.empty(g.n_vertices, dtype=torch.float32).pin_memory().numpy()) for _, g in gs]
    queries = query_mix(gs, C5_QUERIES, SEED)
    for w in range(max(warmup, 1)):
        serve_pass(srv, ids, gs, queries, float("inf"), bufs, SEED + w)
    barrier(world)
    torch.cuda.synchronize()
    l0 = srv.stats()["kernelLaunches"]
    steps_out = []
    kept = {i: None for i in c5_sample(queries, gs)}
    with ClockSampler(local) as clk:
        for k in range(steps):
            infos, wall = serve_pass(srv, ids, gs, queries, float("inf"), bufs, SEED + 100 + k,
                                     keep=kept if k == steps - 1 else None)
            steps_out.append((serve_summary(infos, gs if k == 0 else None), wall))
    launches = srv.stats()["kernelLaunches"] - l0
    span = allreduce_max(world, float(sum(x["span_s"] for x, _ in steps_out)))
    e2e_s = allreduce_max(world, float(sum(w for _, w in steps_out)))
    total_q = allreduce_sum(world, float(C5_QUERIES * steps))
    value = total_q / span
    e2e_value = total_q / e2e_s
    # latency under offered load below capacity
    cap = value / world
    sweep = []
    for frac in C5_SWEEP:
        qs = query_mix(gs, C5_SWEEP_QUERIES, SEED + int(frac * 1000))
        infos, wall = serve_pass(srv, ids, gs, qs, frac * cap, bufs, SEED + 7)
        sm = serve_summary(infos, gs if frac == C5_SWEEP[0] else None)
        sweep.append({"offered_qps": frac * cap, "achieved_qps": sm["qps"], "p50_ms": sm["p50_ms"],
                      "p99_ms": sm["p99_ms"], "mean_batch": sm["mean_batch"]})
        if "cells" in sm:
            sweep[-1]["cells"] = sm["cells"]
    # one query at a time through the plain engine, and parity with serving
    single_qps, cells, singles = plain_one_at_a_time(gs, local, stream.cuda_stream)
    identical, ppr_err = True, 0.0
    alone = {}
    for k, prog, s0, res in singles:
        out = bufs[k][1 if prog == 5 else 0]
        _, info = srv.wait(srv.submit(ids[k], prog, s0), out=out)
        key = f"{gs[k][0]}-{PROGRAM_NAMES[prog]}"
        alone.setdefault(key, []).append(((info["doneNs"] - info["submitNs"]) / 1e6, info["rounds"]))
        if prog == 5:
            ppr_err = max(ppr_err, pr_error(out, res)["rel_l1_vs_fp64"])
        else:
            identical &= bool(np.array_equal(out, res))
    st = srv.stats()
    srv.close()
    cpu, oracle_parity = None, None
    if rank == 0 and with_cpu:
        exact, o_err, n_checked = c5_oracle_check(gs, queries, kept)
        oracle_parity = {"vs": "oracle on the first query of every (graph, program) cell of the "
                               "last timed step (served in the full mix)",
                         "queries": n_checked, "bit_exact_vs_fp32_oracle": exact,
                         "ppr_max_rel_l1_vs_fp64": o_err, "ok": bool(exact and o_err <= 1e-5)}
        cores = os.cpu_count() or 1
        v, n, wall, kind = cpu_cells(gs, c5_cells(gs), cores)
        cpu = {"value": v, "unit": "queries/s", "cores": cores, "kind": kind,
               "sample": f"one random source per (graph, program) cell, {n} queries on {cores} "
                         f"threads in {wall:.0f} s; value = {cores} / (mix-weighted mean run() "
                         f"time); BFS/SSSP on the {kind} engine, PPR on the restatement"}
    d2h = sum(gs[k][1].n_vertices * 4 for k, _, _ in queries)
    last = steps_out[-1][0]
    return {
        "metric": "served queries/s, p50/p99 latency (vs one-at-a-time plain engine)",
        "value": value, "unit": "queries/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": 1e3 * span / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic",
        "config": workload_config("serve-c5"),
        "run": {"queries_per_step": C5_QUERIES, "lanes": args.c5_lanes, "max_batch": 256,
                "graphs": {n: [g.n_vertices, g.n_edges] for n, g in gs},
                "arrivals": "timed steps: every query of the step offered at once (capacity); "
                            "sweep: Poisson at fractions of that capacity",
                "l2": "graphs (R-MAT-22: 4.2 M vertices, 126 M edges) and query state larger than L2"},
        "latency_ms": {"p50": last["p50_ms"], "p99": last["p99_ms"], "at": "capacity (burst)"},
        "sweep": sweep,
        "mean_batch": last["mean_batch"],
        "capacity_cells": steps_out[0][0].get("cells"),
        "alone_served_ms": {k: [float(np.mean([a for a, _ in v])), int(v[0][1])]
                            for k, v in sorted(alone.items())},
        "plain_ms": {f"{gs[k][0]}-{PROGRAM_NAMES[p]}": 1e3 * t for (k, p), t in sorted(cells.items())},
        "one_at_a_time": {"value": single_qps, "unit": "queries/s",
                          "sample_queries": len(singles), "speedup": value / single_qps,
                          "results_identical_bfs_sssp": identical,
                          "ppr_max_rel_l1_vs_plain": ppr_err},
        "parity": oracle_parity,
        "server": {"batches": st["batches"], "memory_waits": st["memoryWaits"],
                   "peak_bytes": st["peakBytesInUse"]},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": 12 * C5_QUERIES,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }


def per_algo_entry(line: dict) -> dict:
    """The per_algo summary of a workload's line."""
    keep = ("value", "unit", "steps", "warmup", "ms_per_step", "dtype", "config", "run", "roofline",
            "cpu_baseline", "parity", "e2e", "gpu_launches", "clocks", "one_at_a_time", "per_set",
            "latency_ms", "sweep", "mean_batch", "plain_ms", "alone_served_ms", "server", "graph500")
    return {k: line[k] for k in keep if k in line}


def run_ours(args):
    world, rank, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    import vertexapi2_gb300 as gas
    gas.load()
    if not gas.device_supported(local):
        raise SystemExit(f"cuda:{local} is not an sm_103 device")
    with_cpu = not args.no_cpu

    def measure(name, steps, warmup):
        if name == "batch-c4":
            return measure_batch_c4(args, steps, warmup, world, rank, local, with_cpu)
        if name == "serve-c5":
            return measure_serve_c5(args, steps, warmup, world, rank, local, with_cpu)
        return measure_plain(name, steps, warmup, world, rank, local, with_cpu, args.stepwise)

    line = measure(args.workload, args.steps, args.warmup)
    if args.workload == HEADLINE and world == 1 and not args.no_per_algo and not args.stepwise:
        per = {}
        for name in PER_ALGO:
            t0 = time.perf_counter()
            per[name] = per_algo_entry(measure(name, args.steps, args.warmup))
            per[name]["bench_wall_s"] = time.perf_counter() - t0
        line["per_algo"] = per
        line["gpu_launches"] += sum(int(x.get("gpu_launches") or 0) for x in per.values())
        line["gpu_launches_note"] = ("headline steps plus every per_algo workload's timed "
                                     "steps (each entry lists its own)")
    if rank == 0:
        line["native_libraries"] = mapped_libraries()
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=HEADLINE)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline and oracle legs")
    ap.add_argument("--no-per-algo", action="store_true",
                    help="headline workload only (no per_algo block)")
    ap.add_argument("--stepwise", action="store_true",
                    help="plain workloads: drive every round from the host (gatherApply / "
                         "scatterActivate / nextIter) instead of run()")
    ap.add_argument("--rmat-scale", type=int, default=None,
                    help="smaller R-MAT scale for the R-MAT workloads (profiling captures)")
    ap.add_argument("--grid-side", type=int, default=1024,
                    help="lattice side of batch-c4 (smaller for profiling captures)")
    ap.add_argument("--c4-sets", default=None,
                    help="batch-c4: comma-separated subset of sets, e.g. grid1024-sssp")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch-c4: default launch configuration instead of the autotuner")
    ap.add_argument("--c4-delta", type=int, default=0,
                    help="batch-c4 with --no-autotune: SSSP bucket width")
    ap.add_argument("--c4-blocks", type=int, default=0,
                    help="batch-c4 with --no-autotune: CTAs per SM (0 = as many as fit)")
    ap.add_argument("--c5-lanes", type=int, default=C5_LANES,
                    help="serve-c5: batches in flight at once")
    ap.add_argument("--c5-graphs", default=None,
                    help="serve-c5: comma-separated subset of the graphs, e.g. rmat20 (profiling)")
    args = ap.parse_args()
    if args.rmat_scale:
        for k in RMAT_SCALE:
            RMAT_SCALE[k] = args.rmat_scale
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
