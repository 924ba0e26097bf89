"""bench.py's multi-rank path on CPU (gloo, world size 2).

With N GPUs the bench runs one independent replica per rank (no data-path
collective): the host-side reductions combine the ranks' timings (max) and
work (sum), and the reference arm runs on rank 0 alone while the other
ranks exit without work.  Both are exercised here without a GPU.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    mx = bench.allreduce_max(w, 1.5 + r)
    sm = bench.allreduce_sum(w, 1.0 + r)
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump({"world": w, "max": mx, "sum": sm}, f)
    dist.destroy_process_group()


def test_rank_reductions_gloo(tmp_path):
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        got = json.load(open(tmp_path / f"rank{r}.json"))
        assert got == {"world": 2, "max": 2.5, "sum": 3.0}


def test_reference_arm_on_two_ranks_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--workload", "bfs-rmat16", "--steps", "1", "--warmup", "0"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [x for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    # the reference arm builds its graphs with the oracle's generators and
    # never maps the product library
    assert not any("libgas_gb300" in p for p in d["native_libraries"]), d["native_libraries"]
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.workload_config("bfs-rmat16", bench.make_workload(
        "bfs-rmat16", source="oracle")["g"])
