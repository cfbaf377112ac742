"""The multi-GPU path of the benchmark is replicas only: each rank evaluates
its own batch with no data-path collective, the step time is the slowest
rank's and rank 0 alone prints. These tests run that host logic on CPU with two
gloo ranks (127.0.0.1), and the reference arm under two ranks."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_worker(rank, ws, port, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms, value = bench.replicas_value(1.0 + rank, 1000, ws, dist)
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in res:
        assert ms == 2.0                      # max over ranks
        assert value == 2 * 1000 / 2e-3       # all ranks' rows over the slowest time


def test_single_rank_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replicas_value(4.0, 500, 1) == (4.0, 500 / 4e-3)


def test_reference_arm_prints_once_under_two_ranks():
    env = dict(os.environ, PGX_REFERENCE_ROOT=os.environ.get("PGX_REFERENCE_ROOT", "/nonexistent"))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
