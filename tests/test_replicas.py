"""The multi-GPU form of this path is replicas only (independent solves,
no inter-GPU traffic): the bench's rank set-up, barrier and max-over-ranks
timing over gloo on CPU (world size 2), and the reference arm under torchrun
(rank 0 alone runs and prints)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": "2",
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "VACGPU_BENCH_GLOO": "1"})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    ws, r, lr = bench.dist_setup()
    bench.barrier(ws)
    # rank 1 is the slow one: the job's time is the max over ranks
    value, el = bench.whole_job(ws, 1000.0, 2.0 if r == 1 else 1.0)
    out.put((r, ws, value, el))
    dist.destroy_process_group()


def test_whole_job_rate_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, ws, value, el in res:
        assert ws == 2 and el == 2.0 and value == 1000.0 * 2 / 2.0


def test_reference_arm_under_torchrun():
    from oracle import oracle
    oracle.build()
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--side", "12"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, VACGPU_BENCH_GLOO="1"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
