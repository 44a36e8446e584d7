"""The multi-GPU bench path on CPU: N replicas over gloo (world size 2).

The ranks are independent replicas; their only communication is the barrier
around the timed region and the max of the per-rank times, which these tests
exercise with the bench's own helpers, plus the reference arm launched the
way the N-GPU bench is (one process per rank, rank 0 alone runs and prints).
"""
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


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank          # the slower rank sets the job's time
    got = bench.max_over_ranks(ms)
    dist.barrier()
    q.put((rank, got, bench.job_value(world, 1000.0, got * 1e-3)))
    dist.destroy_process_group()


def test_max_over_ranks_and_job_value_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value in res:
        assert got == 15.0                       # max over the two ranks
        assert value == pytest.approx(2 * 1000.0 / 0.015)  # both ranks' units over the slowest time


def test_single_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_value(1, 10.0, 2.0) == 5.0


def test_reference_arm_two_ranks_prints_once():
    """`bench.py --impl reference` under torch.distributed.run with two ranks:
    rank 0 times the CPU reference and prints one JSON line; rank 1 exits 0
    without output.  (The FF workload's CPU sample keeps it short.)"""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--workload", "ff"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
