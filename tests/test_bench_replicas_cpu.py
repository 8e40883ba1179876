"""CPU: the multi-rank side of bench.py with two gloo ranks.

The hot path does not shard: N GPUs run N independent replicas of the
workload, and the whole-job rate is every rank's units over the slowest
rank's time.  These tests run the host logic of that path as two processes
on the gloo backend (no GPU): the max-over-ranks reduction and the rate, and
the reference arm under torchrun, where rank 0 alone measures and prints one
JSON line and the other rank exits 0.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) seconds for the same 1e9 units
        t = bench.max_over_ranks(float(rank + 1), world, "cpu")
        out.put((rank, t, bench.replica_rate(1e9, world, t)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time, and the job rate counts both replicas
    assert [r[1] for r in res] == [2.0, 2.0]
    assert all(abs(r[2] - 1e9) < 1e-3 for r in res)



def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.replica_rate(10.0, 1, 2.0) == 5.0


def test_reference_arm_under_torchrun_prints_once(built):
    """--impl reference at N = 2: rank 0 prints one line, both ranks exit 0."""
    port = _free_port()
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--dims", "128,96,64"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
