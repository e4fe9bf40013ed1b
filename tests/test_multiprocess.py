"""The N > 1 host logic of bench.py on CPU: replicas (the path does not
shard; each rank renders its own copy), so the only exchange is the max of
the ranks' timed regions, checked here with two gloo ranks; and the
reference arm, which runs on rank 0 alone while the other ranks exit."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    ms = bench.slowest_rank_ms(10.0 + 5.0 * rank, world, "cpu")
    out.put((rank, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 15.0, 1: 15.0}


def test_reference_arm_runs_on_rank_zero_only():
    base = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
            "--warmup", "3"]
    env1 = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r1 = subprocess.run(base, env=env1, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    env0 = dict(os.environ, RANK="0", WORLD_SIZE="2", LOCAL_RANK="0")
    r0 = subprocess.run(base, env=env0, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r0.returncode == 0, r0.stderr
    line = json.loads(r0.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
