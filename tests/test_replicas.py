"""Replicas-only multi-GPU host logic, on CPU with gloo (world size 2):
timings reduce by maximum over ranks, the job rate counts every rank's
units, and the reference arm prints only on rank 0."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 3.5])
        rate = bench.job_rate(world, 100.0, got[0])
        q.put((rank, got, rate))
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, rate in res:
        assert got == [2.0, 10.0, 3.5]
        assert rate == pytest.approx(2 * 100.0 / 2.0)


def test_max_over_ranks_without_group_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
    assert bench.job_rate(1, 10.0, 2.0) == 5.0


def test_reference_arm_nonzero_rank_exits_silently():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
