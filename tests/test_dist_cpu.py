"""CPU test of the multi-process path of bench.py (replicas only: one universe per GPU,
no collective on the data path).  Two gloo ranks check the barrier and the max-over-ranks
timing that turns per-rank step times into the whole-job value, and that the reference
arm runs on rank 0 only."""

import os
import socket
import sys

import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_env()
        assert (w, r, local) == (world, rank, rank)
        bench.barrier(world)
        slowest = bench.allreduce_max(1.0 + 0.5 * rank, world, 'cpu')
        # value = all ranks' interactions / the slowest rank's time
        n = 1024
        value = world * n * n / (slowest * 1e-3)
        q.put((rank, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res[0][1] == res[1][1] == 1.5
    assert res[0][2] == res[1][2] == 2 * 1024 * 1024 / 1.5e-3


def test_reference_arm_is_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv('RANK', '1')
    monkeypatch.setenv('WORLD_SIZE', '2')

    class A:
        n = 64
        steps = 1
        cpu_seconds = 0.01
        gpus = 2
        warmup = 3
    assert bench.run_reference(A()) == 0   # returns at once, prints nothing
