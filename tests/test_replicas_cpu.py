"""The multi-GPU bench path on CPU: two gloo ranks time a replica run as the
bench does on N GPUs (barrier, slowest rank, whole-job throughput)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from nostrum_pray_gb300 import replicas
        replicas.barrier()
        local = 1.0 + rank  # rank r took 1 + r seconds
        out[rank] = (replicas.world_size(), replicas.slowest(local), replicas.whole_job_rate(100.0, local))
        replicas.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_like_the_bench():
    world = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        ws, slow, rate = out[r]
        assert ws == world
        assert slow == 2.0                 # the slowest rank's time, on every rank
        assert rate == 100.0 * world / 2.0  # all ranks' work over that time


def test_single_process_is_its_own_job():
    from nostrum_pray_gb300 import replicas
    assert replicas.world_size() == 1
    assert replicas.slowest(3.5) == 3.5
    assert replicas.whole_job_rate(10.0, 2.0) == 5.0
