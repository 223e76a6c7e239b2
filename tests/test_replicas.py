"""Multi-GPU host logic on CPU: sharding of independent configurations and
the max-over-ranks job timing, run as two gloo ranks."""

import os
import socket

import pytest

from chimes_calculator_gb300.replicas import shard_bounds, shard_by_atoms


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                a, b = shard_bounds(n, r, world)
                seen.extend(range(a, b))
                assert b - a in (n // world, n // world + 1)
            assert seen == list(range(n))


def test_shard_by_atoms_balances():
    counts = [8, 512, 33, 200, 9, 300, 64, 128, 17, 450]
    parts = [shard_by_atoms(counts, r, 3) for r in range(3)]
    assert sorted(i for p in parts for i in p) == list(range(len(counts)))
    loads = [sum(counts[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(counts)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from chimes_calculator_gb300.replicas import job_time_and_throughput
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = job_time_and_throughput(10.0 + 5.0 * rank, 1024.0, steps=4)
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_job_time_is_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    for r in range(world):
        ms, value = out[r]
        assert ms == pytest.approx(15.0)
        assert value == pytest.approx(2 * 1024.0 * 4 / 15e-3)
