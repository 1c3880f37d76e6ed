"""Replica sharding across ranks, exercised as world-size-2 gloo process groups on CPU."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from pyturb_gb300 import replicas


def test_shard_covers_and_is_disjoint():
    for total in (0, 1, 7, 64, 4096):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                s, c = replicas.shard(total, r, world)
                seen.extend(range(s, s + c))
            assert seen == list(range(total))
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_time_windows_never_overlap():
    a = replicas.time_window(0, 3, 2000, 1e-3)
    b = replicas.time_window(1, 0, 2000, 1e-3)
    assert a.max() < b.min()
    with pytest.raises(ValueError):
        replicas.time_window(0, 600, 2000, 1e-3)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        start, count = replicas.shard(4096, rank, world)
        seed = replicas.rank_seed(1234, rank, world)
        times = replicas.time_window(rank, 1, 2000, 1e-3)
        # gather every rank's share, seed and window
        info = torch.tensor([start, count, seed % (2**31), times[0] * 1e6, times[-1] * 1e6],
                            dtype=torch.float64)
        gathered = [torch.zeros_like(info) for _ in range(world)]
        dist.all_gather(gathered, info)
        slowest = replicas.max_over_ranks(0.5 + rank, dist)
        out[rank] = ([g.tolist() for g in gathered], slowest)
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_replicas():
    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world,
                       start_method="spawn")
    for rank in range(world):
        gathered, slowest = out[rank]
        assert slowest == pytest.approx(0.5 + world - 1)
        starts = [int(g[0]) for g in gathered]
        counts = [int(g[1]) for g in gathered]
        assert starts == [0, 2048] and counts == [2048, 2048]
        assert gathered[0][2] != gathered[1][2]  # independent streams
        assert gathered[0][4] < gathered[1][3]   # disjoint time windows
