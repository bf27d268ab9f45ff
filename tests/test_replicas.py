"""Sharding a render across ranks (slr_gb300/replicas.py), on CPU with the
gloo backend and two processes: the sample ranges are disjoint and cover
every spp, partial films sum to the whole, and timing takes the slowest
rank.  (The GPU side of a shard is slrgpu_render with a sample_base; its
equality with an unsharded render is checked in test_gpu_render.py.)"""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from slr_gb300.replicas import sample_range


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_sample_ranges_partition(world):
    for spp in (1, 2, 7, 16, 64, 1000):
        covered = []
        for r in range(world):
            first, count = sample_range(spp, world, r)
            covered += list(range(first, first + count))
        assert covered == list(range(spp))


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from slr_gb300.replicas import max_over_ranks, reduce_films, sample_range
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        spp = 10
        first, count = sample_range(spp, world, rank)
        # a "film" whose pixel values identify the samples each rank rendered
        film = np.zeros((3, 5, 16), np.float32)
        for s in range(first, first + count):
            film += (s + 1)
        total = reduce_films(film)
        slowest = max_over_ranks(0.5 + rank)
        out.put((rank, float(total.numpy()[0, 0, 0]), slowest))
    finally:
        dist.destroy_process_group()


def test_films_sum_and_timing_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, slowest in res:
        assert total == sum(range(1, 11))          # every sample exactly once
        assert slowest == 1.5
