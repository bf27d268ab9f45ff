"""Sharded rendering through the real render path: two processes (gloo
ranks), each renders its sample range of the same image with render_shard
on the GPU, and the partial films are summed by reduce_films.  The ranks
share one GPU here, as independent replicas whose kernels never wait on
each other (the collective runs on host tensors); the sum must equal the
one-process render of all samples to float rounding (the partial films are
compensated sums over disjoint sample ranges)."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

W = H = 32
SPP, DEPTH, SEED = 12, 8, 21


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    from slr_gb300 import api, scenes
    from slr_gb300.replicas import reduce_films, render_shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        scene = api.Scene(scenes.box_scene(W, H))
        film, _ = render_shard(scene, W, H, SPP, DEPTH, seed=SEED, world=world, rank=rank)
        mine = film.copy()
        total = reduce_films(film)
        out.put((rank, mine, total.numpy().copy()))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_render_equals_one_render(gpu_lib):
    from slr_gb300 import scenes
    whole, _ = gpu_lib.Scene(scenes.box_scene(W, H)).render(W, H, SPP, DEPTH, seed=SEED)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29700 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=300) for _ in procs], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (_, part0, total0), (_, part1, total1) = res
    assert not np.array_equal(part0, part1) and part0.sum() > 0 and part1.sum() > 0
    np.testing.assert_array_equal(total0, total1)
    np.testing.assert_allclose(total0, whole, rtol=2e-5, atol=1e-6)
