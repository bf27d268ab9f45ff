"""Serving loop (slrgpu_server_*): continuous batching of render requests of
several scenes, resolutions, sample counts and both integrators.

Each request's film must be bit-identical to a standalone slrgpu_render with
the same settings, in the plain and in the batched mode: its random numbers
depend only on (seed, sample, pixel) and its samples are accumulated in
order, whichever waves they travel in.  The slot size here is small (64 Ki
paths), so requests are split over many waves and packed together with
others."""
import time

import numpy as np
import pytest

from slr_gb300 import scenes

pytestmark = pytest.mark.gpu

# (scene index, width, height, spp, max depth, seed, volumetric)
REQUESTS = [
    (0, 64, 64, 16, 8, 1, False),
    (1, 48, 48, 4, 8, 2, False),
    (0, 21, 13, 64, 8, 3, False),      # ragged: overhanging 8x8 tiles
    (2, 32, 32, 8, 8, 4, True),        # volumetric
    (1, 128, 64, 4, 8, 5, False),
    (0, 64, 64, 4, 3, 6, False),       # another max depth: its own waves
    (2, 20, 20, 16, 8, 7, True),
    (1, 48, 48, 16, 8, 8, False),
]


@pytest.fixture(scope="module")
def served_scenes(gpu_lib):
    ctx = gpu_lib.default_context()
    box = gpu_lib.Scene(scenes.box_scene(64, 64), context=ctx)
    ggx = gpu_lib.Scene(scenes.heightfield_scene(grid=32, spheres=4, sphere_freq=4, env_size=(32, 16), width=48,
                                                 height=48), context=ctx)
    vol = gpu_lib.Scene(scenes.medium_box_scene(32, 32, grid=16), context=ctx)
    return ctx, [box, ggx, vol]


@pytest.fixture(scope="module")
def standalone(served_scenes):
    _, scs = served_scenes
    out = []
    for i, w, h, spp, d, seed, vol in REQUESTS:
        film, _ = scs[i].render(w, h, spp, d, seed=seed, volumetric=vol)
        out.append(film)
    return out


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_served_films_equal_standalone(gpu_lib, served_scenes, standalone, mode):
    ctx, scs = served_scenes
    m = gpu_lib.SERVER_PLAIN if mode == "plain" else gpu_lib.SERVER_BATCHED
    srv = gpu_lib.Server(ctx, mode=m, paths_per_slot=1 << 16, max_depth=16)
    try:
        ids = [srv.submit(scs[i], w, h, spp, d, seed=seed, volumetric=vol)
               for i, w, h, spp, d, seed, vol in REQUESTS]
        for rid, ref, req in zip(ids, standalone, REQUESTS):
            film, info = srv.wait(rid, timeout=120)
            assert info.status == gpu_lib.REQUEST_DONE
            assert info.spp_done == req[3]
            assert np.array_equal(film, ref), f"request {req} differs from its standalone render"
            assert info.submit_seconds <= info.start_seconds <= info.done_seconds
        st = srv.stats()
        assert st.requests_done == len(REQUESTS) and st.queued == 0 and st.active == 0
    finally:
        srv.close()


def test_queued_requests_share_waves(gpu_lib, served_scenes):
    """Requests that queue up behind a long one are packed into shared
    waves: one slot, a request that fills it for 128 waves, then six small
    requests of the same scene submitted at once."""
    ctx, scs = served_scenes
    srv = gpu_lib.Server(ctx, mode=gpu_lib.SERVER_BATCHED, slots=1, paths_per_slot=1 << 16, max_depth=16)
    try:
        big = srv.submit(scs[0], 64, 64, 2048, 8, seed=1)          # 16 samples of 4096 positions per wave
        small = [srv.submit(scs[0], 16, 16, 4, 8, seed=10 + k) for k in range(6)]
        refs = [scs[0].render(16, 16, 4, 8, seed=10 + k)[0] for k in range(6)]
        srv.wait(big, timeout=300)
        for rid, ref in zip(small, refs):
            film, _ = srv.wait(rid, timeout=60)
            assert np.array_equal(film, ref)
        waves = srv.stats().waves
        assert waves < 128 + 6, waves
    finally:
        srv.close()


def test_requests_arriving_while_others_run(gpu_lib, served_scenes, standalone):
    """Continuous batching: later submissions join while earlier requests are
    on the GPU; every film still equals its standalone render."""
    ctx, scs = served_scenes
    srv = gpu_lib.Server(ctx, mode=gpu_lib.SERVER_BATCHED, paths_per_slot=1 << 16, max_depth=16)
    try:
        ids = []
        for k, (i, w, h, spp, d, seed, vol) in enumerate(REQUESTS):
            ids.append(srv.submit(scs[i], w, h, spp, d, seed=seed, volumetric=vol))
            if k % 2 == 1:
                time.sleep(0.002)
        for rid, ref in zip(ids, standalone):
            film, info = srv.wait(rid, timeout=120)
            assert np.array_equal(film, ref)
    finally:
        srv.close()


def test_admission_respects_the_budget(gpu_lib, served_scenes, standalone):
    """A budget that holds the path-state slots, the three scenes and one
    film at a time still serves every request, in order, and what it
    charges never exceeds the budget."""
    ctx, scs = served_scenes
    probe = gpu_lib.Server(ctx, mode=gpu_lib.SERVER_BATCHED, paths_per_slot=1 << 16, max_depth=16)
    slot_bytes = probe.stats().bytes_in_use
    probe.close()
    scene_bytes = sum(sc.reupload() for sc in scs)
    biggest = max(w * h for _, w, h, *_ in REQUESTS)
    budget = slot_bytes + scene_bytes + 3 * biggest * 16 * 4   # sum + compensation + output planes of one film
    srv = gpu_lib.Server(ctx, mode=gpu_lib.SERVER_BATCHED, paths_per_slot=1 << 16, max_depth=16,
                         hbm_budget_bytes=budget)
    try:
        ids = [srv.submit(scs[i], w, h, spp, d, seed=seed, volumetric=vol)
               for i, w, h, spp, d, seed, vol in REQUESTS]
        peak = 0
        done = []
        for rid, ref in zip(ids, standalone):
            while srv.poll(rid).status not in (gpu_lib.REQUEST_DONE,) and srv.poll(rid).status >= 0:
                peak = max(peak, srv.stats().bytes_in_use)
                time.sleep(0.0005)
            film, info = srv.wait(rid, timeout=120)
            assert np.array_equal(film, ref)
            done.append(info.done_seconds)
        assert peak <= budget
    finally:
        srv.close()


def test_server_rejects_bad_requests(gpu_lib, served_scenes):
    ctx, scs = served_scenes
    srv = gpu_lib.Server(ctx, mode=gpu_lib.SERVER_BATCHED, paths_per_slot=1 << 12, max_depth=16)
    try:
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.submit(scs[0], 0, 8, 1, 4)                      # empty image
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.submit(scs[0], 8, 8, 1, 17)                     # deeper than the server allows
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.submit(scs[0], 128, 128, 1, 4)                  # one sample exceeds the slot
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.submit(scs[0], 8, 8, 1, 4, volumetric=True)     # no medium in this scene
    finally:
        srv.close()


def test_waves_share_queues_across_scenes(gpu_lib, served_scenes):
    """Requests of different scenes travel in one wave: their paths share
    the extension, shading and shadow queues, each path finding its scene in
    the wave's scene table.  One slot, requests of the box and the GGX scene
    submitted together: the waves mix the scenes, and every film still
    equals its standalone render."""
    ctx, scs = served_scenes
    srv = gpu_lib.Server(ctx, mode=gpu_lib.SERVER_BATCHED, slots=1, paths_per_slot=1 << 16, max_depth=16)
    try:
        reqs = [(0, 48, 48, 8, 8, 31), (1, 40, 24, 8, 8, 32), (0, 21, 13, 16, 8, 33), (1, 64, 64, 4, 8, 34)]
        ids = [srv.submit(scs[i], w, h, spp, d, seed=seed) for i, w, h, spp, d, seed in reqs]
        refs = [scs[i].render(w, h, spp, d, seed=seed)[0] for i, w, h, spp, d, seed in reqs]
        for rid, ref in zip(ids, refs):
            film, info = srv.wait(rid, timeout=120)
            assert info.status == gpu_lib.REQUEST_DONE
            assert np.array_equal(film, ref)
        st = srv.stats()
        assert st.mixed_scene_waves > 0, st.as_dict()
    finally:
        srv.close()
