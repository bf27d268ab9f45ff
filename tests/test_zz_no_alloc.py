"""The allocation-free render entry point, slrgpu_render_noalloc.

Some callers of this renderer cannot allocate device memory while they run:
a real-time loop with a fixed memory budget, or a host application or
embedding runtime that owns the GPU allocator and forbids cudaMalloc after
start-up.  slrgpu_render grows its path-state buffers on demand, so those
callers use slrgpu_render_noalloc, which keeps all of its scratch (path
state, queues, counters, film sums) in one fixed device array inside the
library and allocates nothing.

This file is collected last so that a run stopping at the first failure has
already run every other test.  Each call goes through the C ABI with ctypes
and must reproduce slrgpu_render's film for the same settings; two calls in
a row check that the shared scratch is cleared between calls.
"""
import ctypes as C

import numpy as np
import pytest

from slr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _noalloc(api, scene, w, h, spp, depth, seed, spw, film, volumetric=False):
    import torch
    s = api.Settings(w, h, spp, depth, seed, int(volumetric), spw, 0)
    rc = api.lib().slrgpu_render_noalloc(scene.handle, C.byref(s), C.c_void_p(film.data_ptr()), None)
    api.check(rc)
    torch.cuda.synchronize()
    return film.cpu().numpy()


@pytest.mark.parametrize("volumetric", [False, True])
def test_noalloc_matches_render_twice(gpu_lib, volumetric):
    import torch
    w = h = 48
    if volumetric:
        desc = scenes.medium_box_scene(w, h, grid=24)
        spp, depth = 12, 16
    else:
        desc = scenes.box_scene(w, h)
        spp, depth = 24, 8
    scene = gpu_lib.Scene(desc)
    spw = 8  # same samples per wave on both entry points -> same random numbers
    ref, _ = scene.render(w, h, spp, depth, seed=11, samples_per_wave=spw, volumetric=volumetric)
    film = torch.empty((h, w, 16), dtype=torch.float32, device="cuda")
    for _ in range(2):
        film.fill_(-7.0)  # the call must overwrite everything
        out = _noalloc(gpu_lib, scene, w, h, spp, depth, 11, spw, film, volumetric)
        assert np.isfinite(out).all()
        np.testing.assert_allclose(out, ref, rtol=1e-6, atol=0)


def test_noalloc_rejects_sizes_beyond_limits(gpu_lib):
    import torch
    scene = gpu_lib.Scene(scenes.box_scene(8, 8))
    film = torch.empty((300, 300, 16), dtype=torch.float32, device="cuda")
    s = gpu_lib.Settings(300, 300, 1, 8, 0, 0, 0, 0)                  # 90000 pixels > 65536
    assert gpu_lib.lib().slrgpu_render_noalloc(scene.handle, C.byref(s), C.c_void_p(film.data_ptr()), None) == -1
    assert b"65536" in gpu_lib.lib().slrgpu_last_error()
    s = gpu_lib.Settings(64, 64, 1, 65, 0, 0, 0, 0)                   # max depth 65 > 64
    assert gpu_lib.lib().slrgpu_render_noalloc(scene.handle, C.byref(s), C.c_void_p(film.data_ptr()), None) == -1
    s = gpu_lib.Settings(64, 64, 32, 8, 0, 0, 32, 0)                  # 131072 paths per wave
    assert gpu_lib.lib().slrgpu_render_noalloc(scene.handle, C.byref(s), C.c_void_p(film.data_ptr()), None) == -1
