"""Serving loop under cancellation, deadlines, budget pressure and injected
faults.  Every fault is made on the host: a cancelled or expired request, a
film allocation or wave launch that the server is told has failed
(slrgpu_debug_inject_fault), a corrupted mesh or a destroyed scene; nothing
faults, traps or hangs the GPU.  After each fault the server goes on serving,
and the films of the other requests still equal their standalone renders."""
import time

import numpy as np
import pytest

from slr_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def box(gpu_lib):
    return gpu_lib.Scene(scenes.box_scene(64, 64), context=gpu_lib.default_context())


def _server(gpu_lib, **kw):
    kw.setdefault("mode", gpu_lib.SERVER_BATCHED)
    kw.setdefault("paths_per_slot", 1 << 14)
    kw.setdefault("max_depth", 16)
    return gpu_lib.Server(gpu_lib.default_context(), **kw)


def _expect_status(gpu_lib, srv, rid, code):
    with pytest.raises(gpu_lib.SlrGpuError) as e:
        srv.wait(rid, timeout=60)
    assert e.value.code == code, e.value


def test_cancel_queued_and_running_requests(gpu_lib, box):
    """One slot: a long request runs (64x64 at 65536 spp: 16384 waves of 4
    samples), two more queue behind it.  Cancelling the queued one ends it
    at once; cancelling the running one ends it after its wave in flight;
    the third request is served and equals its standalone render."""
    srv = _server(gpu_lib, slots=1)
    try:
        long_id = srv.submit(box, 64, 64, 1 << 16, 8, seed=1)
        queued_id = srv.submit(box, 64, 64, 4096, 8, seed=2)
        last_id = srv.submit(box, 16, 16, 8, 8, seed=3)
        ref, _ = box.render(16, 16, 8, 8, seed=3)
        srv.cancel(queued_id)
        assert srv.poll(queued_id).status == gpu_lib.ERR_CANCELLED
        while srv.poll(long_id).spp_done == 0:
            time.sleep(0.001)
        srv.cancel(long_id)
        _expect_status(gpu_lib, srv, long_id, gpu_lib.ERR_CANCELLED)
        _expect_status(gpu_lib, srv, queued_id, gpu_lib.ERR_CANCELLED)
        film, info = srv.wait(last_id, timeout=60)
        assert info.status == gpu_lib.REQUEST_DONE and np.array_equal(film, ref)
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.cancel(last_id)                 # released by wait: unknown now
    finally:
        srv.close()


def test_deadline_cancels_late_requests(gpu_lib, box):
    """A request that cannot finish within its deadline ends with
    SLRGPU_ERR_TIMEOUT well before it would have finished; a request with a
    generous deadline finishes normally."""
    srv = _server(gpu_lib, slots=1)
    try:
        late = srv.submit(box, 64, 64, 1 << 16, 8, seed=4)     # minutes of work in 4-sample waves
        srv.set_deadline(late, 0.05)
        ok = srv.submit(box, 16, 16, 4, 8, seed=5)
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.set_deadline(ok, -1.0)                          # negative
        srv.set_deadline(ok, 120.0)
        t0 = time.time()
        _expect_status(gpu_lib, srv, late, gpu_lib.ERR_TIMEOUT)
        assert time.time() - t0 < 30
        film, info = srv.wait(ok, timeout=60)
        assert np.array_equal(film, box.render(16, 16, 4, 8, seed=5)[0])
        with pytest.raises(gpu_lib.SlrGpuError):
            srv.set_deadline(12345, 1.0)                        # unknown request
    finally:
        srv.close()


def test_injected_film_allocation_failure(gpu_lib, box):
    srv = _server(gpu_lib)
    try:
        gpu_lib.inject_fault(gpu_lib.FAULT_SERVER_FILM_ALLOC, 1)
        bad = srv.submit(box, 32, 32, 4, 8, seed=6)
        good = srv.submit(box, 32, 32, 4, 8, seed=7)
        _expect_status(gpu_lib, srv, bad, -4)                   # SLRGPU_ERR_OUT_OF_MEMORY
        film, _ = srv.wait(good, timeout=60)
        assert np.array_equal(film, box.render(32, 32, 4, 8, seed=7)[0])
    finally:
        gpu_lib.inject_fault(gpu_lib.FAULT_SERVER_FILM_ALLOC, 0)
        srv.close()


def test_injected_wave_launch_failure(gpu_lib, box):
    """The requests of a wave whose launch fails end with SLRGPU_ERR_CUDA;
    the server launches the next waves normally."""
    srv = _server(gpu_lib, slots=1)
    try:
        gpu_lib.inject_fault(gpu_lib.FAULT_SERVER_WAVE_LAUNCH, 1)
        bad = srv.submit(box, 32, 32, 4, 8, seed=8)
        _expect_status(gpu_lib, srv, bad, -3)
        good = srv.submit(box, 32, 32, 4, 8, seed=9)
        film, _ = srv.wait(good, timeout=60)
        assert np.array_equal(film, box.render(32, 32, 4, 8, seed=9)[0])
    finally:
        gpu_lib.inject_fault(gpu_lib.FAULT_SERVER_WAVE_LAUNCH, 0)
        srv.close()


def test_budget_counts_slots_scenes_and_films(gpu_lib, box):
    """bytes_in_use starts at the path-state slots, grows by the scene and
    the film while a request is admitted and returns once it is released;
    a budget below the slots refuses to create the server."""
    srv = _server(gpu_lib, slots=2)
    try:
        slots = srv.stats().bytes_in_use
        assert slots >= 2 * (1 << 14) * 256
        scene_bytes = box.reupload()
        film_bytes = 3 * 64 * 64 * 16 * 4
        rid = srv.submit(box, 64, 64, 1 << 16, 8, seed=10)
        while srv.poll(rid).status == gpu_lib.REQUEST_QUEUED:
            time.sleep(0.001)
        assert srv.stats().bytes_in_use == slots + scene_bytes + film_bytes
        srv.cancel(rid)
        _expect_status(gpu_lib, srv, rid, gpu_lib.ERR_CANCELLED)
        assert srv.stats().bytes_in_use == slots
    finally:
        srv.close()
    with pytest.raises(gpu_lib.SlrGpuError):
        _server(gpu_lib, slots=2, hbm_budget_bytes=1 << 20)
    probe = _server(gpu_lib, slots=1)
    one_slot = probe.stats().bytes_in_use
    probe.close()
    small = _server(gpu_lib, slots=1, hbm_budget_bytes=one_slot + scene_bytes + 32 * 32 * 16 * 12)
    try:
        ok = small.submit(box, 32, 32, 1, 8)                  # a 32x32 film fits exactly
        small.wait(ok, timeout=60)
        with pytest.raises(gpu_lib.SlrGpuError):
            small.submit(box, 64, 64, 1, 8)                   # its film can never fit the budget
    finally:
        small.close()


def test_corrupted_inputs_are_refused(gpu_lib, box):
    """A mesh with non-finite positions is refused when it is added; a
    destroyed scene cannot take requests; a scene with unfinished requests
    cannot be destroyed."""
    bad = scenes.box_scene(8, 8)
    bad.meshes[0].positions = bad.meshes[0].positions.copy()
    bad.meshes[0].positions[1, 1] = np.nan
    with pytest.raises(gpu_lib.SlrGpuError):
        gpu_lib.Scene(bad)
    gone = gpu_lib.Scene(scenes.box_scene(8, 8))
    handle = gone.handle
    gone.close()
    srv = _server(gpu_lib, slots=1)
    try:
        import ctypes as C
        s = gpu_lib.Settings(8, 8, 1, 4, 0, 0, 0, 0)
        rid = C.c_uint64()
        assert gpu_lib.lib().slrgpu_server_submit(srv.handle, handle, C.byref(s), C.byref(rid)) == -2
        busy = gpu_lib.Scene(scenes.box_scene(64, 64))
        long_id = srv.submit(busy, 64, 64, 1 << 16, 8, seed=11)
        assert gpu_lib.lib().slrgpu_scene_destroy(busy.handle) == -6     # SLRGPU_ERR_STATE
        srv.cancel(long_id)
        _expect_status(gpu_lib, srv, long_id, gpu_lib.ERR_CANCELLED)
        busy.close()
    finally:
        srv.close()
