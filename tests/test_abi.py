"""C ABI: the library loads without a GPU, exports every declared symbol and
rejects bad arguments with error codes (no compute calls)."""
import ctypes as C

import numpy as np
import pytest


def test_exports_every_header_symbol(gpu_lib):
    L = gpu_lib.lib()
    syms = gpu_lib.header_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_invalid_handles_and_arguments(gpu_lib):
    L = gpu_lib.lib()
    assert L.slrgpu_scene_destroy(12345) == -2
    assert b"invalid" in L.slrgpu_last_error()
    h = C.c_uint64()
    assert L.slrgpu_scene_create(0, C.byref(h)) == 0
    out = C.c_int()
    assert L.slrgpu_material_matte(h.value, 3, C.byref(out)) == -1          # no such spectrum
    assert L.slrgpu_spectrum_rgb(h.value, 7, 1, 1, 1, C.byref(out)) == -1   # bad spectrum type
    assert L.slrgpu_spectrum_rgb(h.value, 0, 0.5, 0.5, 0.5, C.byref(out)) == 0
    assert L.slrgpu_material_matte(h.value, out.value, C.byref(out)) == 0
    p = np.zeros((3, 3), np.float32)
    idx = np.array([[0, 1, 5]], np.uint32)                                 # index out of range
    fp = p.ctypes.data_as(C.POINTER(C.c_float))
    assert L.slrgpu_scene_add_mesh(h.value, fp, fp, fp, None, 3, idx.ctypes.data_as(C.POINTER(C.c_uint32)), 1,
                                   0) == -1
    # rendering an uncommitted scene is refused before any device work
    st = gpu_lib.Settings(8, 8, 1, 1, 0, 0, 0, 0)
    film = np.zeros(8 * 8 * 16, np.float32)
    assert L.slrgpu_render(h.value, C.byref(st), C.c_void_p(film.ctypes.data), 0, None) == -5
    assert L.slrgpu_scene_destroy(h.value) == 0


@pytest.mark.parametrize("entry", ["slrgpu_render", "slrgpu_render_noalloc"])
def test_image_size_limits_checked_before_any_device_work(gpu_lib, entry):
    """Sides above 2^20 (where rounding a 32-bit side up to the 8 x 8 sensor
    tiles would wrap to 0) and tile-padded grids above 2^31 - 1 positions are
    rejected as invalid arguments before the scene's state is looked at."""
    L = gpu_lib.lib()
    h = C.c_uint64()
    assert L.slrgpu_scene_create(0, C.byref(h)) == 0
    film = np.zeros(16, np.float32)
    fn = getattr(L, entry)
    tail = (0, None) if entry == "slrgpu_render" else (None,)
    for w, hh in ((0xFFFFFFF9, 8), (8, 0xFFFFFFFF), ((1 << 20) + 1, 1), (1 << 20, 1 << 12), (0, 8)):
        st = gpu_lib.Settings(w, hh, 1, 1, 0, 0, 0, 0)
        assert fn(h.value, C.byref(st), C.c_void_p(film.ctypes.data), *tail) == -1, (w, hh)
        assert b"width" in L.slrgpu_last_error() or b"too large" in L.slrgpu_last_error()
    st = gpu_lib.Settings(8, 8, 1, 1, 0, 0, 0, 0)
    assert fn(h.value, C.byref(st), C.c_void_p(film.ctypes.data), *tail) == -5   # valid size: the scene state is next
    assert L.slrgpu_scene_destroy(h.value) == 0


def test_host_build_of_empty_scene(gpu_lib):
    from slr_gb300.scene_desc import SceneDesc
    s = gpu_lib.Scene(SceneDesc(), host_only=True)
    assert s.bvh_stats.num_triangles == 0


def test_density_grid_file_round_trip(tmp_path, gpu_lib):
    """The reference's raw density-grid format: written and read back by the
    Python helpers, accepted by slrgpu_medium_density_grid_file (host side
    only), and a truncated file is rejected."""
    import ctypes as C
    from slr_gb300.scene_desc import read_density_grid, write_density_grid
    rng = np.random.default_rng(0)
    d = rng.random((5, 4, 3)).astype(np.float32)
    path = str(tmp_path / "grid.raw")
    write_density_grid(path, d)
    assert np.array_equal(read_density_grid(path), d)
    raw = open(path, "rb").read()
    assert np.frombuffer(raw[:12], np.uint32).tolist() == [3, 4, 5]
    L = gpu_lib.lib()
    h = C.c_uint64()
    assert L.slrgpu_scene_create(0, C.byref(h)) == 0                      # host-only scene
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    vals = np.array([2.0, 2.0], np.float32)
    sid = C.c_int()
    assert L.slrgpu_spectrum_regular(h.value, 360.0, 830.0, fp(vals), 2, C.byref(sid)) == 0
    lo = np.zeros(3, np.float32)
    hi = np.ones(3, np.float32)
    short = str(tmp_path / "short.raw")
    open(short, "wb").write(raw[:-4])
    assert L.slrgpu_medium_density_grid_file(h.value, short.encode(), fp(lo), fp(hi), sid.value, sid.value, 0.3) == -1
    assert b"malformed" in L.slrgpu_last_error()
    assert L.slrgpu_medium_density_grid_file(h.value, path.encode(), fp(lo), fp(hi), sid.value, sid.value, 0.3) == 0
    assert L.slrgpu_scene_destroy(h.value) == 0


def test_fault_injection_sites(gpu_lib):
    """The host-side fault-injection hook takes the two server sites and
    refuses others (no device work: the counters are armed and cleared)."""
    L = gpu_lib.lib()
    assert L.slrgpu_debug_inject_fault(7, 1) == -1
    for site in (gpu_lib.FAULT_SERVER_FILM_ALLOC, gpu_lib.FAULT_SERVER_WAVE_LAUNCH):
        assert L.slrgpu_debug_inject_fault(site, 2) == 0
        assert L.slrgpu_debug_inject_fault(site, 0) == 0
