"""Path-level parity by tape replay.

The reference renders one sample per pixel with one thread while its random
number generator records every uniform each path draws (oracle build patch
P12), in the reference's draw order (PTRenderer.cpp:103-276).  The GPU path
tracer then traces the same pixels with those uniforms in place of its own
(slrgpu_render_replay), so each pixel of the two films holds the same path's
contribution: the images must agree pixel by pixel, not only in
distribution.  Residual differences come from FP32 rounding of functions the
two sides compute with different libraries (sqrt, sin, cos in sampling); a
path whose sampled direction then passes on the other side of an edge
diverges entirely, which the tolerance allows for a small share of pixels.

The scenes light by area lights of equal importance, for which the GPU's
alias table and the reference's CDF map a uniform to the same light; the
environment's alias table maps uniforms to directions differently from the
reference's CDF inversion (same densities), so image-lit scenes are left to
the statistical tests."""
import numpy as np
import pytest

from slr_gb300 import scenes

pytestmark = pytest.mark.gpu
STRIDE = 256


def grid_tapes(tapes, w, h):
    """The reference's k-th path, in its tile order (8 x 8 tiles row by row,
    pixels row by row within a tile), at its pixel's slot of the GPU's
    tile-padded grid."""
    gw, gh = (w + 7) // 8 * 8, (h + 7) // 8 * 8
    grid = np.full((gh * gw, STRIDE), 0.5, np.float32)
    ntx = gw // 8
    for k, t in enumerate(tapes):
        tile, within = divmod(k, 64)
        ty, tx = divmod(tile, ntx)
        ly, lx = divmod(within, 8)
        x, y = tx * 8 + lx, ty * 8 + ly
        assert len(t) <= STRIDE
        grid[y * gw + x, :len(t)] = t
    return grid


@pytest.mark.parametrize("name", ["box", "glossy_box"])
def test_replayed_paths_match_the_reference_pixel_by_pixel(gpu_lib, oracle_lib, name):
    w = h = 32
    depth = 8
    desc = scenes.box_scene(w, h) if name == "box" else scenes.glossy_box_scene(w, h)
    ref = oracle_lib.RefScene(desc)
    rfilm, tapes = ref.render_record(w, h, depth, seed=5)
    assert len(tapes) == w * h
    gfilm, _ = gpu_lib.Scene(desc).render_replay(w, h, depth, grid_tapes(tapes, w, h))
    r = rfilm.reshape(-1, 16).astype(np.float64)
    g = gfilm.reshape(-1, 16).astype(np.float64)
    exact = np.all(rfilm.reshape(-1, 16) == gfilm.reshape(-1, 16), axis=1)
    scale = np.maximum(np.abs(r).max(1), 1e-30)
    rel = np.abs(g - r).max(1) / scale
    close = rel <= 1e-4
    report = {"pixels": len(r), "bit_exact": float(exact.mean()), "within_1e-4": float(close.mean()),
              "lit_pixels": int((scale > 1e-30).sum()), "worst": float(rel.max())}
    print(name, report)
    # the same paths: nearly every pixel agrees to FP32 rounding, and the
    # image sums agree to well below the Monte Carlo noise of one sample
    assert close.mean() >= 0.98, report
    assert abs(g.sum() - r.sum()) <= 0.02 * r.sum(), report


def test_replay_rejects_unsupported_settings(gpu_lib):
    s = gpu_lib.Scene(scenes.box_scene(8, 8))
    tapes = np.full((64, STRIDE), 0.5, np.float32)
    import ctypes as C
    st = gpu_lib.Settings(8, 8, 2, 4, 0, 0, 0, 0)                 # two samples per pixel
    film = np.zeros((8, 8, 16), np.float32)
    rc = gpu_lib.lib().slrgpu_render_replay(s.handle, C.byref(st), gpu_lib._fp(tapes), gpu_lib._fp(film), None)
    assert rc == -8
