"""Image parity on the GPU against the reference renderer.

Per pixel and film bin, the GPU's Monte Carlo mean agrees with the
reference's within 3 standard errors (expected exceedance 0.27 % per bin; the
limit allows for standard errors that are themselves estimated from a finite
number of batches), and the per-batch image sums agree within 4 standard
errors.  The reference statistics come from one-thread reference renders
(tests/image_cases.py), so every verdict is a fixed function of fixed seeds.
"""
import numpy as np
import pytest

from slr_gb300 import scenes
from tests import image_cases as IC

pytestmark = pytest.mark.gpu

PT_CASES = ["box_32", "ragged_box", "ragged_ggx_ibl", "ggx_ibl_24", "volumetric_20", "thin_lens", "equirect"]


def dropped_rates_agree(g, r, case):
    """Both renderers drop the same kind of non-finite samples (next-event
    estimation from a vertex on the light toward a coplanar light point in
    the volumetric tracer): the dropped fractions agree within 4 standard
    errors of a two-sample binomial comparison."""
    grid = ((case.w + 7) // 8 * 8) * ((case.h + 7) // 8 * 8)     # sample positions, whole 8 x 8 tiles
    nr, ng = r["batches"] * grid * case.spp, g["batches"] * grid * case.spp
    pr, pg = r["dropped"] / nr, g["dropped"] / ng
    pooled = (r["dropped"] + g["dropped"]) / (nr + ng)
    se = np.sqrt(pooled * (1 - pooled) * (1 / nr + 1 / ng)) + 1e-12
    assert abs(pr - pg) < 4 * se, (pr, pg, se)


@pytest.mark.parametrize("name", PT_CASES)
def test_image_matches_reference(gpu_lib, name):
    """The box (32^2); ragged images whose sides are not multiples of the
    8 x 8 sensor tiles, where the last column and row also collect the
    overhanging tile positions (ImageSensor.cpp:125-130, PTRenderer.cpp:104-110),
    with and without the image-based environment and its 5e4 sun; GGX
    conductors and dielectrics under the environment; the fBm medium
    (VolumetricPTRenderer); the thin-lens and equirectangular cameras
    (PerspectiveCamera.cpp:31-83, EquirectangularCamera.cpp:25-69)."""
    case = IC.CASES[name]
    r = IC.load_reference(case)
    g = IC.gpu_stats(gpu_lib, case)
    rep = IC.parity_report(g, r, ragged=name.startswith("ragged"))
    IC.assert_parity(rep, case.frac_limit, name)
    assert g["mean"].sum() > 0
    dropped_rates_agree(g, r, case)
    if name in ("box_32", "ragged_box"):
        # Same estimator, same noise: the summed per-bin variance of a batch
        # mean matches the reference's, so equal sample counts give equal
        # RMSE (the throughput ratios compare at matched RMSE).
        assert 0.75 < rep["var_ratio"] < 1.33, rep


def test_render_settings_validation(gpu_lib):
    desc = scenes.box_scene(8, 8)
    s = gpu_lib.Scene(desc)
    with pytest.raises(gpu_lib.SlrGpuError):
        s.render(0, 8, 1, 1)
    film, st = s.render(8, 8, 3, 0)          # max depth 0: camera-visible emission only
    assert st.shadow_rays == 0 and np.isfinite(film).all()


def test_renderer_interface(gpu_lib):
    desc = scenes.box_scene(16, 16)
    scene = gpu_lib.Scene(desc)
    renderer = gpu_lib.PathTracingRenderer(spp=4, max_depth=8)
    settings = gpu_lib.RenderSettings(ImageWidth=16, ImageHeight=16, RNGSeed=3)
    film = renderer.render(scene, settings)
    assert film.shape == (16, 16, 16) and film.sum() > 0
    assert renderer.last_stats.path_samples == 16 * 16 * 4


def test_volumetric_film_is_reproducible(gpu_lib):
    """The transmittance walks are handed to lanes in whatever order the
    warps draw them from a shared counter, but each (shadow ray, wavelength)
    draws its own random stream and adds to its own path, and paths reach the
    film in sample order: the same seed gives the same film bit for bit, in
    one wave or in several."""
    desc = scenes.medium_box_scene(24, 24, grid=32)
    s = gpu_lib.Scene(desc)
    a, _ = s.render(24, 24, 8, 16, seed=11, volumetric=True)
    b, _ = s.render(24, 24, 8, 16, seed=11, volumetric=True)
    c, _ = s.render(24, 24, 8, 16, seed=11, volumetric=True, samples_per_wave=3)
    assert np.array_equal(a, b)
    assert np.array_equal(a, c)
    assert a.sum() > 0


def test_sharded_render_sums_to_whole(gpu_lib):
    """Three ranks' sample ranges (slr_gb300/replicas.py) rendered with
    sample_base sum to the unsharded film: the same samples, summed in a
    different grouping (relative difference at float rounding level)."""
    from slr_gb300.replicas import render_shard
    s = gpu_lib.Scene(scenes.box_scene(32, 32))
    whole, _ = s.render(32, 32, 16, 8, seed=5)
    parts = [render_shard(s, 32, 32, 16, 8, seed=5, world=3, rank=r)[0] for r in range(3)]
    np.testing.assert_allclose(sum(parts), whole, rtol=2e-5, atol=1e-6)
    assert not np.array_equal(parts[0], parts[1])


def test_degenerate_scenes(gpu_lib):
    """A scene of only an environment (no triangles) renders the environment;
    a closed scene without emitters renders exactly black; a 1x1 image and a
    max depth of 0 work."""
    from slr_gb300.scene_desc import SceneDesc
    env_only = SceneDesc()
    env_only.environment = scenes.lognormal_environment(32, 16, 3)
    env_only.camera = scenes.box_scene(8, 8).camera
    film, st = gpu_lib.Scene(env_only).render(8, 8, 4, 5, seed=1)
    assert np.isfinite(film).all() and film.min() >= 0 and film.sum() > 0 and st.dropped_samples == 0
    dark = scenes.box_scene(8, 8)
    light_mat = dark.meshes[-1].material
    dark.materials[light_mat] = dark.materials[dark.meshes[0].material]     # the light becomes a white wall
    film, _ = gpu_lib.Scene(dark).render(8, 8, 4, 5, seed=1)
    assert np.all(film == 0)
    film, _ = gpu_lib.Scene(scenes.box_scene(1, 1)).render(1, 1, 16, 0, seed=2)
    assert film.shape == (1, 1, 16) and np.isfinite(film).all()


@pytest.mark.parametrize("volumetric", [False, True])
def test_checkpointed_render_equals_one_call(gpu_lib, tmp_path, volumetric):
    """A frame rendered over sample ranges, its compensated film state saved
    to a file and loaded back between the calls (slrgpu_render_continue),
    equals the one-call film bit for bit, with the same dropped count."""
    desc = scenes.medium_box_scene(24, 16, grid=16) if volumetric else scenes.box_scene(24, 16)
    s = gpu_lib.Scene(desc)
    whole, st = s.render(24, 16, 13, 8, seed=21, volumetric=volumetric)
    ck = gpu_lib.FilmCheckpoint(24, 16, 8, seed=21, volumetric=volumetric)
    for spp in (5, 1, 7):
        s.render_continue(ck, spp)
        path = str(tmp_path / "ck.npz")
        ck.save(path)
        ck = gpu_lib.FilmCheckpoint.load(path)
    assert ck.next_sample == 13 and ck.dropped == st.dropped_samples
    np.testing.assert_array_equal(ck.film().view(np.uint32), whole.view(np.uint32))
    with pytest.raises(gpu_lib.SlrGpuError):
        s.render_continue(ck, 1, flags=gpu_lib.FLAG_BPT)


def test_queue_counts_account_for_every_ray(gpu_lib):
    """The per-bounce queue counters of a one-wave render
    (slrgpu_context_queue_counts, 11 columns per bounce) add up to the
    render's ray statistics: extension queues (column 7) to the extension
    rays, shadow rays (column 8) to the shadow rays.  At the first bounce,
    where no roulette is drawn, every extension ray lands in one shading
    class (columns 0-5); past it, the paths the roulette at the hit ended are
    in no class, and a bounce's extension rays never exceed the surface
    paths the previous bounce shaded."""
    ctx = gpu_lib.Context(0)
    s = gpu_lib.Scene(scenes.glossy_box_scene(32, 32), context=ctx)
    try:
        _, st = s.render(32, 32, 16, 8, seed=3)
        q = ctx.queue_counts().astype(np.int64)
        assert q.shape[1] == 11 and q.shape[0] >= 10
        assert q[0, 7] == 32 * 32 * 16
        assert q[:, 7].sum() == st.extension_rays
        assert q[:, 8].sum() == st.shadow_rays
        assert q[0, 0:6].sum() == q[0, 7]
        for b in range(1, q.shape[0]):
            assert q[b, 0:6].sum() <= q[b, 7]
            assert q[b, 7] <= q[b - 1, 0:5].sum()
            assert q[b, 8] <= q[b, 0:5].sum()
        assert q[9:, :].sum() == 0          # bounces past max depth 8
        assert (q[:, 9:11] == 0).all()      # the volumetric columns of a surface render
    finally:
        s.close()
        ctx.close()
