"""Bidirectional path tracing on the GPU (BPTRenderer semantics) against the
reference's own BPTRenderer run as the oracle, with the same cap on the
vertices per subpath on both sides.

The statistic is the one of the path tracer's image parity tests: per pixel
and film bin, the two Monte Carlo means agree within 3 standard errors
(expected exceedance 0.27 %; the limit allows for standard errors that are
themselves estimated), and the per-batch image sums agree within 4 standard
errors.  The light-tracing connections (t = 1) land on other pixels than the
one that started the path, so every pixel mixes both kinds of estimate."""
import os

import numpy as np
import pytest

from slr_gb300 import scenes
from test_gpu_render import check_statistical_parity

pytestmark = pytest.mark.gpu


def oracle_bpt_batches(oracle_lib, desc, w, h, spp, depth, batches, seed0, volumetric=False):
    means, dropped = [], 0
    for k in range(batches):
        ref = oracle_lib.RefScene(desc)      # one BPT render per reference sensor
        film, _ = ref.render_bpt(w, h, spp, depth, seed=seed0 + k, threads=os.cpu_count(), volumetric=volumetric)
        dropped += ref.last_dropped
        means.append(film.astype(np.float64) / spp)
    return np.stack(means), dropped


def gpu_bpt_batches(gpu_lib, desc, w, h, spp, depth, batches, seed0=70000, **kw):
    s = gpu_lib.Scene(desc)
    means, dropped = [], 0
    for k in range(batches):
        film, st = s.render(w, h, spp, depth, seed=seed0 + k, bpt=True, **kw)
        dropped += st.dropped_samples
        means.append(film.astype(np.float64) / spp)
    return np.stack(means), dropped


def compare(gm, rm, frac_limit=0.015):
    kg, kr = len(gm), len(rm)
    return check_statistical_parity(gm.mean(0), gm.var(0, ddof=1), kg, rm.mean(0), rm.var(0, ddof=1), kr,
                                    frac_limit=frac_limit, tg=gm.reshape(kg, -1).sum(1),
                                    tr=rm.reshape(kr, -1).sum(1))


def test_bpt_box_matches_reference(gpu_lib, oracle_lib):
    """Lambertian box under an area light, 20 x 12 pixels (neither side a
    multiple of the 8 x 8 sensor tiles)."""
    desc = scenes.box_scene(20, 12)
    w, h, spp, depth = 20, 12, 8, 16
    rm, rdrop = oracle_bpt_batches(oracle_lib, desc, w, h, spp, depth, 48, 500)
    gm, gdrop = gpu_bpt_batches(gpu_lib, desc, w, h, spp, depth, 192)
    compare(gm, rm)
    assert rdrop == 0 and gdrop == 0
    # the same estimator has the same noise (matched RMSE at equal spp)
    ratio = gm.var(0, ddof=1).sum() / rm.var(0, ddof=1).sum()
    assert 0.75 < ratio < 1.33, ratio


def test_bpt_every_bsdf_matches_reference(gpu_lib, oracle_lib):
    """GGX conductor and dielectric, delta glass and mirror: adjoint BSDFs,
    reverse densities, delta vertices in the MIS weights and the wavelength
    selection of dispersive refraction."""
    desc = scenes.glossy_box_scene(24, 24)
    w, h, spp, depth = 24, 24, 8, 12
    rm, _ = oracle_bpt_batches(oracle_lib, desc, w, h, spp, depth, 48, 900)
    gm, _ = gpu_bpt_batches(gpu_lib, desc, w, h, spp, depth, 192)
    compare(gm, rm, frac_limit=0.02)


@pytest.mark.parametrize("camera", ["thin_lens", "equirect"])
def test_bpt_cameras_match_reference(gpu_lib, oracle_lib, camera):
    """The lens vertex of a thin lens (a non-delta position, so t = 1 and
    t = 2 strategies both count) and of the equirectangular camera."""
    import math

    from slr_gb300.scene_desc import Camera
    from slr_gb300.scenes import look_at
    w, h = 16, 16
    desc = scenes.box_scene(w, h)
    if camera == "thin_lens":
        desc.camera = Camera("perspective", look_at((0.5, 0.5, 2.3), (0.5, 0.5, 0.0)), sensitivity=1.0,
                             aspect=1.0, fov_y=math.radians(38.0), lens_radius=0.04, img_plane_dist=1.0,
                             obj_plane_dist=2.3)
    else:
        desc.camera = Camera("equirect", look_at((0.5, 0.5, 0.8), (0.5, 0.5, 0.0)), sensitivity=1.0,
                             phi_angle=math.radians(120.0), theta_angle=math.radians(90.0))
    spp, depth = 8, 12
    rm, _ = oracle_bpt_batches(oracle_lib, desc, w, h, spp, depth, 48, 1300)
    gm, _ = gpu_bpt_batches(gpu_lib, desc, w, h, spp, depth, 192)
    compare(gm, rm, frac_limit=0.02)


def test_bpt_agrees_with_path_tracing(gpu_lib):
    """Both estimators are unbiased for the same image: on the box, BPT with
    32 vertices per subpath and PT with 64 bounces agree within their
    combined Monte Carlo error (per-batch image sums, 4 sigma)."""
    desc = scenes.box_scene(16, 16)
    s = gpu_lib.Scene(desc)
    k = 64
    tb = np.array([s.render(16, 16, 16, 32, seed=100 + i, bpt=True)[0].sum(dtype=np.float64) / 16 for i in range(k)])
    tp = np.array([s.render(16, 16, 16, 64, seed=900 + i)[0].sum(dtype=np.float64) / 16 for i in range(k)])
    z = (tb.mean() - tp.mean()) / np.sqrt(tb.var(ddof=1) / k + tp.var(ddof=1) / k)
    assert abs(z) < 4.0, (tb.mean(), tp.mean(), z)
    # the bidirectional estimate is the less noisy one on this scene
    assert tb.var(ddof=1) < tp.var(ddof=1)


def test_bpt_waves_sum_like_one(gpu_lib):
    """Splitting a render into waves (and into sample ranges) changes nothing
    but the order of the film's additions of per-path sums; the splat film
    takes atomic additions, so films agree to float rounding."""
    desc = scenes.box_scene(16, 16)
    s = gpu_lib.Scene(desc)
    a, _ = s.render(16, 16, 8, 8, seed=5, bpt=True)
    b, _ = s.render(16, 16, 8, 8, seed=5, bpt=True, samples_per_wave=2)
    c0, _ = s.render(16, 16, 3, 8, seed=5, bpt=True)
    c1, _ = s.render(16, 16, 5, 8, seed=5, bpt=True, sample_base=3)
    np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(a, c0 + c1, rtol=1e-4, atol=1e-5)


def test_bpt_environment_matches_reference(gpu_lib, oracle_lib):
    """GGX conductors and dielectrics under the image-based environment (a
    small version of the 1M-triangle scene): light subpaths that start on
    the environment at infinity (IBLEDF, world-disc origins), eye subpaths
    that escape to it, and connections toward a vertex at infinity."""
    desc = scenes.heightfield_scene(grid=24, spheres=5, sphere_freq=3, env_size=(64, 32), width=20, height=20)
    w = h = 20
    spp, depth = 8, 8
    # The 2-degree sun of radiance 5e4 makes the per-bin estimates heavy
    # tailed; enough batches keep the estimated standard errors honest
    # (with 40 reference batches the exceedance fraction ranged up to 2 %).
    rm, _ = oracle_bpt_batches(oracle_lib, desc, w, h, spp, depth, 96, 1700)
    gm, _ = gpu_bpt_batches(gpu_lib, desc, w, h, spp, depth, 384)
    compare(gm, rm, frac_limit=0.02)


def test_volumetric_bpt_matches_reference(gpu_lib, oracle_lib):
    """VolumetricBPTRenderer: the fBm medium (sigma_t max 20, albedo 0.9,
    Henyey-Greenstein g = 0.7) in the box.  Subpaths stop at scattering
    points in the medium (delta tracking with spectral ratio-tracking
    throughput), medium vertices connect through albedo x phase function,
    and every connection carries its spectral transmittance."""
    desc = scenes.medium_box_scene(16, 16, grid=16)
    w = h = 16
    spp, depth = 8, 16
    rm, _ = oracle_bpt_batches(oracle_lib, desc, w, h, spp, depth, 48, 2100, volumetric=True)
    gm, _ = gpu_bpt_batches(gpu_lib, desc, w, h, spp, depth, 192, volumetric=True)
    compare(gm, rm, frac_limit=0.02)


def test_bpt_rejects_invalid_settings(gpu_lib):
    box = gpu_lib.Scene(scenes.box_scene(8, 8))
    with pytest.raises(gpu_lib.SlrGpuError):
        box.render(8, 8, 1, 4, bpt=True, volumetric=True)  # volumetric render of a scene without medium
    with pytest.raises(gpu_lib.SlrGpuError):
        box.render(8, 8, 1, 0, bpt=True)                   # no vertex beyond the first
    with pytest.raises(gpu_lib.SlrGpuError):
        box.render(8, 8, 1, 64, bpt=True)
    film, st = box.render(8, 8, 1, 1, bpt=True)            # the smallest cap still renders
    assert np.isfinite(film).all() and film.sum() > 0
