"""Bidirectional path tracing on the GPU (BPTRenderer semantics) against the
reference's own BPTRenderer run as the oracle, with the same cap on the
vertices per subpath on both sides.

The statistic is the one of the path tracer's image parity tests: per pixel
and film bin, the two Monte Carlo means agree within 3 standard errors
(expected exceedance 0.27 %; the limit allows for standard errors that are
themselves estimated), and the per-batch image sums agree within 4 standard
errors.  The light-tracing connections (t = 1) land on other pixels than the
one that started the path, so every pixel mixes both kinds of estimate."""
import numpy as np
import pytest

from slr_gb300 import scenes
from tests import image_cases as IC

pytestmark = pytest.mark.gpu

BPT_CASES = ["bpt_box", "bpt_every_bsdf", "bpt_thin_lens", "bpt_equirect", "bpt_env", "vbpt"]


@pytest.mark.parametrize("name", BPT_CASES)
def test_bpt_image_matches_reference(gpu_lib, name):
    """bpt_box: Lambertian box under an area light, 20 x 12 pixels (neither
    side a multiple of the 8 x 8 sensor tiles).  bpt_every_bsdf: GGX
    conductor and dielectric, delta glass and mirror (adjoint BSDFs, reverse
    densities, delta vertices in the MIS weights, the wavelength selection of
    dispersive refraction).  bpt_thin_lens / bpt_equirect: the lens vertex of
    a thin lens (a non-delta position, so t = 1 and t = 2 strategies both
    count) and of the equirectangular camera.  bpt_env: GGX objects under the
    image-based environment (light subpaths that start at infinity, IBLEDF,
    world-disc origins; connections toward a vertex at infinity).  vbpt:
    VolumetricBPTRenderer in the fBm medium box (medium vertices, albedo x
    phase connections, spectral transmittance on every connection)."""
    case = IC.CASES[name]
    r = IC.load_reference(case)
    g = IC.gpu_stats(gpu_lib, case)
    rep = IC.parity_report(g, r)
    IC.assert_parity(rep, case.frac_limit, name)
    assert g["mean"].sum() > 0
    if name == "bpt_box":
        assert r["dropped"] == 0 and g["dropped"] == 0
        # the same estimator has the same noise (matched RMSE at equal spp)
        assert 0.75 < rep["var_ratio"] < 1.33, rep


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
