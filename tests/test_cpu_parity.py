"""Host-side parity with the reference (no GPU): the SBVH build, RGB spectral
upsampling, sampled spectra and the environment importance tables must be
bit-identical to the reference's on the same inputs; the numpy restatement of
the triangle test is pinned against the reference accelerator."""
import os

import numpy as np
import pytest

from slr_gb300 import scenes
from slr_gb300.scene_desc import LIGHT_SOURCE, REFLECTANCE, SceneDesc
from tests import helpers


def _sbvh_equal(gpu_lib, oracle_lib, desc):
    g = gpu_lib.Scene(desc, host_only=True)
    r = oracle_lib.RefScene(desc, build=False)
    rs = r.sbvh_stats()
    st = g.bvh_stats
    assert (st.num_fragments, st.depth, st.num_binary_nodes) == (rs["fragments"], rs["depth"], rs["nodes"])
    assert np.float32(st.sah_cost) == np.float32(rs["cost"])
    gb, gw, gl = g.sbvh_dump()
    rb, rw, rl = r.sbvh_dump()
    np.testing.assert_array_equal(gb.view(np.uint32), rb.view(np.uint32))
    np.testing.assert_array_equal(gw, rw)
    np.testing.assert_array_equal(gl, rl)
    return st


def test_sbvh_box_scene(gpu_lib, oracle_lib):
    _sbvh_equal(gpu_lib, oracle_lib, scenes.box_scene())


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (500, 2), (4000, 3)])
def test_sbvh_triangle_soup(gpu_lib, oracle_lib, n, seed):
    st = _sbvh_equal(gpu_lib, oracle_lib, helpers.triangle_soup(n, seed))
    if n >= 500:
        assert st.num_fragments > n  # spatial splits were exercised


def test_sbvh_heightfield(gpu_lib, oracle_lib):
    d = scenes.heightfield_scene(grid=48, spheres=4, sphere_freq=4, env_size=(16, 8))
    _sbvh_equal(gpu_lib, oracle_lib, d)


def test_upsampled_and_tabulated_spectra(gpu_lib, oracle_lib):
    # RGB spectra of type IndexOfRefraction are not compared: the reference's
    # constructor (spectrum_types.cpp:482-520) converts only Reflectance and
    # LightSource colours and leaves XYZ uninitialised otherwise.
    rng = np.random.default_rng(5)
    d = SceneDesc()
    for k in range(60):
        d.spectrum_rgb([REFLECTANCE, LIGHT_SOURCE][k % 2], *rng.random(3) * (1 + 20 * (k % 2 == 1)))
    d.spectrum_rgb(REFLECTANCE, 0, 0, 0)
    d.spectrum_rgb(LIGHT_SOURCE, 1, 0, 0)
    d.spectrum_rgb(REFLECTANCE, 0, 0, 1)
    d.spectrum_regular(rng.random(95) + 0.5, 360, 830)
    d.spectrum_regular(rng.random(7) + 1.0, 400, 700)
    wl = np.sort(rng.uniform(350, 850, 12)).astype(np.float32)
    d.spectrum_irregular(wl, rng.random(12))
    d.material("matte", (0,))
    g = gpu_lib.Scene(d, host_only=True)
    r = oracle_lib.RefScene(d, build=False)
    offs = rng.random(200).astype(np.float32)
    lam = (360.0 + 470.0 * (np.arange(16)[None, :] + offs[:, None]) / 16).astype(np.float32)
    lam = np.concatenate([lam, rng.uniform(300, 900, (50, 16)).astype(np.float32)])
    for i in range(len(d.spectra)):
        a = g.spectrum_evaluate(i, lam)
        b = r.spectrum_eval(i, lam)
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32), err_msg=f"spectrum {i}")


def test_restated_triangle_test_pinned(oracle_lib):
    d = helpers.triangle_soup(300, 9)
    rays = helpers.random_rays(d, 3000, seed=4)
    ref = oracle_lib.RefScene(d, build=False)
    rp, rt, _, _ = ref.trace(rays)
    from oracle.restate import brute_force_closest
    bp, bt = brute_force_closest(d.triangle_arrays(), rays)
    np.testing.assert_array_equal(bt.view(np.uint32), rt.view(np.uint32))
    res = helpers.compare_hits(d, rays, bp, bt, rp, rt)
    assert res["mismatch"] == 0, res


def test_bsdf_restatement_matches_golden():
    """The float64 restatement of the reference's non-delta BSDFs
    (tests/bsdf_f64.py), whose condition numbers set the GPU BSDF test's
    tolerance, reproduces the reference's own FP32 outputs on every query:
    the same sampling successes, and sampled directions, sampled values and
    pdfs, evaluated values and pdfs within 1e-5 + kappa * 16 * 2^-24."""
    from tests import bsdf_f64
    from tests.bsdf_cases import bsdf_cases
    golden = np.load(os.path.join(os.path.dirname(__file__), "golden", "bsdf_kat.npz"))
    u = 16 * 2.0 ** -24

    def rel(a, b):
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.abs(a - b) / np.abs(b)
        return np.where((a == 0) & (b == 0), 0.0, np.nan_to_num(r, nan=np.inf))

    for c in bsdf_cases():
        if c["kind"] not in bsdf_f64.KINDS_RESTATED:
            continue
        args = (c["kind"], c["spec0"], c.get("spec1", c["spec0"]), c.get("ax", 0.0), c.get("ay", 0.0), c["queries"])
        ref = golden[c["name"]]
        fs, d, pdf, ok = bsdf_f64.sample(*args)
        fe, pe = bsdf_f64.evaluate(*args)
        kd, ks, ke = bsdf_f64.conditions(*args)
        okr = ref[:, 19] > 0
        np.testing.assert_array_equal(ok, okr, err_msg=c["name"])
        assert np.all(np.abs(d[ok] - ref[ok, 16:19]).max(1) <= 1e-5 + kd[ok] * u), c["name"]
        es = np.maximum(rel(fs[ok], ref[ok, 0:16]).max(1), rel(pdf[ok], ref[ok, 19]))
        assert np.all(es <= 1e-5 + ks[ok] * u), c["name"]
        ee = np.maximum(rel(fe, ref[:, 21:37]).max(1), rel(pe, ref[:, 37]))
        assert np.all(ee <= 1e-5 + ke * u), c["name"]


def test_sbvh_full_ggx_scene(gpu_lib, oracle_lib):
    """The benchmark's 1,034,242-triangle scene: the whole SBVH (every node's
    box and words, every leaf reference) equals the reference's."""
    st = _sbvh_equal(gpu_lib, oracle_lib, scenes.heightfield_scene(seed=0))
    assert st.num_triangles == 1034242


def test_film_colour_matching_bins_bit_exact(gpu_lib, oracle_lib):
    """The 16-bin colour matching functions and their integral used to turn
    films into RGB equal the reference's DiscretizedSpectrum tables."""
    bins, integ = gpu_lib.film_cmf()
    rb, ri = oracle_lib.film_cmf()
    assert np.array_equal(bins.reshape(-1).view(np.uint32), rb.view(np.uint32))
    assert np.float32(integ).view(np.uint32) == np.float32(ri).view(np.uint32)


def _alias_pmf(prob, alias):
    n = len(prob)
    pmf = prob.astype(np.float64) / n
    np.add.at(pmf, alias, (1.0 - prob.astype(np.float64)) / n)
    return pmf


def test_alias_tables_carry_the_reference_pmfs(gpu_lib):
    """The GPU samples lights and the environment with alias tables; the
    probability each table gives every bin equals the PMF of the CDF the
    reference inverts (bit-identical CDFs are checked above)."""
    desc = scenes.heightfield_scene(grid=24, spheres=2, sphere_freq=2, env_size=(64, 32))
    s = gpu_lib.Scene(desc, host_only=True)
    tabs = s.alias_tables()
    env = s.environment_tables()
    np.testing.assert_allclose(_alias_pmf(*tabs["top"]), np.diff(env["top_cdf"].astype(np.float64)), rtol=1e-5,
                               atol=1e-7)
    rows_p, rows_a = tabs["rows"]
    for y in range(rows_p.shape[0]):
        np.testing.assert_allclose(_alias_pmf(rows_p[y], rows_a[y]), np.diff(env["row_cdf"][y].astype(np.float64)),
                                   rtol=1e-5, atol=1e-7)
    box = gpu_lib.Scene(scenes.box_scene(8, 8), host_only=True)
    lp, la = box.alias_tables()["lights"]
    assert len(lp) == 2
    np.testing.assert_allclose(_alias_pmf(lp, la), [0.5, 0.5])


def test_reference_bpt_agrees_with_pt(oracle_lib):
    """The oracle's bidirectional renderer (BPTRenderer with the subpath cap,
    its light-tracing buffers summed into the film) and its path tracer
    estimate the same image of the box: per-batch image sums within 4
    combined standard errors.  A film that missed the separated buffers
    (the t = 1 connections) would fall short by their share."""
    desc = scenes.box_scene(16, 16)
    k, spp = 12, 32
    tb, tp = [], []
    for i in range(k):
        ref = oracle_lib.RefScene(desc)
        tb.append(ref.render_bpt(16, 16, spp, 40, seed=10 + i, threads=os.cpu_count())[0].sum(dtype=np.float64) / spp)
        tp.append(ref.render(16, 16, spp, 40, seed=100 + i, threads=os.cpu_count())[0].sum(dtype=np.float64) / spp)
    tb, tp = np.array(tb), np.array(tp)
    z = (tb.mean() - tp.mean()) / np.sqrt(tb.var(ddof=1) / k + tp.var(ddof=1) / k)
    assert abs(z) < 4.0, (tb.mean(), tp.mean(), z)


def test_reference_path_tapes(oracle_lib):
    """Recording the reference's uniforms (oracle patch P12) changes nothing
    it renders: the one-thread, one-sample film equals a plain render with
    the same seed; one tape per pixel sample, each at least the seven camera
    draws long (time, pixel 2, wavelength, wavelength selection, lens 2)."""
    from slr_gb300 import scenes
    desc = scenes.box_scene(16, 8)
    ref = oracle_lib.RefScene(desc)
    film, tapes = ref.render_record(16, 8, 8, seed=9)
    plain, _ = ref.render(16, 8, 1, 8, seed=9, threads=1)
    np.testing.assert_array_equal(film, plain)
    assert len(tapes) == 16 * 8
    assert min(len(t) for t in tapes) >= 7
    assert all(((t >= 0) & (t < 1)).all() for t in tapes)


def test_flat_index_case_takes_the_pair_path():
    """The flat-index dielectric case of the BSDF tests holds between two and
    four distinct (exterior, interior) pairs over its 16 wavelengths, so the
    GPU evaluates it through its index-pair path, with more than one pair
    (the per-wavelength loop takes five or more)."""
    from tests.bsdf_cases import bsdf_cases
    c = [x for x in bsdf_cases() if x["name"] == "ggx_bsdf_flat"][0]
    pairs = set(zip(np.asarray(c["spec0"], np.float32).view(np.uint32),
                    np.asarray(c["spec1"], np.float32).view(np.uint32)))
    assert 2 <= len(pairs) <= 4
