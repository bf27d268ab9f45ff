"""Density-grid medium routines on the GPU against the reference's
DensityGridMediumDistribution (MediumDistribution/DensityGridMediumDistribution.cpp),
query by query, with both sides drawing the same replayed uniforms:
free-path sampling by delta tracking over super voxels with the ratio
estimator for the other wavelengths (interact, :402-575), ratio-tracking
transmittance with Russian roulette (evaluateTransmittance, :577-744) and the
trilinear extinction coefficient (evaluateExtinctionCoefficient, :756-759).

The medium is off-centre, its grid is not cubic (20 x 28 x 36 samples) and its
extinction varies with wavelength, so an axis or stride mix-up, a wrong
super-voxel walk or a wavelength mix-up changes the answers.  The GPU code
rounds differently from the reference's x86 build in the last bits (fused
multiply-adds), so a query whose uniform lands on a decision boundary can
branch the other way; at most 1% of queries may take a different branch, and
the rest must agree to float tolerance."""
import numpy as np
import pytest

from slr_gb300 import scenes
from slr_gb300.scene_desc import Medium

pytestmark = pytest.mark.gpu

BMIN = np.array([0.1, 0.05, 0.2])
BMAX = np.array([0.9, 0.85, 0.7])


def _scene():
    d = scenes.box_scene(8, 8)
    se = d.spectrum_regular(np.linspace(8, 24, 8).astype(np.float32), 360.0, 830.0)
    ss = d.spectrum_regular(np.linspace(6, 20, 8).astype(np.float32), 360.0, 830.0)
    rng = np.random.default_rng(5)
    dens = (scenes.fbm_density_grid(36, seed=3)[:, :28, :20] * 0.7 + 0.3 * rng.random((36, 28, 20))).astype(np.float32)
    d.medium = Medium(tuple(BMIN), tuple(BMAX), dens, ss, se, 0.5)
    return d


def _queries(n, seed, exit_fraction=True):
    rng = np.random.default_rng(seed)
    org = BMIN + rng.random((n, 3)) * (BMAX - BMIN)
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    t_exit = np.where(dirs > 0, (BMAX - org) / dirs, (BMIN - org) / dirs).min(1)
    dmin = np.where(rng.random(n) < 0.3, rng.random(n) * 0.3 * t_exit, 0.0)
    frac = rng.random(n) if exit_fraction else np.ones(n)
    dmax = dmin + (t_exit - dmin) * frac * 0.999
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3], rays[:, 3], rays[:, 4:7], rays[:, 7] = org, dmin, dirs, dmax
    off = rng.random(n)
    lam = (360 + 470 * (np.arange(16)[None, :] + off[:, None]) / 16).astype(np.float32)
    sel = (rng.integers(0, 16, n) | np.where(rng.random(n) < 0.25, 0x100, 0)).astype(np.int32)
    vals = rng.integers(0, 2 ** 32, (n, 512), dtype=np.uint64).astype(np.uint32)
    return rays, lam, sel, vals


def _close(a, b, rtol, atol):
    return np.abs(a - b) <= atol + rtol * np.abs(b)


@pytest.fixture(scope="module")
def scenes_pair(gpu_lib, oracle_lib):
    desc = _scene()
    return gpu_lib.Scene(desc), oracle_lib.RefScene(desc)


def test_extinction_coefficient_matches_reference(scenes_pair):
    g, r = scenes_pair
    rays, lam, sel, vals = _queries(4096, 11)
    rng = np.random.default_rng(12)
    rays[:, 0:3] = rng.random((len(rays), 3))
    rays[:64, 0:3] = np.round(rays[:64, 0:3])          # corners and faces of the grid
    out_g = g.medium_query(2, rays, lam, sel, vals[:, :0])
    out_r = r.medium_query(2, rays, lam, sel, vals[:, :0])
    assert _close(out_g[:, 6:22], out_r[:, 6:22], 2e-6, 1e-6).all()


@pytest.mark.parametrize("mode", [0, 1], ids=["interact", "transmittance"])
def test_medium_queries_match_reference(scenes_pair, mode):
    g, r = scenes_pair
    rays, lam, sel, vals = _queries(8192, 20 + mode)
    out_g = g.medium_query(mode, rays, lam, sel, vals)
    out_r = r.medium_query(mode, rays, lam, sel, vals)
    assert (out_r[:, 5] < vals.shape[1]).all()          # no query ran out of uniforms
    same_branch = (out_g[:, 0] == out_r[:, 0]) & (out_g[:, 5] == out_r[:, 5])
    assert same_branch.mean() >= 0.99, same_branch.mean()
    gs, rs = out_g[same_branch], out_r[same_branch]
    hit = rs[:, 0] == 1
    if mode == 0:
        assert 0.2 < hit.mean() < 0.8
        assert _close(gs[hit, 1], rs[hit, 1], 1e-4, 1e-6).all()
        assert _close(gs[hit, 2:5], rs[hit, 2:5], 1e-4, 1e-5).all()
    spec_ok = _close(gs[:, 6:22], rs[:, 6:22], 1e-3, 1e-6).all(1)
    assert spec_ok.mean() >= 0.995, spec_ok.mean()
    # nontrivial answers on both sides
    assert np.abs(rs[:, 6:22]).sum() > 0 and (rs[:, 6:22] != 1).any()


def test_medium_query_rejects_bad_mode(scenes_pair, gpu_lib):
    g, _ = scenes_pair
    rays, lam, sel, vals = _queries(4, 1)
    with pytest.raises(gpu_lib.SlrGpuError):
        g.medium_query(7, rays, lam, sel, vals)


@pytest.mark.parametrize("mode", [3, 4], ids=["aggregate_interact", "aggregate_transmittance"])
def test_medium_boundary_walk_matches_reference(scenes_pair, mode):
    """Segments that start outside, inside or on the medium's faces, with
    finite or unbounded ends, through the aggregate's boundary walk."""
    g, r = scenes_pair
    n = 8192
    rays, lam, sel, vals = _queries(n, 40 + mode)
    rng = np.random.default_rng(50 + mode)
    lo, hi = BMIN - 0.3, BMAX + 0.3
    org = lo + rng.random((n, 3)) * (hi - lo)
    face = rng.random(n) < 0.25                      # a quarter start on a face
    axis = rng.integers(0, 3, n)
    side = rng.random(n) < 0.5
    org[face, axis[face]] = np.where(side[face], BMIN[axis[face]], BMAX[axis[face]])
    rays[:, 0:3] = org
    aim = rng.random(n) < 0.7                        # most rays aim into the medium
    target = BMIN + rng.random((n, 3)) * (BMAX - BMIN)
    d = target - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays[aim, 4:7] = d[aim]
    # A segment that starts on a face at distance 0 is left out: the
    # reference's walk steps to distToNextBoundary * (1 + epsilon), which
    # makes no progress from 0 and never ends.  Paths never start there
    # (camera rays start outside, later rays start epsilon away).
    rays[:, 3] = np.where(face | (rng.random(n) < 0.5), 1e-4, 0.0)
    dmax = rays[:, 3] + 0.05 + 1.5 * rng.random(n)
    if mode == 4:
        rays[:, 7] = dmax
    else:
        rays[:, 7] = np.where(rng.random(n) < 0.3, np.inf, dmax)
    out_g = g.medium_query(mode, rays, lam, sel, vals)
    out_r = r.medium_query(mode, rays, lam, sel, vals)
    assert (out_r[:, 5] < vals.shape[1]).all()
    same_branch = (out_g[:, 0] == out_r[:, 0]) & (out_g[:, 5] == out_r[:, 5])
    assert same_branch.mean() >= 0.99, same_branch.mean()
    gs, rs = out_g[same_branch], out_r[same_branch]
    hit = rs[:, 0] == 1
    if mode == 3:
        assert 0.1 < hit.mean() < 0.9
        assert _close(gs[hit, 1], rs[hit, 1], 1e-4, 1e-6).all()
    spec_ok = _close(gs[:, 6:22], rs[:, 6:22], 1e-3, 1e-6).all(1)
    assert spec_ok.mean() >= 0.995, spec_ok.mean()
    assert (rs[:, 5] > 0).mean() > 0.3                # most segments cross the medium
