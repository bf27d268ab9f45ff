"""Traversal parity on the GPU: the same ray sets give the reference SBVH's
closest hit (same primitive id, bit-identical t; exact ties at equal t are
classified with the restated triangle test) and the same any-hit answers."""
import os

import numpy as np
import pytest

from slr_gb300 import scenes
from tests import helpers

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _gpu_trace(gpu_lib, desc, rays):
    import torch
    s = gpu_lib.Scene(desc)
    r = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    prim, t, b1, b2 = s.trace(r)
    occ, _, _, _ = s.trace(r, any_hit=True)
    torch.cuda.synchronize()
    return (prim.cpu().numpy().view(np.uint32), t.cpu().numpy(), b1.cpu().numpy(), b2.cpu().numpy(),
            occ.cpu().numpy().astype(bool))


@pytest.mark.parametrize("name,desc_fn", [("trace_box", lambda: scenes.box_scene(32, 32)),
                                          ("trace_soup", lambda: helpers.triangle_soup(3000, 7))])
def test_trace_matches_golden(gpu_lib, name, desc_fn):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    desc = desc_fn()
    prim, t, b1, b2, occ = _gpu_trace(gpu_lib, desc, g["rays"])
    res = helpers.compare_hits(desc, g["rays"], prim, t, g["prim"], g["t"])
    assert res["mismatch"] == 0, res
    same = prim == g["prim"]
    np.testing.assert_array_equal(b1[same].view(np.uint32), g["b1"][same].view(np.uint32))
    np.testing.assert_array_equal(occ, g["occluded"].astype(bool))


def test_trace_matches_oracle_heightfield(gpu_lib, oracle_lib):
    desc = scenes.heightfield_scene(grid=96, spheres=6, sphere_freq=6, env_size=(16, 8))
    rays = helpers.random_rays(desc, 60000, seed=21)
    prim, t, _, _, occ = _gpu_trace(gpu_lib, desc, rays)
    ref = oracle_lib.RefScene(desc, build=False)
    rp, rt, _, _ = ref.trace(rays)
    ro, _, _, _ = ref.trace(rays, anyhit=True)
    res = helpers.compare_hits(desc, rays, prim, t, rp, rt)
    assert res["mismatch"] == 0, res
    np.testing.assert_array_equal(occ, ro)


def test_trace_edge_cases(gpu_lib, oracle_lib):
    """Axis-parallel rays, rays starting on triangle edges/vertices, zero-
    length segments and degenerate (zero-area) triangles."""
    d = helpers.triangle_soup(50, 3)
    tris = d.triangle_arrays()
    from slr_gb300.scene_desc import REFLECTANCE
    m = d.material("matte", (d.spectrum_rgb(REFLECTANCE, 0.5, 0.5, 0.5),))
    d.mesh(np.array([[0.2, 0.2, 0.2], [0.4, 0.4, 0.4], [0.6, 0.6, 0.6]], np.float32), np.array([[0, 1, 2]]), m)
    rays = []
    rng = np.random.default_rng(0)
    for tri in tris[:40]:
        for v in (tri[0], 0.5 * (tri[0] + tri[1]), tri.mean(0)):
            for ax in range(3):
                for sgn in (1.0, -1.0):
                    dvec = np.zeros(3)
                    dvec[ax] = sgn
                    o = v - 0.5 * dvec
                    rays.append(np.r_[o, 0.0, dvec, rng.choice([0.5, np.inf, 0.0])])
    rays = np.array(rays, np.float32)
    prim, t, _, _, occ = _gpu_trace(gpu_lib, d, rays)
    ref = oracle_lib.RefScene(d, build=False)
    rp, rt, _, _ = ref.trace(rays)
    ro, _, _, _ = ref.trace(rays, anyhit=True)
    res = helpers.compare_hits(d, rays, prim, t, rp, rt)
    assert res["mismatch"] == 0, res
    np.testing.assert_array_equal(occ, ro)


def test_trace_empty_batch_and_empty_scene(gpu_lib):
    import torch
    from slr_gb300.scene_desc import SceneDesc
    s = gpu_lib.Scene(helpers.triangle_soup(10, 1))
    prim, _, _, _ = s.trace(torch.zeros((0, 8), device="cuda"))
    assert prim.numel() == 0
    e = gpu_lib.Scene(SceneDesc())
    rays = torch.tensor([[0, 0, 0, 0, 0, 0, 1, float("inf")]], device="cuda")
    prim, t, _, _ = e.trace(rays)
    assert int(prim.cpu().numpy().view(np.uint32)[0]) == 0xffffffff


def _edge_rays(P, T, origins):
    """Rays from each origin through every vertex and every edge midpoint of
    the mesh (P, T): exactly the points a non-watertight test can slip
    through."""
    targets = [P]
    for a, b in ((0, 1), (1, 2), (2, 0)):
        targets.append(0.5 * (P[T[:, a]] + P[T[:, b]]))
    targets = np.concatenate(targets)
    rays = []
    for o in origins:
        d = targets - o
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        r = np.zeros((len(d), 8), np.float32)
        r[:, 0:3] = o
        r[:, 4:7] = d
        r[:, 7] = np.inf
        rays.append(r)
    return np.concatenate(rays)


def test_watertight_closed_mesh_has_no_leaks(gpu_lib):
    """A closed geodesic sphere, rays from inside through every vertex and
    edge midpoint: the watertight test hits on every ray (the reference's
    Moller-Trumbore test may let some through; counted, not required)."""
    import torch
    from slr_gb300.scene_desc import REFLECTANCE, SceneDesc
    P, T = scenes.geodesic_sphere(12)          # closed: every edge shared by two triangles
    P = P.astype(np.float32) * np.float32(0.73)
    d = SceneDesc()
    m = d.material("matte", (d.spectrum_rgb(REFLECTANCE, 0.5, 0.5, 0.5),))
    d.mesh(P, T, m)
    rng = np.random.default_rng(4)
    origins = [np.zeros(3)] + list(rng.uniform(-0.3, 0.3, (5, 3)))
    rays = _edge_rays(P.astype(np.float64), T, origins)
    s = gpu_lib.Scene(d)
    r = torch.from_numpy(rays).cuda()
    wt, _, _, _ = s.trace(r, watertight=True)
    mt, _, _, _ = s.trace(r)
    torch.cuda.synchronize()
    wt = wt.cpu().numpy().view(np.uint32)
    mt = mt.cpu().numpy().view(np.uint32)
    assert (wt != 0xffffffff).all(), int((wt == 0xffffffff).sum())
    assert len(rays) > 20000
    print("reference-order test misses:", int((mt == 0xffffffff).sum()), "of", len(rays))


def test_watertight_agrees_with_reference_away_from_edges(gpu_lib, oracle_lib):
    """Random rays: the watertight test finds the reference's primitive
    except where the hit lies within rounding of an edge or vertex (smallest
    barycentric weight below 1e-5) or at an exact tie."""
    import torch
    desc = scenes.heightfield_scene(grid=96, spheres=6, sphere_freq=6, env_size=(16, 8))
    rays = helpers.random_rays(desc, 60000, seed=31)
    s = gpu_lib.Scene(desc)
    r = torch.from_numpy(rays).cuda()
    prim, t, b1, b2 = s.trace(r, watertight=True)
    occ, _, _, _ = s.trace(r, any_hit=True, watertight=True)
    torch.cuda.synchronize()
    prim = prim.cpu().numpy().view(np.uint32)
    t = t.cpu().numpy()
    ref = oracle_lib.RefScene(desc, build=False)
    rp, rt, rb1, rb2 = ref.trace(rays)
    ro, _, _, _ = ref.trace(rays, anyhit=True)
    diff = np.nonzero(prim != rp)[0]
    wmin = np.minimum(np.minimum(rb1, rb2), 1 - rb1 - rb2)
    near_edge = (rp[diff] != 0xffffffff) & (wmin[diff] < 1e-5)
    tie = (prim[diff] != 0xffffffff) & (rp[diff] != 0xffffffff) & (np.abs(t[diff] - rt[diff]) <= 1e-6 * np.abs(rt[diff]))
    unexplained = diff[~(near_edge | tie)]
    assert len(unexplained) == 0, (len(diff), unexplained[:10])
    assert len(diff) <= 1e-3 * len(rays)
    same = prim == rp
    hit = same & (rp != 0xffffffff)
    # same triangle: t from a different formula, equal to float rounding
    # (relative 1e-5, plus 1e-6 absolute for the hits just past tmin)
    assert np.all(np.abs(t[hit] - rt[hit]) <= 1e-5 * np.abs(rt[hit]) + 1e-6)
    assert (occ.cpu().numpy().astype(bool) != ro).mean() <= 1e-3
