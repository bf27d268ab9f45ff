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
