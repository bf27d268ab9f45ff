"""GPU side of the traversal parity test on the 1M-triangle benchmark scene.

Run as a script (``python -m tests.traversal_sets OUT.npz``) it traces the
ray sets with whichever library variant SLRGPU_LIB_VARIANT selects and saves
the results, so that a test can check the 8-wide BVH build in a process of
its own."""
from __future__ import annotations

import sys

import numpy as np

N_PER_SET = 1 << 20


def ray_sets(desc, device="cuda"):
    """1,048,576 coherent rays (every 16th pixel centre of the 4096 x 4096
    pinhole image) and 1,048,576 incoherent rays (surface origins, uniform
    directions, t_max uniform in [0.1, 10])."""
    from slr_gb300 import raysets
    return {"coherent": raysets.coherent_rays(desc, 4096, device, stride=16),
            "incoherent": raysets.incoherent_rays(desc, N_PER_SET, device, seed=0)}


def gpu_trace_sets(api, desc) -> dict:
    import torch
    scene = api.Scene(desc)
    out = {"bvh_width": scene.bvh_stats.width}
    for name, rays in ray_sets(desc).items():
        out[f"{name}_rays"] = rays.cpu().numpy()
        for wt in (False, True):
            tag = f"{name}_{'wt' if wt else 'mt'}"
            prim, t, b1, b2 = scene.trace(rays, watertight=wt)
            occ, _, _, _ = scene.trace(rays, any_hit=True, watertight=wt)
            torch.cuda.synchronize()
            out[f"{tag}_prim"] = prim.cpu().numpy().view(np.uint32)
            out[f"{tag}_t"] = t.cpu().numpy()
            out[f"{tag}_b1"] = b1.cpu().numpy()
            out[f"{tag}_b2"] = b2.cpu().numpy()
            out[f"{tag}_occ"] = occ.cpu().numpy().astype(bool)
    scene.close()
    return out


def main(path: str) -> int:
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from slr_gb300 import api, scenes
    res = gpu_trace_sets(api, scenes.heightfield_scene(seed=0))
    np.savez(path, **res)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1]))
