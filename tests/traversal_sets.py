"""GPU side of the traversal parity test on the 1M-triangle benchmark scene.

Run as a script (``python -m tests.traversal_sets RAYS.npz OUT.npz``) it
traces the saved ray sets with whichever library variant SLRGPU_LIB_VARIANT
selects and saves the results, so that a test can check the 8-wide BVH build
in a process of its own.  The ray sets are generated once per test session
(torch's multinomial sampling on the GPU need not repeat bit for bit)."""
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


def gpu_trace_sets(api, desc, sets: dict) -> dict:
    """Traces the given ray sets ({name: (n, 8) float32 numpy array})."""
    import torch
    scene = api.Scene(desc)
    out = {"bvh_width": scene.bvh_stats.width}
    for name, host_rays in sets.items():
        rays = torch.from_numpy(np.ascontiguousarray(host_rays)).cuda()
        out[f"{name}_rays"] = host_rays
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


def main(rays_path: str, out_path: str) -> int:
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from slr_gb300 import api, scenes
    sets = dict(np.load(rays_path))
    res = gpu_trace_sets(api, scenes.heightfield_scene(seed=0), sets)
    np.savez(out_path, **res)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1], sys.argv[2]))
