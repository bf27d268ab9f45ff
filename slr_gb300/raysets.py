"""Ray sets of the traversal microbenchmark on the 1M-triangle scene.

* coherent: primary rays of an n x n pinhole image through the pixel centres,
  in the scene camera's frame (the image x axis mirrored as in
  PerspectiveCamera.cpp:31-62), t_max infinite;
* incoherent: origins uniform over the surface area (area-weighted triangle,
  then a uniform point of it), directions uniform on the sphere, t_min 1e-4
  (the reference's continuation-ray epsilon), t_max uniform in [0.1, 10].

Rays are (n, 8) float32 rows (origin, t_min, direction, t_max) on the given
torch device, generated from a seeded torch generator.
"""
from __future__ import annotations

import math

import numpy as np


def coherent_rays(desc, n_side: int = 4096, device="cuda", stride: int = 1):
    """Every `stride`-th ray (row-major) of the n_side x n_side pinhole image."""
    import torch
    cam = desc.camera
    m = torch.tensor(cam.cam_to_world, dtype=torch.float64, device=device)
    th = math.tan(cam.fov_y / 2)
    idx = torch.arange(0, n_side * n_side, stride, dtype=torch.int64, device=device)
    y = (idx // n_side).double() + 0.5
    x = (idx % n_side).double() + 0.5
    lx = (0.5 - x / n_side) * 2 * th * cam.aspect      # mirrored image x (PerspectiveCamera)
    ly = (0.5 - y / n_side) * 2 * th
    dl = torch.stack([lx, ly, torch.ones_like(lx)], -1)
    dw = dl @ m[:3, :3].T
    dw = dw / dw.norm(dim=1, keepdim=True)
    rays = torch.zeros((len(idx), 8), dtype=torch.float32, device=device)
    rays[:, 0:3] = m[:3, 3].float()
    rays[:, 4:7] = dw.float()
    rays[:, 7] = float("inf")
    return rays


def incoherent_rays(desc, n: int = 1 << 24, device="cuda", seed: int = 0):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    tris = torch.tensor(desc.triangle_arrays(), dtype=torch.float32, device=device)
    area = 0.5 * torch.linalg.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]).norm(dim=1)
    pick = torch.multinomial(area, n, replacement=True, generator=g)
    u0 = torch.rand(n, device=device, generator=g)
    u1 = torch.rand(n, device=device, generator=g)
    su = u0.sqrt()
    b0, b1 = 1 - su, u1 * su
    t = tris[pick]
    org = b0[:, None] * t[:, 0] + b1[:, None] * t[:, 1] + (1 - b0 - b1)[:, None] * t[:, 2]
    z = torch.rand(n, device=device, generator=g) * 2 - 1
    phi = torch.rand(n, device=device, generator=g) * 2 * np.pi
    sz = (1 - z * z).clamp_min(0).sqrt()
    rays = torch.zeros((n, 8), dtype=torch.float32, device=device)
    rays[:, 0:3] = org
    rays[:, 3] = 1e-4
    rays[:, 4] = sz * torch.cos(phi)
    rays[:, 5] = sz * torch.sin(phi)
    rays[:, 6] = z
    rays[:, 7] = 0.1 + 9.9 * torch.rand(n, device=device, generator=g)
    return rays
