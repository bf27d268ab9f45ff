"""Shared test utilities: ray sets and hit comparison."""
from __future__ import annotations

import numpy as np

from oracle.restate import moller_trumbore


def random_rays(desc, n: int, seed: int = 0, surface_fraction: float = 0.5, tmax_range=(0.1, 10.0)) -> np.ndarray:
    """(n, 8) float32 rays (org.xyz, tmin, dir.xyz, tmax): half start inside
    the scene bounds, half on surfaces (area-weighted triangle, uniform point);
    directions uniform on the sphere; tmax uniform in tmax_range, with one in
    eight unbounded."""
    rng = np.random.default_rng(seed)
    tris = desc.triangle_arrays().astype(np.float64)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    ext = hi - lo
    ns = int(n * surface_fraction)
    org = np.empty((n, 3))
    org[ns:] = lo - 0.05 * ext + rng.random((n - ns, 3)) * 1.1 * ext
    area = 0.5 * np.linalg.norm(np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]), axis=1)
    pick = rng.choice(len(tris), size=ns, p=area / area.sum())
    u0, u1 = rng.random(ns), rng.random(ns)
    su = np.sqrt(u0)
    b0, b1 = 1 - su, u1 * su
    b2 = 1 - b0 - b1
    t = tris[pick]
    org[:ns] = b0[:, None] * t[:, 0] + b1[:, None] * t[:, 1] + b2[:, None] * t[:, 2]
    z = rng.uniform(-1, 1, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - z * z)
    d = np.stack([s * np.cos(phi), s * np.sin(phi), z], 1)
    tmax = rng.uniform(*tmax_range, n)
    tmax[rng.random(n) < 0.125] = np.inf
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = org
    rays[:, 3] = np.where(np.arange(n) < ns, 1e-4, 0.0)
    rays[:, 4:7] = d
    rays[:, 7] = tmax
    return rays


def compare_hits(desc, rays, gprim, gt, rprim, rt) -> dict:
    """Closest-hit parity.  Same primitive: t must be bit-identical.
    Different primitives with bit-identical t are exact ties (the reference
    keeps the last triangle tested at equal t, so the winner depends on
    traversal order); they are checked with the numpy restatement and counted
    separately.  Anything else is a mismatch."""
    gprim = np.asarray(gprim, np.uint32)
    rprim = np.asarray(rprim, np.uint32)
    miss = np.uint32(0xffffffff)
    both_miss = (gprim == miss) & (rprim == miss)
    same = (gprim == rprim) & ~both_miss
    t_bad = same & (gt.view(np.uint32) != rt.view(np.uint32))
    diff = (gprim != rprim)
    ties = 0
    mismatch_idx = []
    tris = desc.triangle_arrays()
    for i in np.nonzero(diff)[0]:
        if gprim[i] != miss and rprim[i] != miss and gt[i] == rt[i]:
            hit, t, _, _ = moller_trumbore(tris[[gprim[i]]], rays[i:i + 1, 0:3], rays[i:i + 1, 4:7],
                                           rays[i:i + 1, 3], rays[i:i + 1, 7])
            if hit[0] and t[0] == rt[i]:
                ties += 1
                continue
        mismatch_idx.append(int(i))
    return {"rays": int(len(gprim)), "hits": int(((rprim != miss)).sum()), "ties": ties,
            "mismatch": len(mismatch_idx) + int(t_bad.sum()), "mismatch_idx": mismatch_idx[:10]}


def triangle_soup(n: int, seed: int = 0):
    """Random triangle soup in the unit cube (for traversal tests)."""
    from slr_gb300.scene_desc import REFLECTANCE, SceneDesc
    rng = np.random.default_rng(seed)
    d = SceneDesc()
    m = d.material("matte", (d.spectrum_rgb(REFLECTANCE, 0.5, 0.5, 0.5),))
    c = rng.random((n, 1, 3))
    p = (c + 0.08 * rng.standard_normal((n, 3, 3))).astype(np.float32).reshape(-1, 3)
    d.mesh(p, np.arange(3 * n, dtype=np.uint32).reshape(-1, 3), m)
    return d
