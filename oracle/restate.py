"""CPU restatement (numpy, float32, no fused operations) of the reference's
ray-triangle and ray-box tests.  TEST INFRASTRUCTURE ONLY.

numpy evaluates every float32 operation with its own rounding, which is the
reference's arithmetic when compiled with -ffp-contract=off, so these
functions reproduce its results bit for bit.  Used to classify closest-hit
differences as exact ties (two triangles hit at the same t, where the
reference keeps the last one tested) and to check hits independently of both
BVHs.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def moller_trumbore(tris: np.ndarray, org: np.ndarray, dir_: np.ndarray, tmin: np.ndarray, tmax: np.ndarray):
    """TriangleSurfaceShape::intersect (libSLR/SurfaceShape/TriangleSurfaceShape.cpp:205-257).

    tris: (n, 3, 3) float32 vertex positions; org/dir: (n, 3); tmin/tmax: (n,).
    Returns (hit bool, t, b1, b2) with the reference's inclusive acceptance."""
    tris = tris.astype(f32)
    org = org.astype(f32)
    dir_ = dir_.astype(f32)
    v0 = tris[:, 0]
    e1 = tris[:, 1] - v0
    e2 = tris[:, 2] - v0
    with np.errstate(all="ignore"):
        p = _cross(dir_, e2)
        det = _dot(e1, p)
        inv = f32(1.0) / det
        d = org - v0
        b1 = _dot(d, p) * inv
        q = _cross(d, e1)
        b2 = _dot(dir_, q) * inv
        t = _dot(e2, q) * inv
        hit = (det != 0) & ~((b1 < 0) | (b1 > 1)) & ~((b2 < 0) | (b1 + b2 > 1)) & ~((t < tmin) | (t > tmax))
    return hit, t, b1, b2


def brute_force_closest(tris: np.ndarray, rays: np.ndarray, chunk: int = 256):
    """Closest hit by testing every triangle (small scenes only).  Returns
    (prim or 0xffffffff, t); among equal t the highest index wins."""
    n = len(rays)
    prim = np.full(n, 0xffffffff, np.uint32)
    tbest = np.full(n, np.inf, f32)
    for i0 in range(0, n, chunk):
        r = rays[i0:i0 + chunk]
        m = len(r)
        nt = len(tris)
        org = np.repeat(r[:, None, 0:3], nt, axis=1).reshape(-1, 3)
        dr = np.repeat(r[:, None, 4:7], nt, axis=1).reshape(-1, 3)
        tmin = np.repeat(r[:, 3:4], nt, axis=1).reshape(-1)
        tmax = np.repeat(r[:, 7:8], nt, axis=1).reshape(-1)
        tt = np.tile(tris, (m, 1, 1))
        hit, t, _, _ = moller_trumbore(tt, org, dr, tmin, tmax)
        t = np.where(hit, t, np.inf).reshape(m, nt)
        best = t.min(axis=1)
        has = np.isfinite(best)
        # last index attaining the minimum
        last = nt - 1 - np.argmax((t == best[:, None])[:, ::-1], axis=1)
        prim[i0:i0 + m] = np.where(has, last, 0xffffffff)
        tbest[i0:i0 + m] = best
    return prim, tbest
