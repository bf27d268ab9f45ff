"""Procedural scenes for the benchmark and parity configurations.

All scenes are synthetic and seeded; the only file they touch is the cache of
large noise grids (:func:`fbm_density_grid`).

* :func:`box_scene`   - the closed-box scene: a [0,1]^3 box of 10 triangles
  (open front face), two rotated boxes of 12 triangles each and a 0.25 x 0.25
  ceiling area light of radiance 15, seen by a pinhole camera.
* :func:`heightfield_scene` - the ~1M-triangle GGX scene: a 512 x 512-vertex
  height field displaced by 6-octave improved Perlin noise, 64 geodesic
  spheres of 8000 triangles, GGX conductors and dielectrics, and a seeded
  512 x 256 log-normal environment with a 2-degree sun.
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

from .scene_desc import (Camera, Environment, LIGHT_SOURCE, REFLECTANCE, SceneDesc)


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera-to-world matrix for the reference's camera frame, whose local
    +z is the viewing direction and whose image x axis is mirrored
    (PerspectiveCamera.cpp:71-83): local x = -right, local y = up."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[:3, 0] = -r
    m[:3, 1] = u
    m[:3, 2] = f
    m[:3, 3] = eye
    return m.astype(np.float32)


def _quad(p0, p1, p2, p3):
    return np.array([p0, p1, p2, p3], np.float32), np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def _box(center, size, angle_y):
    """12-triangle box rotated about the y axis, outward-facing winding."""
    cx, cy, cz = center
    sx, sy, sz = (0.5 * s for s in size)
    c, s = math.cos(angle_y), math.sin(angle_y)
    corners = []
    for dy in (-sy, sy):
        for dz in (-sz, sz):
            for dx in (-sx, sx):
                x, z = c * dx + s * dz, -s * dx + c * dz
                corners.append((cx + x, cy + dy, cz + z))
    v = np.array(corners, np.float32)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    pos, idx = [], []
    for f in faces:
        base = len(pos)
        pos.extend(v[list(f)])
        idx.extend([[base, base + 1, base + 2], [base, base + 2, base + 3]])
    return np.array(pos, np.float32), np.array(idx, np.uint32)


def box_scene(width: int = 256, height: int = 256) -> SceneDesc:
    d = SceneDesc()
    white = d.material("matte", (d.spectrum_rgb(REFLECTANCE, 0.73, 0.73, 0.73),))
    red = d.material("matte", (d.spectrum_rgb(REFLECTANCE, 0.63, 0.06, 0.05),))
    green = d.material("matte", (d.spectrum_rgb(REFLECTANCE, 0.14, 0.45, 0.09),))
    light = d.material("emitter", (d.spectrum_rgb(LIGHT_SOURCE, 15.0, 15.0, 15.0),), base=white)
    # Walls (front face z = 1 open), vertex normals face inward.
    walls = [
        (_quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)), white),   # floor
        (_quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)), white),   # ceiling
        (_quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)), white),   # back
        (_quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), red),     # left  x = 0
        (_quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)), green),   # right x = 1
    ]
    inward = [(0, 1, 0), (0, -1, 0), (0, 0, 1), (1, 0, 0), (-1, 0, 0)]
    for ((p, idx), mat), n in zip(walls, inward):
        nrm = np.tile(np.array(n, np.float32), (4, 1))
        d.mesh(p, idx, mat, normals=nrm, tangents=_tangent_for(nrm), uvs=_quad_uv())
    for center, size, ang in (((0.66, 0.15, 0.62), (0.3, 0.3, 0.3), -0.3),
                              ((0.33, 0.3, 0.35), (0.3, 0.6, 0.3), 0.3)):
        p, idx = _box(center, size, ang)
        tri = p[idx]
        fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
        fn /= np.linalg.norm(fn, axis=1, keepdims=True)
        nrm = np.zeros_like(p)
        nrm[idx[:, 0]] = fn
        nrm[idx[:, 1]] = fn
        nrm[idx[:, 2]] = fn
        d.mesh(p, idx, white, normals=nrm, tangents=_tangent_for(nrm), uvs=np.zeros((len(p), 2), np.float32))
    # Ceiling light 0.25 x 0.25 just below y = 1, emitting downward.
    y = 0.999
    p, idx = _quad((0.375, y, 0.375), (0.625, y, 0.375), (0.625, y, 0.625), (0.375, y, 0.625))
    nrm = np.tile(np.array((0, -1, 0), np.float32), (4, 1))
    d.mesh(p, idx, light, normals=nrm, tangents=_tangent_for(nrm), uvs=_quad_uv())
    d.camera = Camera("perspective", look_at((0.5, 0.5, 2.3), (0.5, 0.5, 0.0)), sensitivity=1.0,
                      aspect=width / height, fov_y=math.radians(38.0), lens_radius=0.0,
                      img_plane_dist=1.0, obj_plane_dist=2.3)
    return d


def glossy_box_scene(width: int = 256, height: int = 256) -> SceneDesc:
    """The box scene with every BSDF kind under its ceiling light: the tall
    block a rough GGX conductor (anisotropic), the short block smooth glass
    (delta reflection / refraction), a small floating block rough GGX glass
    and a mirror (delta conductor) on the back wall.  No environment, so both
    the unidirectional and the bidirectional tracers take it."""
    d = box_scene(width, height)
    white = 0

    def flat(v):
        return d.spectrum_regular(np.array([v, v], np.float32), 360.0, 830.0)

    metal = d.material("microfacet_reflection", (flat(1.5), flat(2.0)), 0.3, 0.15)
    glass = d.material("specular_scattering", (d.spectrum_rgb(REFLECTANCE, 1.0, 1.0, 1.0), flat(1.0), flat(1.5)))
    rough_glass = d.material("microfacet_scattering", (flat(1.0), flat(1.45)), 0.2, 0.2)
    mirror = d.material("specular_reflection", (d.spectrum_rgb(REFLECTANCE, 0.95, 0.95, 0.95), flat(0.2), flat(3.0)))
    # the two blocks of the box scene are its last two white meshes before the light
    blocks = [i for i, m in enumerate(d.meshes) if m.material == white][-2:]
    d.meshes[blocks[0]] = dataclasses.replace(d.meshes[blocks[0]], material=glass)
    d.meshes[blocks[1]] = dataclasses.replace(d.meshes[blocks[1]], material=metal)
    p, idx = _box((0.5, 0.62, 0.55), (0.12, 0.12, 0.12), 0.7)
    d.mesh(p, idx, rough_glass)
    q, qidx = _quad((0.55, 0.3, 0.001), (0.9, 0.3, 0.001), (0.9, 0.75, 0.001), (0.55, 0.75, 0.001))
    nrm = np.tile(np.array((0, 0, 1), np.float32), (4, 1))
    d.mesh(q, qidx, mirror, normals=nrm, tangents=_tangent_for(nrm), uvs=_quad_uv())
    return d


class ImprovedPerlin:
    """Ken Perlin's improved noise (SIGGRAPH 2002): quintic fade, 12 gradient
    directions picked by a hashed permutation table (seeded here)."""

    _GRAD = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
                      [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1], [1, 1, 0], [0, -1, 1],
                      [-1, 1, 0], [0, -1, -1]], np.float64)

    def __init__(self, seed: int):
        rng = np.random.default_rng(seed)
        p = rng.permutation(256)
        self.perm = np.concatenate([p, p]).astype(np.int64)

    def __call__(self, x, y, z):
        x, y, z = (np.asarray(a, np.float64) for a in (x, y, z))
        xi, yi, zi = (np.floor(a).astype(np.int64) & 255 for a in (x, y, z))
        xf, yf, zf = x - np.floor(x), y - np.floor(y), z - np.floor(z)
        fade = lambda t: t * t * t * (t * (t * 6 - 15) + 10)  # noqa: E731
        u, v, w = fade(xf), fade(yf), fade(zf)
        P = self.perm
        A, B = P[xi] + yi, P[xi + 1] + yi
        AA, AB, BA, BB = P[A] + zi, P[A + 1] + zi, P[B] + zi, P[B + 1] + zi

        def g(h, dx, dy, dz):
            gr = self._GRAD[P[h] & 15]
            return gr[..., 0] * dx + gr[..., 1] * dy + gr[..., 2] * dz

        lerp = lambda t, a, b: a + t * (b - a)  # noqa: E731
        x1 = lerp(u, g(AA, xf, yf, zf), g(BA, xf - 1, yf, zf))
        x2 = lerp(u, g(AB, xf, yf - 1, zf), g(BB, xf - 1, yf - 1, zf))
        x3 = lerp(u, g(AA + 1, xf, yf, zf - 1), g(BA + 1, xf - 1, yf, zf - 1))
        x4 = lerp(u, g(AB + 1, xf, yf - 1, zf - 1), g(BB + 1, xf - 1, yf - 1, zf - 1))
        return lerp(w, lerp(v, x1, x2), lerp(v, x3, x4))

    def fbm(self, x, y, z, octaves: int, base_freq: float = 1.0, persistence: float = 0.5):
        total = 0.0
        amp, freq, norm = 1.0, base_freq, 0.0
        for _ in range(octaves):
            total = total + amp * self(x * freq, y * freq, z * freq)
            norm += amp
            amp *= persistence
            freq *= 2.0
        return total / norm


def geodesic_sphere(freq: int):
    """Icosahedron with every face split into freq^2 triangles, projected
    onto the unit sphere (20 freq^2 triangles, shared vertices)."""
    t = (1 + 5 ** 0.5) / 2
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    pts, tris = [], []
    for a, b, c in F:
        base = len(pts)
        ids = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                k = freq - i - j
                ids[(i, j)] = len(pts)
                pts.append((V[a] * k + V[b] * i + V[c] * j) / freq)
        for i in range(freq):
            for j in range(freq - i):
                tris.append((ids[(i, j)], ids[(i + 1, j)], ids[(i, j + 1)]))
                if j + i + 1 < freq:
                    tris.append((ids[(i + 1, j)], ids[(i + 1, j + 1)], ids[(i, j + 1)]))
        del base
    P = np.array(pts)
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    key = np.round(P * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    P = P[first]
    T = inv.reshape(-1)[np.array(tris)]
    # outward winding
    tri = P[T]
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    flip = (nrm * tri.mean(1)).sum(1) < 0
    T[flip] = T[flip][:, [0, 2, 1]]
    return P, T


def lognormal_environment(width: int, height: int, seed: int, sun_radiance: float = 5e4, sun_diameter_deg: float = 2.0,
                          sun_dir=(0.35, 0.75, -0.55), store_scale: float = 16.0) -> Environment:
    """Seeded equirectangular environment: per-texel log-normal radiance
    (mu = 0, sigma = 1) with a mild per-channel tint, plus a sun disk.  Texel
    (x, y) covers the direction fromPolarYUp(phi, theta) with
    phi = 2 pi (x + 0.5) / W, theta = pi (y + 0.5) / H, the reference's
    environment parameterisation (Vector3D.h:71-73, surface_object.cpp:201-238).
    Values are stored divided by store_scale and the environment scale is
    store_scale, so half-float texels stay finite."""
    rng = np.random.default_rng(seed)
    lum = rng.lognormal(0.0, 1.0, (height, width))
    tint = rng.uniform(0.8, 1.2, (height, width, 3))
    rgb = lum[..., None] * tint
    phi = 2 * np.pi * (np.arange(width) + 0.5) / width
    theta = np.pi * (np.arange(height) + 0.5) / height
    th, ph = np.meshgrid(theta, phi, indexing="ij")
    d = np.stack([-np.sin(ph) * np.sin(th), np.cos(th), np.cos(ph) * np.sin(th)], -1)
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    cosang = d @ s
    in_sun = cosang >= np.cos(np.radians(sun_diameter_deg / 2))
    if not in_sun.any():
        in_sun[np.unravel_index(np.argmax(cosang), cosang.shape)] = True
    rgb[in_sun] = sun_radiance
    rgba = np.ones((height, width, 4), np.float32)
    rgba[..., :3] = rgb / store_scale
    return Environment(rgba.astype(np.float16), float(store_scale))


def heightfield_scene(grid: int = 512, spheres: int = 64, sphere_freq: int = 20, env_size=(512, 256),
                      width: int = 1024, height: int = 1024, seed: int = 0) -> SceneDesc:
    """~1M-triangle GGX scene: height field grid x grid vertices over
    [-1, 1]^2 displaced by 6-octave improved Perlin fBm (amplitude 0.2), plus
    `spheres` geodesic spheres (20 freq^2 triangles each) with scale
    log-uniform in [0.05, 0.3].  Every object gets a GGX conductor or
    dielectric: alpha ~ U[0.05, 0.6], anisotropy a ~ U[0, 0.8] mapped to
    alpha_x = alpha / sqrt(1 - 0.9 a), alpha_y = alpha sqrt(1 - 0.9 a),
    eta ~ U[1.3, 1.7] (flat spectrum), conductor k ~ U[1, 3] (flat).
    Lit by the seeded log-normal environment with a 2-degree sun."""
    rng = np.random.default_rng(seed)
    noise = ImprovedPerlin(seed + 1)
    d = SceneDesc()

    def flat(v):
        return d.spectrum_regular(np.array([v, v], np.float32), 360.0, 830.0)

    def ggx_material():
        alpha = rng.uniform(0.05, 0.6)
        a = rng.uniform(0.0, 0.8)
        ax, ay = alpha / math.sqrt(1 - 0.9 * a), alpha * math.sqrt(1 - 0.9 * a)
        eta = rng.uniform(1.3, 1.7)
        if rng.random() < 0.5:
            return d.material("microfacet_reflection", (flat(eta), flat(rng.uniform(1.0, 3.0))), ax, ay)
        return d.material("microfacet_scattering", (flat(1.0), flat(eta)), ax, ay)

    # Height field.
    xs = np.linspace(-1.0, 1.0, grid)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    H = 0.2 * noise.fbm(X * 2.0, np.zeros_like(X) + 0.37, Z * 2.0, octaves=6)
    pos = np.stack([X, H, Z], -1).reshape(-1, 3)
    dx = xs[1] - xs[0]
    gx = np.gradient(H, dx, axis=1)
    gz = np.gradient(H, dx, axis=0)
    nrm = np.stack([-gx, np.ones_like(H), -gz], -1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    tan = np.stack([np.ones_like(H), gx, np.zeros_like(H)], -1).reshape(-1, 3)
    tan -= (tan * nrm).sum(1, keepdims=True) * nrm
    tan /= np.linalg.norm(tan, axis=1, keepdims=True)
    uv = np.stack([(X + 1) / 2, (Z + 1) / 2], -1).reshape(-1, 2)
    i = np.arange(grid - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    v00 = (J * grid + I).reshape(-1)
    v10, v01, v11 = v00 + 1, v00 + grid, v00 + grid + 1
    idx = np.concatenate([np.stack([v00, v01, v10], 1), np.stack([v10, v01, v11], 1)])
    d.mesh(pos, idx, ggx_material(), normals=nrm, tangents=tan, uvs=uv)

    # Geodesic spheres resting on the height field.
    SP, ST = geodesic_sphere(sphere_freq)
    stan = np.cross(np.array([0.0, 1.0, 0.0]), SP)
    bad = np.linalg.norm(stan, axis=1) < 1e-6
    stan[bad] = (1.0, 0.0, 0.0)
    stan /= np.linalg.norm(stan, axis=1, keepdims=True)
    for _ in range(spheres):
        r = math.exp(rng.uniform(math.log(0.05), math.log(0.3)))
        cx, cz = rng.uniform(-0.85, 0.85, 2)
        cy = 0.2 * noise.fbm(np.array([cx * 2.0]), np.array([0.37]), np.array([cz * 2.0]), octaves=6)[0] + 0.6 * r
        p = SP * r + np.array([cx, cy, cz])
        d.mesh(p, ST, ggx_material(), normals=SP, tangents=stan,
               uvs=np.zeros((len(SP), 2), np.float32))

    d.environment = lognormal_environment(env_size[0], env_size[1], seed + 2)
    d.camera = Camera("perspective", look_at((0.0, 1.25, 2.15), (0.0, 0.0, -0.1)), sensitivity=1.0,
                      aspect=width / height, fov_y=math.radians(45.0), lens_radius=0.0,
                      img_plane_dist=1.0, obj_plane_dist=2.5)
    return d


def fbm_density_grid(n: int, seed: int = 0, octaves: int = 5) -> np.ndarray:
    """n^3 density grid [z][y][x]: max(0, 5-octave fBm improved Perlin),
    normalised to a maximum of 1.  Evaluated in slabs of z (the same numbers
    as one whole-grid evaluation, with far smaller temporaries); grids of
    128^3 and larger are kept in slr_gb300/_cache (or $SLR_GB300_CACHE) after
    the first evaluation, which takes about half a minute at 256^3."""
    cache_dir = os.environ.get("SLR_GB300_CACHE", os.path.join(os.path.dirname(os.path.abspath(__file__)), "_cache"))
    path = os.path.join(cache_dir, f"fbm_{n}_{seed}_{octaves}.npy")
    if n >= 128 and os.path.isfile(path):
        try:
            d = np.load(path)
            if d.shape == (n, n, n) and d.dtype == np.float32:
                return d
        except (OSError, ValueError):
            pass
    noise = ImprovedPerlin(seed + 7)
    c = (np.arange(n) + 0.5) / n
    Y, X = np.meshgrid(c, c, indexing="ij")
    d = np.empty((n, n, n), np.float64)
    slab = max(1, (1 << 20) // (n * n))
    for z0 in range(0, n, slab):
        zs = c[z0:z0 + slab]
        Z = np.broadcast_to(zs[:, None, None], (len(zs), n, n))
        d[z0:z0 + slab] = np.maximum(noise.fbm(np.broadcast_to(X * 3.0 + 0.13, Z.shape),
                                               np.broadcast_to(Y * 3.0 + 0.71, Z.shape), Z * 3.0 + 0.37,
                                               octaves=octaves), 0.0)
    m = d.max()
    if m > 0:
        d /= m
    d = d.astype(np.float32)
    if n >= 128:
        try:
            os.makedirs(cache_dir, exist_ok=True)
            tmp = f"{path}.{os.getpid()}.tmp.npy"
            np.save(tmp, d)
            os.replace(tmp, path)
        except OSError:
            pass
    return d


def medium_box_scene(width: int = 512, height: int = 512, grid: int = 256, seed: int = 0, sigma_t_max: float = 20.0,
                     albedo: float = 0.9, g: float = 0.7) -> SceneDesc:
    """The closed-box scene filled with a heterogeneous medium over [0,1]^3:
    a grid^3 fBm density, extinction sigma_t_max * density (flat spectrum),
    scattering albedo * extinction, Henyey-Greenstein phase with asymmetry g."""
    from .scene_desc import Medium
    d = box_scene(width, height)
    s_e = d.spectrum_regular(np.array([sigma_t_max, sigma_t_max], np.float32), 360.0, 830.0)
    s_s = d.spectrum_regular(np.array([albedo * sigma_t_max] * 2, np.float32), 360.0, 830.0)
    d.medium = Medium((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), fbm_density_grid(grid, seed), s_s, s_e, g)
    return d


def _quad_uv():
    return np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)


def _tangent_for(nrm: np.ndarray) -> np.ndarray:
    a = np.where(np.abs(nrm[:, :1]) < 0.9, np.array([[1.0, 0, 0]], np.float32), np.array([[0, 0, 1.0]], np.float32))
    t = a - (a * nrm).sum(1, keepdims=True) * nrm
    return (t / np.linalg.norm(t, axis=1, keepdims=True)).astype(np.float32)


def serving_scenes(seed: int = 0, count: int = 8, min_tris: int = 1000, max_tris: int = 2_000_000):
    """The serving workload's scenes: `count` height-field + sphere scenes
    built as heightfield_scene, with triangle counts log-spaced from min_tris
    to max_tris (half in the height field, half in 8 geodesic spheres); every
    second scene also carries the volumetric benchmark's medium (a 256^3 fBm
    density grid, sigma_t max 20, albedo 0.9, Henyey-Greenstein g = 0.7) as a
    fog layer over the terrain, y in [-0.25, 0.15]; the media share one
    density grid.  Square images."""
    from .scene_desc import Medium
    out = []
    density = None
    for k, n in enumerate(np.geomspace(min_tris, max_tris, count)):
        f = max(1, int(round(math.sqrt(n * 0.5 / (8 * 20)))))
        g = max(4, int(round(math.sqrt(n * 0.5 / 2))) + 1)
        d = heightfield_scene(grid=g, spheres=8, sphere_freq=f, env_size=(512, 256), width=512, height=512,
                              seed=seed + 17 * k)
        if k % 2 == 1:
            s_e = d.spectrum_regular(np.array([20.0, 20.0], np.float32), 360.0, 830.0)
            s_s = d.spectrum_regular(np.array([18.0, 18.0], np.float32), 360.0, 830.0)
            if density is None:
                density = fbm_density_grid(256, seed)
            d.medium = Medium((-1.0, -0.25, -1.0), (1.0, 0.15, 1.0), density, s_s, s_e, 0.7)
        out.append(d)
    return out
