"""Deterministic BSDF query sets for the BSDF parity test.

The setups follow the reference's BSDF test harness
(SLR_Test/bsdf_tests.cpp:72-83): incident directions normal, (1,1,1) and
grazing (z = 0.001) along the tangent and bitangent, mirrored to the lower
hemisphere, times geometric normals (0,0,1), (0.25,0.25,1) and (-1,-1,1);
materials as in bsdf_tests.cpp:245-507 (Lambert, specular conductor,
specular dielectric, GGX conductor with alpha (0.05, 0.2), GGX dielectric).
Named index-of-refraction tables are replaced by smooth synthetic spectra.
"""
from __future__ import annotations

import numpy as np

WL = 360.0 + 470.0 * (np.arange(16) + 0.5) / 16


def _norm(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


INCIDENT = [_norm((0, 0, 1)), _norm((1, 1, 1)), _norm((1, 0, 0.001)), _norm((0, 1, 0.001))]
GNORMALS = [_norm((0, 0, 1)), _norm((0.25, 0.25, 1)), _norm((-1, -1, 1))]


def make_queries(n_per_setup: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    qs = []
    for lower in (False, True):
        for v in INCIDENT:
            d = v.copy()
            if lower:
                d[2] = -d[2]
            for gn in GNORMALS:
                for _ in range(n_per_setup):
                    q = np.zeros(16, np.float32)
                    q[0:3] = d
                    q[3:6] = gn
                    q[6] = rng.integers(0, 16)
                    q[7] = 0
                    q[8:11] = rng.random(3)
                    z = rng.uniform(-1, 1)
                    ph = rng.uniform(0, 2 * np.pi)
                    s = np.sqrt(1 - z * z)
                    # half the evaluation directions near the mirror direction
                    if rng.random() < 0.5:
                        m = np.array([-d[0], -d[1], d[2]]) + 0.3 * np.array([s * np.cos(ph), s * np.sin(ph), z])
                        q[11:14] = _norm(m)
                    else:
                        q[11:14] = (s * np.cos(ph), s * np.sin(ph), z)
                    qs.append(q)
    return np.stack(qs)


def _flat_interpolated(v: float, offset: float) -> np.ndarray:
    """(1 - t) v + t v in float32 at the 16 stratified wavelengths of a path
    with wavelength offset `offset`, t = (lambda - 360) / 470."""
    f = np.float32
    lam = (f(360) + (f(470) * (np.arange(16, dtype=f) + f(offset))).astype(f) * f(0.0625)).astype(f)
    x = (lam - f(360)).astype(f)
    # x / 470 correctly rounded, as the renderer computes it (one FMA-refined quotient)
    z = f(1.0 / 470.0)
    q = (x * z).astype(f)
    r = (x.astype(np.float64) - q.astype(np.float64) * 470.0).astype(f)
    t = (r.astype(np.float64) * np.float64(z) + q.astype(np.float64)).astype(f)
    return (((f(1) - t).astype(f) * f(v)).astype(f) + (t * f(v)).astype(f)).astype(f)


def bsdf_cases(n_per_setup: int = 64):
    eta_al = (1.2 + 0.4 * (WL - 360) / 470).astype(np.float32)
    k_al = (8.0 - 2.0 * (WL - 360) / 470).astype(np.float32)
    ones = np.ones(16, np.float32)
    diamond = (2.38 + 1.5e4 / (WL * WL)).astype(np.float32)  # Cauchy-like dispersion
    glass = (1.5 + 4.0e3 / (WL * WL)).astype(np.float32)
    refl = (0.3 + 0.5 * np.sin(WL / 60.0) ** 2).astype(np.float32)
    # a flat index spectrum as a path sees it: the two-sample regular spectrum
    # (v, v) over 360-830 nm interpolated in float32 at one path's 16
    # wavelengths, which rounds some of them one unit in the last place away
    # from v (two or three distinct index pairs, the GPU's pair path)
    flat_ext, flat_int = _flat_interpolated(1.0, 0.03), _flat_interpolated(1.45, 0.03)
    cases = [
        dict(name="lambert", kind="lambert", spec0=refl),
        dict(name="specular_brdf", kind="specular_brdf", spec0=(0.9 * ones).astype(np.float32), spec1=eta_al, spec2=k_al),
        dict(name="specular_bsdf", kind="specular_bsdf", spec0=ones, spec1=ones, spec2=glass),
        dict(name="ggx_brdf_aniso", kind="ggx_brdf", spec0=eta_al, spec1=k_al, ax=0.05, ay=0.2),
        dict(name="ggx_brdf_rough", kind="ggx_brdf", spec0=eta_al, spec1=k_al, ax=0.5, ay=0.5),
        dict(name="ggx_bsdf_diamond", kind="ggx_bsdf", spec0=ones, spec1=diamond, ax=0.05, ay=0.2),
        dict(name="ggx_bsdf_glass", kind="ggx_bsdf", spec0=ones, spec1=glass, ax=0.3, ay=0.3),
        dict(name="ggx_bsdf_flat", kind="ggx_bsdf", spec0=flat_ext, spec1=flat_int, ax=0.3, ay=0.3),
    ]
    for i, c in enumerate(cases):
        c["queries"] = make_queries(n_per_setup, seed=100 + i)
    return cases
