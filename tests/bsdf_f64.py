"""Float64 restatement of the reference's non-delta BSDFs, for the condition
numbers behind the BSDF parity test's tolerance.

Restated from the reference (float64 throughout, vectorised over queries):
* the BSDF wrapper's shading-normal correction |d.z / dot(d, n_g)|
  (Core/directional_distribution_functions.h:295-349, non-adjoint);
* LambertianBRDF (BSDF/basic_bsdfs.cpp:13-58) with the concentric-disk
  cosine sampling (Core/distributions.h:30-37, distributions.cpp:59-94);
* MicrofacetBRDF (BSDF/microfacet_bsdfs.cpp:11-113) with FresnelConductor
  (Core/directional_distribution_functions.cpp:118-138);
* MicrofacetBSDF (BSDF/microfacet_bsdfs.cpp:116-328) with FresnelDielectric
  (directional_distribution_functions.cpp:142-211);
* GGXMicrofacetDistribution: D, Smith G1 and visible-normal sampling
  (directional_distribution_functions.cpp:247-315).

A query row is the 16 floats of the BSDF tests (tests/bsdf_cases.py): query
direction (0:3), geometric normal (3:6), selected wavelength (6), uniforms
uComponent, uDir[0], uDir[1] (8:11), evaluation direction (11:14).

The condition numbers are finite-difference sensitivities of each output to
perturbations of the query's inputs, computed here in float64 from the
query alone: the tolerance of a comparison between two FP32
implementations of the same function (the reference's on the CPU and the
GPU's) grows with them, never with the observed GPU error.
"""
from __future__ import annotations

import numpy as np

from tests.bsdf_conditioning import _fresnel, _ggx_d, _ggx_g1, microfacet_bsdf

KINDS_RESTATED = ("lambert", "ggx_brdf", "ggx_bsdf")


def _norm(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _importance(s, wl):
    """SampledSpectrum::importance (spectrum_types.h:473-486): 0.9 on the
    selected wavelength, 0.1 spread over the other 15."""
    idx = np.arange(len(s))
    return s.sum(1) * (0.1 / 15) + s[idx, wl] * (0.9 - 0.1 / 15)


def _snc(d, ng):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.abs(d[:, 2] / (d * ng).sum(1))


def _concentric_disk(u0, u1):
    sx, sy = 2 * u0 - 1, 2 * u1 - 1
    r = np.zeros_like(sx)
    th = np.zeros_like(sx)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = (sx >= -sy) & (sx > sy)
        b = (sx >= -sy) & ~(sx > sy)
        c = (sx < -sy) & (sx <= sy)
        d = (sx < -sy) & (sx > sy)
        r = np.where(a, sx, np.where(b, sy, np.where(c, -sx, -sy)))
        th = np.where(a, sy / sx, np.where(b, 2 - sx / sy, np.where(c, 4 + sy / sx, 6 + sx / sy)))
    th = th * (np.pi / 4)
    zero = (sx == 0) & (sy == 0)
    return np.where(zero, 0.0, r * np.cos(th)), np.where(zero, 0.0, r * np.sin(th))


def _fresnel_conductor(c, eta, k):
    c = np.abs(c)[:, None]
    c2 = c * c
    two = 2 * eta[None] * c
    tf = eta[None] ** 2 + k[None] ** 2
    t = tf * c2
    rpar = (t - two + 1) / (t + two + 1)
    rper = (tf - two + c2) / (tf + two + c2)
    return (rpar + rper) / 2


def _vndf(v, u0, u1, ax, ay):
    sv = _norm(np.stack([ax * v[:, 0], ay * v[:, 1], v[:, 2]], 1))
    dist = np.sqrt(sv[:, 0] ** 2 + sv[:, 1] ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = np.where((sv[:, 2] < 0.9999)[:, None], np.stack([sv[:, 1] / dist, -sv[:, 0] / dist, 0 * dist], 1),
                      np.array([1.0, 0.0, 0.0]))
    t2 = np.stack([t1[:, 1] * sv[:, 2], -t1[:, 0] * sv[:, 2], dist], 1)
    a = 1 / (1 + sv[:, 2])
    r = np.sqrt(u0)
    lower = u1 < a
    with np.errstate(divide="ignore", invalid="ignore"):
        phi = np.pi * np.where(lower, u1 / a, 1 + (u1 - a) / (1 - a))
    p1 = r * np.cos(phi)
    p2 = r * np.sin(phi) * np.where(lower, 1.0, sv[:, 2])
    m = p1[:, None] * t1 + p2[:, None] * t2 + np.sqrt(np.maximum(0.0, 1 - p1 * p1 - p2 * p2))[:, None] * sv
    return _norm(np.stack([ax * m[:, 0], ay * m[:, 1], m[:, 2]], 1))


def _mpdf(v, m, ax, ay):
    with np.errstate(divide="ignore", invalid="ignore"):
        return _ggx_g1(v, m, ax, ay) * np.abs((v * m).sum(1)) * _ggx_d(m, ax, ay) / np.abs(v[:, 2])


def sample(kind, spec0, spec1, ax, ay, q):
    """(fs (n, 16) with the shading-normal correction, direction (n, 3), pdf
    (n,), ok (n,)) of BSDF::sample at the queries' uniforms."""
    q = np.asarray(q, np.float64)
    wo, ng, wl = q[:, 0:3], q[:, 3:6], q[:, 6].astype(int)
    uc, u0, u1 = q[:, 8], q[:, 9], q[:, 10]
    n = len(q)
    s0, s1 = np.asarray(spec0, np.float64), np.asarray(spec1, np.float64)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        if kind == "lambert":
            x, y = _concentric_disk(u0, u1)
            d = np.stack([x, y, np.sqrt(np.maximum(0.0, 1 - x * x - y * y))], 1)
            pdf = d[:, 2] / np.pi
            d[:, 2] *= np.where(wo[:, 2] > 0, 1.0, -1.0)
            fs = np.broadcast_to(s0 / np.pi, (n, 16)).copy()
            ok = pdf > 0
        else:
            sign = np.where(wo[:, 2] >= 0, 1.0, -1.0)
            m = _vndf(sign[:, None] * wo, u0, u1, ax, ay)
            dm = _ggx_d(m, ax, ay)
            mpdf = _mpdf(sign[:, None] * wo, m, ax, ay)
            hv = (wo * m).sum(1)
            ok = hv * sign > 0
            refl_d = 2 * hv[:, None] * m - wo
            if kind == "ggx_brdf":
                d = refl_d
                ok &= d[:, 2] * wo[:, 2] > 0
                pdf = mpdf / (4 * hv * sign)
                g = _ggx_g1(wo, m, ax, ay) * _ggx_g1(d, m, ax, ay)
                fs = _fresnel_conductor(hv, s0, s1) * (dm * g / (4 * wo[:, 2] * d[:, 2]))[:, None]
            else:
                idx = np.arange(n)
                fall = _fresnel(hv[:, None], s0[None], s1[None])
                rp = _importance(fall, wl)
                reflect = uc < rp
                e_en = np.where((sign > 0)[:, None], s0[None], s1[None])
                e_ex = np.where((sign > 0)[:, None], s1[None], s0[None])
                een, eex = e_en[idx, wl], e_ex[idx, wl]
                rel = een / eex
                inner = 1 + rel * rel * (hv * hv - 1)
                trans_d = (rel * hv - sign * np.sqrt(np.maximum(inner, 0)))[:, None] * m - rel[:, None] * wo
                d = np.where(reflect[:, None], refl_d, trans_d)
                ok &= np.where(reflect, d[:, 2] * wo[:, 2] > 0, (inner >= 0) & (d[:, 2] * wo[:, 2] < 0))
                hl = (d * m).sum(1)
                g = _ggx_g1(wo, m, ax, ay) * _ggx_g1(d, m, ax, ay)
                pdf_r = rp / (4 * hv * sign) * mpdf
                pdf_t = (1 - rp) / (een * hv + eex * hl) ** 2 * mpdf * eex * eex * np.abs(hl)
                pdf = np.where(reflect, pdf_r, pdf_t)
                fs_r = fall * (dm * g / (4 * wo[:, 2] * d[:, 2]))[:, None]
                fs_t, _ = microfacet_bsdf(wo, d, wl, s0, s1, ax, ay)   # per-wavelength transmission value
                fs = np.where(reflect[:, None], fs_r, fs_t)
        fs = fs * _snc(d, ng)[:, None]
    return fs, d, pdf, ok & np.isfinite(pdf) & (pdf > 0)


def evaluate(kind, spec0, spec1, ax, ay, q):
    """(fs (n, 16) with the shading-normal correction, pdf (n,)) of
    BSDF::evaluate / evaluatePDF at the queries' evaluation directions."""
    q = np.asarray(q, np.float64)
    wo, ng, wl, wi = q[:, 0:3], q[:, 3:6], q[:, 6].astype(int), q[:, 11:14]
    n = len(q)
    s0, s1 = np.asarray(spec0, np.float64), np.asarray(spec1, np.float64)
    same = wo[:, 2] * wi[:, 2] > 0
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        if kind == "lambert":
            fs = np.where(same[:, None], s0[None] / np.pi, 0.0) * np.ones((n, 1))
            pdf = np.where(same, np.abs(wi[:, 2]) / np.pi, 0.0)
        elif kind == "ggx_brdf":
            sign = np.where(wo[:, 2] >= 0, 1.0, -1.0)
            m = sign[:, None] * _norm(wo + wi)
            hv = (wo * m).sum(1)
            g = _ggx_g1(wo, m, ax, ay) * _ggx_g1(wi, m, ax, ay)
            fs = _fresnel_conductor(hv, s0, s1) * (_ggx_d(m, ax, ay) * g / (4 * wo[:, 2] * wi[:, 2]))[:, None]
            fs = np.where(same[:, None], fs, 0.0)
            pdf = np.where(same & (hv * sign > 0), _mpdf(sign[:, None] * wo, m, ax, ay) / (4 * hv * sign), 0.0)
        else:
            fs, pdf = microfacet_bsdf(wo, wi, wl, s0, s1, ax, ay)
        fs = fs * _snc(wi, ng)[:, None]
    return fs, pdf


def _perturb_dir(v, eps, rng):
    return _norm(v + eps * rng.normal(size=v.shape))


def _rel_change(a, b):
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(b != 0, np.abs(a - b) / np.abs(b), np.where(a != 0, np.inf, 0.0))
    return np.nan_to_num(r, nan=np.inf)


def conditions(kind, spec0, spec1, ax, ay, q, eps=1e-7, trials=8, seed=0):
    """Per query: kappa_dir (largest change of the sampled direction per unit
    perturbation of the query direction, the geometric normal, the uniforms
    and the two spectra), kappa_s (largest relative change of the sampled
    value or pdf per unit perturbation) and kappa_e (the same for the
    evaluated value and pdf, perturbing the query and evaluation directions,
    the normal and the spectra).  The spectra are perturbed because an FP32
    evaluation rounds what it derives from them (the index ratio of the
    dielectric's Fresnel term and refraction), which near total internal
    reflection moves the result far more than the rounding of the directions
    does.  Perturbations cross branch boundaries (total internal reflection,
    the hemisphere tests) only where a query lies within about eps of one,
    which then shows as an infinite condition number."""
    q = np.asarray(q, np.float64)
    rng = np.random.default_rng(seed)
    fs0, d0, p0, ok0 = sample(kind, spec0, spec1, ax, ay, q)
    fe0, pe0 = evaluate(kind, spec0, spec1, ax, ay, q)
    kd = np.zeros(len(q))
    ks = np.zeros(len(q))
    ke = np.zeros(len(q))
    for _ in range(trials):
        qp = q.copy()
        qp[:, 0:3] = _perturb_dir(q[:, 0:3], eps, rng)
        qp[:, 3:6] = _perturb_dir(q[:, 3:6], eps, rng)
        qp[:, 8:11] = np.clip(q[:, 8:11] + eps * rng.normal(size=(len(q), 3)), 0.0, np.nextafter(1.0, 0.0))
        qp[:, 11:14] = _perturb_dir(q[:, 11:14], eps, rng)
        s0p = np.asarray(spec0, np.float64) * (1.0 + eps * rng.normal(size=16))
        s1p = np.asarray(spec1, np.float64) * (1.0 + eps * rng.normal(size=16))
        fs1, d1, p1, ok1 = sample(kind, s0p, s1p, ax, ay, qp)
        fe1, pe1 = evaluate(kind, s0p, s1p, ax, ay, qp)
        flip = ok1 != ok0
        kd = np.maximum(kd, np.where(flip, np.inf, np.nan_to_num(np.abs(d1 - d0).max(1), nan=np.inf) / eps))
        rs = np.maximum(_rel_change(fs1, fs0).max(1), _rel_change(p1, p0))
        ks = np.maximum(ks, np.where(flip, np.inf, rs / eps))
        re = np.maximum(_rel_change(fe1, fe0).max(1), _rel_change(pe1, pe0))
        ke = np.maximum(ke, re / eps)
    return np.maximum(kd, 1.0), np.maximum(ks, 1.0), np.maximum(ke, 1.0)
