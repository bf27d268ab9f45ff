"""Float64 restatement of the GGX dielectric BSDF's value and pdf
(MicrofacetBSDF, libSLR/BSDF/microfacet_bsdfs.cpp:213-300), with the
dielectric Fresnel term (Core/directional_distribution_functions.cpp:142-211)
and the GGX normal distribution and Smith G1 (:262-315); tests/bsdf_f64.py
builds the other BSDFs and the condition numbers on it.  Near total internal
reflection the factor (1 - F) cancels and the exit cosine sqrt(1 - sin^2)
loses digits, so an FP32 evaluation, on any hardware, carries relative
errors far above 1e-5 there.
"""
from __future__ import annotations

import numpy as np


def _normalize(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _fresnel(cos_enter, e_ext, e_int):
    c = np.clip(cos_enter, -1.0, 1.0)
    entering = c > 0
    e_en = np.where(entering, e_ext, e_int)
    e_ex = np.where(entering, e_int, e_ext)
    sin_ex = e_en / e_ex * np.sqrt(np.maximum(0.0, 1.0 - c * c))
    c = np.abs(c)
    cos_ex = np.sqrt(np.maximum(0.0, 1.0 - sin_ex * sin_ex))
    with np.errstate(divide="ignore", invalid="ignore"):
        rpar = (e_ex * c - e_en * cos_ex) / (e_ex * c + e_en * cos_ex)
        rper = (e_en * c - e_ex * cos_ex) / (e_en * c + e_ex * cos_ex)
        f = (rpar * rpar + rper * rper) / 2.0
    return np.where(sin_ex >= 1.0, 1.0, f)


def _ggx_d(m, ax, ay):
    t = m[..., 0] ** 2 / ax ** 2 + m[..., 1] ** 2 / ay ** 2 + m[..., 2] ** 2
    with np.errstate(divide="ignore"):
        d = 1.0 / (np.pi * ax * ay * t * t)
    return np.where(m[..., 2] <= 0, 0.0, d)


def _ggx_g1(v, m, ax, ay):
    with np.errstate(divide="ignore", invalid="ignore"):
        chi = ((v * m).sum(-1) / v[..., 2]) > 0
        t = (v[..., 0] ** 2 * ax * ax + v[..., 1] ** 2 * ay * ay) / (v[..., 2] ** 2)
        return np.where(chi, 2.0 / (1.0 + np.sqrt(1.0 + t)), 0.0)


def microfacet_bsdf(wo, wi, wl, e_ext, e_int, ax, ay):
    """fs (n, 16) and pdf (n,) of MicrofacetBSDF::evaluateInternal /
    evaluatePDFInternal for local directions wo (query), wi (n, 3), selected
    wavelength index wl (n,) and indices of refraction (16,)."""
    n = len(wo)
    e_ext = np.broadcast_to(np.asarray(e_ext, np.float64), (n, 16))
    e_int = np.broadcast_to(np.asarray(e_int, np.float64), (n, 16))
    entering = wo[:, 2] >= 0
    sign = np.where(entering, 1.0, -1.0)
    dd = wi[:, 2] * wo[:, 2]
    e_en = np.where(entering[:, None], e_ext, e_int)
    e_ex = np.where(entering[:, None], e_int, e_ext)
    fs = np.zeros((n, 16))
    with np.errstate(divide="ignore", invalid="ignore"):
        # reflection
        m = sign[:, None] * _normalize(wo + wi)
        hv = (wo * m).sum(1)
        refl = _fresnel(hv[:, None], e_ext, e_int) * (_ggx_d(m, ax, ay) * _ggx_g1(wo, m, ax, ay) *
                                                      _ggx_g1(wi, m, ax, ay) / (4 * dd))[:, None]
        # transmission, per wavelength
        mw = _normalize(-(e_en[:, :, None] * wo[:, None, :] + e_ex[:, :, None] * wi[:, None, :]))
        hvw = (wo[:, None, :] * mw).sum(-1)
        hlw = (wi[:, None, :] * mw).sum(-1)
        fw = _fresnel(hvw, e_ext, e_int)
        gw = _ggx_g1(np.broadcast_to(wo[:, None, :], mw.shape), mw, ax, ay) * \
            _ggx_g1(np.broadcast_to(wi[:, None, :], mw.shape), mw, ax, ay)
        trans = np.abs(hvw * hlw) * (1 - fw) * gw * _ggx_d(mw, ax, ay) / (e_en * hvw + e_ex * hlw) ** 2
        trans = trans / np.abs(dd)[:, None] * e_en * e_en
        fs = np.where((dd > 0)[:, None], refl, np.where((dd < 0)[:, None], trans, 0.0))
        # pdf at the selected wavelength
        idx = np.arange(n)
        een, eex = e_en[idx, wl], e_ex[idx, wl]
        mp = np.where((dd > 0)[:, None], sign[:, None] * _normalize(wo + wi),
                      _normalize(-(een[:, None] * wo + eex[:, None] * wi)))
        hv = (wo * mp).sum(1)
        hl = (wi * mp).sum(1)
        sv = sign[:, None] * wo
        mpdf = _ggx_g1(sv, mp, ax, ay) * np.abs((sv * mp).sum(1)) * _ggx_d(mp, ax, ay) / np.abs(sv[:, 2])
        # reflection probability: SampledSpectrum::importance(wl) of F
        # (spectrum_types.h:473-483), 0.9 on the selected wavelength
        fall = _fresnel(hv[:, None], e_ext, e_int)
        fr = fall.sum(1) * (0.1 / 15) + fall[idx, wl] * (0.9 - 0.1 / 15)
        pdf_r = fr / (4 * hv * sign) * mpdf
        pdf_t = (1 - fr) / (een * hv + eex * hl) ** 2 * mpdf * eex * eex * np.abs(hl)
        pdf = np.where(dd > 0, pdf_r, pdf_t)
        pdf = np.where((hv * sign <= 0) | (dd == 0), 0.0, pdf)
    return fs, pdf
