// BSDFs with reverse quantities and adjoint transport, as bidirectional path
// tracing queries them (BSDFQuery with requestReverse, adjoint:
// libSLR/Core/directional_distribution_functions.h:154-160, 295-349).
//
// For a query direction wo and a second direction wi the reference returns,
// besides the forward value f(wo -> wi) and pdf p(wi | wo), the reverse
// value and pdf (those of sampling wo from wi).  Adjoint queries (light
// subpaths) change two things: the shading-normal correction uses the query
// direction instead of the sampled one, and refraction carries the
// (eExit / eEnter)^2 factor the other way.  The reference multiplies the
// reverse value by the forward shading-normal correction; so does this code.
#pragma once
#include "device_bsdf.cuh"

namespace slrgpu {

struct RevQuery {
    V3 dir;        // query direction (toward the previous vertex), shading frame
    V3 gn;         // geometric normal, shading frame
    int wl;        // selected wavelength index
    bool adjoint;  // light subpath
};

__device__ __forceinline__ float snCorrection(const RevQuery &q, V3 other) {
    return q.adjoint ? fabsf(q.dir.z / dot(q.dir, q.gn)) : fabsf(other.z / dot(other, q.gn));
}

// Sampling (basic_bsdfs.cpp:13-153, microfacet_bsdfs.cpp:11-211).  res->pdf
// == 0 on failure; on success fs and revFs carry the shading-normal
// correction.
static __device__ __noinline__ void bsdfSampleRev(const Bsdf &B, const RevQuery &q, float uc, float u0, float u1,
                                           BsdfSample* res, Spec &fs, float* revPdf, Spec &revFs) {
    res->pdf = 0.0f;
    res->type = 0;
    res->dir = V3{0, 0, 1};
    *revPdf = 0.0f;
    fs = specConst(0.0f);
    revFs = specConst(0.0f);
    switch (B.kind) {
    case kMatMatte: {
        V3 d = cosineSampleHemisphere(u0, u1);
        res->pdf = d.z * kInvPiF;
        res->type = kDirReflection | kDirLowFreq;
        d.z *= q.dir.z > 0 ? 1.0f : -1.0f;
        res->dir = d;
        specScale(B.a, 1.0f / kPiF, fs);
        revFs = fs;
        *revPdf = fabsf(q.dir.z) * kInvPiF;
        break;
    }
    case kMatSpecularReflection: {
        res->dir = V3{-q.dir.x, -q.dir.y, q.dir.z};
        res->pdf = 1.0f;
        res->type = kDirReflection | kDirDelta0D;
        Spec F;
        fresnelConductorFor<kMatSpecularReflection>(B, B.b, B.c, q.dir.z, F);
        float r = 1.0f / fabsf(q.dir.z);
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) fs.v[i] = (B.a.v[i] * F.v[i]) * r;
        revFs = fs;
        *revPdf = 1.0f;
        break;
    }
    case kMatSpecularScattering: {
        Spec F;
        fresnelDielectricFor<kMatSpecularScattering>(B, B.b, B.c, q.dir.z, F);
        float reflectProb = importance(F, q.wl);
        if (uc < reflectProb) {
            if (q.dir.z == 0.0f) return;
            res->dir = V3{-q.dir.x, -q.dir.y, q.dir.z};
            res->pdf = reflectProb;
            res->type = kDirReflection | kDirDelta0D;
            float r = 1.0f / fabsf(q.dir.z);
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) fs.v[i] = (B.a.v[i] * F.v[i]) * r;
            revFs = fs;
            *revPdf = reflectProb;
            break;
        }
        bool entering = q.dir.z > 0.0f;
        float eExtW = specAt(B.b, q.wl), eIntW = specAt(B.c, q.wl);
        float eEnter = entering ? eExtW : eIntW;
        float eExit = entering ? eIntW : eExtW;
        float sinEnter2 = 1.0f - q.dir.z * q.dir.z;
        float rrEta = eEnter / eExit;
        float sinExit2 = rrEta * rrEta * sinEnter2;
        if (sinExit2 >= 1.0f) return;
        float cosExit = sqrtf(fmaxf(0.0f, 1.0f - sinExit2));
        if (entering) cosExit = -cosExit;
        res->dir = V3{rrEta * -q.dir.x, rrEta * -q.dir.y, cosExit};
        res->pdf = 1.0f - reflectProb;
        res->type = kDirTransmission | kDirDelta0D | (B.dispersive ? kDirDispersive : 0u);
        float val = specAt(B.a, q.wl) * (1.0f - specAt(F, q.wl));
        float rev = val / fabsf(q.dir.z);
        if (q.adjoint) rev *= (eExit * eExit) / (eEnter * eEnter);
        *revPdf = 1.0f - reflectProb;
        if (!q.adjoint) val *= (eEnter * eEnter) / (eExit * eExit);
        float r = 1.0f / fabsf(cosExit);
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) {
            fs.v[i] = (i == q.wl) ? val * r : 0.0f;
            revFs.v[i] = (i == q.wl) ? rev : 0.0f;
        }
        break;
    }
    case kMatGGXReflection: {
        bool entering = q.dir.z >= 0.0f;
        float sign = entering ? 1.0f : -1.0f;
        V3 m;
        float mPdf;
        float D = ggxSample(B.ax, B.ay, sign * q.dir, u0, u1, &m, &mPdf);
        float dotHV = dot(q.dir, m);
        if (dotHV * sign <= 0) return;
        V3 d = (2 * dotHV) * m - q.dir;
        if (d.z * q.dir.z <= 0) return;
        float common = 1.0f / (4 * dotHV * sign);
        res->dir = d;
        res->pdf = common * mPdf;
        res->type = kDirReflection | kDirHighFreq;
        Spec F;
        fresnelConductorFor<kMatGGXReflection>(B, B.a, B.b, dotHV, F);
        float G = ggxG1(B.ax, B.ay, q.dir, m) * ggxG1(B.ax, B.ay, d, m);
        float r = 1.0f / (4 * q.dir.z * d.z);
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) fs.v[i] = ((F.v[i] * D) * G) * r;
        *revPdf = common * ggxPdf(B.ax, B.ay, sign * d, m);
        revFs = fs;
        break;
    }
    case kMatGGXScattering: {
        bool entering = q.dir.z >= 0.0f;
        float sign = entering ? 1.0f : -1.0f;
        V3 m;
        float mPdf;
        float D = ggxSample(B.ax, B.ay, sign * q.dir, u0, u1, &m, &mPdf);
        float dotHV = dot(q.dir, m);
        if (dotHV * sign <= 0 || isnan(D)) return;
        Spec F;
        fresnelDielectricFor<kMatGGXScattering>(B, B.a, B.b, dotHV, F);
        float reflectProb = importance(F, q.wl);
        if (uc < reflectProb) {
            V3 d = (2 * dotHV) * m - q.dir;
            if (d.z * q.dir.z <= 0) return;
            float common = reflectProb / (4 * dotHV * sign);
            res->dir = d;
            res->pdf = common * mPdf;
            res->type = kDirReflection | kDirHighFreq;
            float G = ggxG1(B.ax, B.ay, q.dir, m) * ggxG1(B.ax, B.ay, d, m);
            float r = 1.0f / (4 * q.dir.z * d.z);
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) fs.v[i] = ((F.v[i] * D) * G) * r;
            *revPdf = common * ggxPdf(B.ax, B.ay, sign * d, m);
            revFs = fs;
            break;
        }
        float eExtW = specAt(B.a, q.wl), eIntW = specAt(B.b, q.wl);
        float eEnterW = entering ? eExtW : eIntW;
        float eExitW = entering ? eIntW : eExtW;
        float recRelIOR = eEnterW / eExitW;
        float innerRoot = 1 + recRelIOR * recRelIOR * (dotHV * dotHV - 1);
        if (innerRoot < 0) return;
        V3 d = (recRelIOR * dotHV - sign * sqrtf(innerRoot)) * m - recRelIOR * q.dir;
        if (d.z * q.dir.z >= 0) return;
        float dotHL = dot(d, m);
        float den = eEnterW * dotHV + eExitW * dotHL;
        float common = (1 - reflectProb) / (den * den);
        res->dir = d;
        res->pdf = common * mPdf * eExitW * eExitW * fabsf(dotHL);
        res->type = kDirTransmission | kDirHighFreq;
        float r = 1.0f / fabsf(q.dir.z * d.z);
        ggxTransmitPairs(B, entering, q.dir, d, r, fs, q.adjoint);
        *revPdf = common * ggxPdf(B.ax, B.ay, -sign * d, m) * eEnterW * eEnterW * fabsf(dotHV);
        revFs = fs;
        break;
    }
    default:
        return;
    }
    if (res->pdf == 0.0f) return;
    const float sn = snCorrection(q, res->dir);
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) {
        fs.v[i] *= sn;
        revFs.v[i] *= sn;
    }
}

// Evaluation with the reverse value (basic_bsdfs.cpp:28-39, microfacet_bsdfs.cpp:48-72, 213-265).
static __device__ __noinline__ void bsdfEvalRev(const Bsdf &B, const RevQuery &q, V3 dir, Spec &fs, Spec &revFs) {
    fs = specConst(0.0f);
    switch (B.kind) {
    case kMatMatte:
        if (q.dir.z * dir.z > 0.0f) specScale(B.a, 1.0f / kPiF, fs);
        break;
    case kMatGGXReflection: {
        if (dir.z * q.dir.z <= 0) break;
        float sign = q.dir.z >= 0.0f ? 1.0f : -1.0f;
        V3 m = sign * normalize(q.dir + dir);
        float dotHV = dot(q.dir, m);
        float D = ggxD(B.ax, B.ay, m);
        Spec F;
        fresnelConductorFor<kMatGGXReflection>(B, B.a, B.b, dotHV, F);
        float G = ggxG1(B.ax, B.ay, q.dir, m) * ggxG1(B.ax, B.ay, dir, m);
        float r = 1.0f / (4 * q.dir.z * dir.z);
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) fs.v[i] = ((F.v[i] * D) * G) * r;
        break;
    }
    case kMatGGXScattering: {
        bool entering = q.dir.z >= 0.0f;
        float sign = entering ? 1.0f : -1.0f;
        float dNVNL = dir.z * q.dir.z;
        if (dNVNL > 0) {
            V3 m = sign * normalize(q.dir + dir);
            float dotHV = dot(q.dir, m);
            float D = ggxD(B.ax, B.ay, m);
            Spec F;
            fresnelDielectricFor<kMatGGXScattering>(B, B.a, B.b, dotHV, F);
            float G = ggxG1(B.ax, B.ay, q.dir, m) * ggxG1(B.ax, B.ay, dir, m);
            float r = 1.0f / (4 * dNVNL);
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) fs.v[i] = ((F.v[i] * D) * G) * r;
        } else if (dNVNL < 0) {
            float r = 1.0f / fabsf(dNVNL);
            ggxTransmitPairs(B, entering, q.dir, dir, r, fs, q.adjoint);
        }
        break;
    }
    default:  // delta BSDFs evaluate to zero
        break;
    }
    const float sn = snCorrection(q, dir);
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) {
        fs.v[i] *= sn;
        revFs.v[i] = fs.v[i];
    }
}

// Density with the reverse density (basic_bsdfs.cpp:41-50, microfacet_bsdfs.cpp:74-102, 267-318).
static __device__ __noinline__ float bsdfPdfRev(const Bsdf &B, const RevQuery &q, V3 dir, float* revPdf) {
    *revPdf = 0.0f;
    switch (B.kind) {
    case kMatMatte:
        if (q.dir.z * dir.z <= 0.0f) return 0.0f;
        *revPdf = fabsf(q.dir.z) * kInvPiF;
        return fabsf(dir.z) * kInvPiF;
    case kMatGGXReflection: {
        if (dir.z * q.dir.z <= 0) return 0.0f;
        float sign = q.dir.z >= 0.0f ? 1.0f : -1.0f;
        V3 m = sign * normalize(q.dir + dir);
        float dotHV = dot(q.dir, m);
        if (dotHV * sign <= 0) return 0.0f;
        float mPdf = ggxPdf(B.ax, B.ay, sign * q.dir, m);
        float common = 1.0f / (4 * dotHV * sign);
        *revPdf = common * ggxPdf(B.ax, B.ay, sign * dir, m);
        return common * mPdf;
    }
    case kMatGGXScattering: {
        bool entering = q.dir.z >= 0.0f;
        float sign = entering ? 1.0f : -1.0f;
        float dNVNL = dir.z * q.dir.z;
        if (dNVNL == 0) return 0.0f;
        float eExtW = specAt(B.a, q.wl), eIntW = specAt(B.b, q.wl);
        float eEnterW = entering ? eExtW : eIntW;
        float eExitW = entering ? eIntW : eExtW;
        V3 m = dNVNL > 0 ? sign * normalize(q.dir + dir) : normalize(-(eEnterW * q.dir + eExitW * dir));
        float dotHV = dot(q.dir, m);
        if (dotHV * sign <= 0) return 0.0f;
        float mPdf = ggxPdf(B.ax, B.ay, sign * q.dir, m);
        Spec F;
        fresnelDielectricFor<kMatGGXScattering>(B, B.a, B.b, dotHV, F);
        float reflectProb = importance(F, q.wl);
        if (dNVNL > 0) {
            float common = reflectProb / (4 * dotHV * sign);
            *revPdf = common * ggxPdf(B.ax, B.ay, sign * dir, m);
            return common * mPdf;
        }
        float dotHL = dot(dir, m);
        float den = eEnterW * dotHV + eExitW * dotHL;
        float common = (1 - reflectProb) / (den * den);
        *revPdf = common * ggxPdf(B.ax, B.ay, -sign * dir, m) * eEnterW * eEnterW * fabsf(dotHV);
        return common * mPdf * eExitW * eExitW * fabsf(dotHL);
    }
    default:
        return 0.0f;
    }
}

}  // namespace slrgpu
