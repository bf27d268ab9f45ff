// BSDFs on the device: Lambert, specular reflection / scattering, GGX
// microfacet reflection / scattering with visible-normal sampling, and the
// shading-normal correction of the reference's BSDF wrapper
// (libSLR/Core/directional_distribution_functions.h:295-349).  Non-adjoint
// queries with the "All" direction filter, which is what the path tracers use.
#pragma once
#include "device_common.cuh"

namespace slrgpu {

// DirectionType bits (directional_distribution_functions.h:18-50).
constexpr uint32_t kDirLowFreq = 1u << 0;
constexpr uint32_t kDirHighFreq = 1u << 1;
constexpr uint32_t kDirDelta0D = 1u << 2;
constexpr uint32_t kDirDelta1D = 1u << 3;
constexpr uint32_t kDirReflection = 1u << 4;
constexpr uint32_t kDirTransmission = 1u << 5;
constexpr uint32_t kDirDispersive = 1u << 6;
constexpr uint32_t kDirNonDelta = kDirLowFreq | kDirHighFreq;
constexpr uint32_t kDirDelta = kDirDelta0D | kDirDelta1D;

__device__ __forceinline__ bool dirIsDelta(uint32_t t) { return (t & kDirDelta) && !(t & kDirNonDelta); }

struct Bsdf {
    uint32_t kind;
    Spec a, b, c;          // see MaterialKind
    float ax, ay;
    bool dispersive;       // SpecularBSDF built while no wavelength is selected
    // Fresnel-pair kinds (prepareIorPairs): the slot of each wavelength's
    // index pair, 2 bits each, the number of slots (0: evaluate every
    // wavelength) and the pairs of the slots
    uint32_t iorSlots, iorCount;
    float iorX[4], iorY[4];
};

struct BsdfQuery {
    V3 dir;                // outgoing direction in the shading frame
    V3 gn;                 // geometric normal in the shading frame
    int wl;                // selected wavelength index
};

struct BsdfSample {
    V3 dir;
    float pdf;
    uint32_t type;
};

__device__ __forceinline__ bool bsdfHasNonDelta(uint32_t kind) {
    return kind == kMatMatte || kind == kMatGGXReflection || kind == kMatGGXScattering;
}

// ---- sampling helpers (distributions.cpp:59-91, distributions.h:30-73) ----
__device__ __forceinline__ void concentricSampleDisk(float u0, float u1, float* dx, float* dy) {
    float r, theta;
    float sx = 2 * u0 - 1;
    float sy = 2 * u1 - 1;
    if (sx == 0 && sy == 0) { *dx = 0; *dy = 0; return; }
    if (sx >= -sy) {
        if (sx > sy) { r = sx; theta = sy / sx; }
        else { r = sy; theta = 2 - sx / sy; }
    } else {
        if (sx > sy) { r = -sy; theta = 6 + sx / sy; }
        else { r = -sx; theta = 4 + sy / sx; }
    }
    theta *= 0.785398163397448309616f;
    float s, c;
    sincosf(theta, &s, &c);
    *dx = r * c;
    *dy = r * s;
}

__device__ __forceinline__ V3 cosineSampleHemisphere(float u0, float u1) {
    float x, y;
    concentricSampleDisk(u0, u1, &x, &y);
    return V3{x, y, sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y))};
}

// ---- Fresnel (directional_distribution_functions.cpp:118-211) ----
__device__ __forceinline__ float fresnelConductor1(float eta, float k, float cosEnter) {
    cosEnter = fabsf(cosEnter);
    float c2 = cosEnter * cosEnter;
    float twoEtaCos = 2.0f * eta * cosEnter;
    float tmpF = eta * eta + k * k;
    float tmp = tmpF * c2;
    float rparl2 = (tmp - twoEtaCos + 1) / (tmp + twoEtaCos + 1);
    float rperp2 = (tmpF - twoEtaCos + c2) / (tmpF + twoEtaCos + c2);
    return (rparl2 + rperp2) * 0.5f;
}

__device__ __forceinline__ float fresnelEvalF(float etaEnter, float etaExit, float cosEnter, float cosExit) {
    float rparl = ((etaExit * cosEnter) - (etaEnter * cosExit)) / ((etaExit * cosEnter) + (etaEnter * cosExit));
    float rperp = ((etaEnter * cosEnter) - (etaExit * cosExit)) / ((etaEnter * cosEnter) + (etaExit * cosExit));
    return (rparl * rparl + rperp * rperp) * 0.5f;
}

__device__ __forceinline__ float fresnelDielectric1(float etaExt, float etaInt, float cosEnter) {
    cosEnter = fminf(fmaxf(cosEnter, -1.0f), 1.0f);
    bool entering = cosEnter > 0.0f;
    float eEnter = entering ? etaExt : etaInt;
    float eExit = entering ? etaInt : etaExt;
    float sinExit = eEnter / eExit * sqrtf(fmaxf(0.0f, 1.0f - cosEnter * cosEnter));
    cosEnter = fabsf(cosEnter);
    if (sinExit >= 1.0f) return 1.0f;
    float cosExit = sqrtf(fmaxf(0.0f, 1.0f - sinExit * sinExit));
    return fresnelEvalF(eEnter, eExit, cosEnter, cosExit);
}

__device__ __forceinline__ void fresnelConductor(const Spec &eta, const Spec &k, float cosEnter, Spec &out) {
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) out.v[i] = fresnelConductor1(eta.v[i], k.v[i], cosEnter);
}

__device__ __forceinline__ void fresnelDielectric(const Spec &etaExt, const Spec &etaInt, float cosEnter, Spec &out) {
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) out.v[i] = fresnelDielectric1(etaExt.v[i], etaInt.v[i], cosEnter);
}

// ---- distinct index pairs of a BSDF's Fresnel spectra ----
// The Fresnel terms take a pair of spectra per wavelength: (eta, k) of a
// conductor, (exterior, interior) indices of a dielectric.  A spectrum that
// is flat in the scene description still differs between the 16 wavelengths
// by the rounding of its interpolation (one unit in the last place either
// way), so a path sees two or three distinct pairs.  prepareIorPairs finds
// them, bit for bit, up to kIorPairSlots, when the BSDF is made;
// evalIorPairs then evaluates a per-wavelength term once per distinct pair
// and hands its value to every wavelength of that pair, which is the value
// that wavelength's own evaluation gives.  With more distinct pairs (a
// dispersive medium) every wavelength is evaluated on its own.  The pair
// spectra are (a, b) of the GGX kinds and (b, c) of the specular kinds.
#ifndef SLRGPU_IOR_PAIRS
#define SLRGPU_IOR_PAIRS 1
#endif
// material kinds that look for pairs (bit = MaterialKind)
#ifndef SLRGPU_IOR_PAIR_KINDS
#define SLRGPU_IOR_PAIR_KINDS 0x10u
#endif
#ifndef SLRGPU_IOR_PAIR_SLOTS
#define SLRGPU_IOR_PAIR_SLOTS 4
#endif
// shape of the dielectric Fresnel loop when the pairs do not fit
#ifndef SLRGPU_IOR_FRESNEL_UNROLL
#define SLRGPU_IOR_FRESNEL_UNROLL 1
#endif
constexpr int kIorPairSlots = SLRGPU_IOR_PAIR_SLOTS;
static_assert(kIorPairSlots >= 1 && kIorPairSlots <= 4, "pair slots take 2 bits per wavelength");

__device__ __forceinline__ void prepareIorPairs(Bsdf &B, const Spec &X, const Spec &Y) {
    uint32_t kx[4] = {0, 0, 0, 0}, ky[4] = {0, 0, 0, 0};
    uint32_t n = 0, slots = 0;
    bool fits = SLRGPU_IOR_PAIRS != 0;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) {
        const uint32_t x = __float_as_uint(X.v[i]), y = __float_as_uint(Y.v[i]);
        uint32_t s = kIorPairSlots;
#pragma unroll
        for (int k = kIorPairSlots - 1; k >= 0; --k)
            if ((uint32_t)k < n && kx[k] == x && ky[k] == y) s = (uint32_t)k;
        if (s == kIorPairSlots) {
            if (n == kIorPairSlots) {
                fits = false;
                s = 0;
            } else {
#pragma unroll
                for (int k = 0; k < kIorPairSlots; ++k)
                    if ((uint32_t)k == n) { kx[k] = x; ky[k] = y; }
                s = n++;
            }
        }
        slots |= s << (2 * i);
    }
    B.iorSlots = slots;
    B.iorCount = fits ? n : 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        B.iorX[k] = __uint_as_float(kx[k]);
        B.iorY[k] = __uint_as_float(ky[k]);
    }
}

// The pair spectra of the BSDF's kind, for the kinds where looking for
// pairs pays (the conductor's Fresnel term costs less than the search).
__device__ __forceinline__ void prepareIorPairs(Bsdf &B) {
    B.iorCount = 0u;
    if (!((SLRGPU_IOR_PAIR_KINDS >> B.kind) & 1u)) return;
    if (B.kind == kMatGGXReflection || B.kind == kMatGGXScattering) prepareIorPairs(B, B.a, B.b);
    else if (B.kind == kMatSpecularReflection || B.kind == kMatSpecularScattering) prepareIorPairs(B, B.b, B.c);
}

// out.v[i] = fn(X.v[i], Y.v[i]) for every wavelength, X and Y the pair
// spectra B was prepared with.  UNROLL picks the shape of the per-wavelength
// loop when the pairs did not fit (unrolled for short terms, rolled for
// long ones).
template <bool UNROLL, class FN>
__device__ __forceinline__ void evalIorPairs(const Bsdf &B, const Spec &X, const Spec &Y, FN fn, Spec &out) {
    const uint32_t n = B.iorCount;
    if (n == 0) {
        if constexpr (UNROLL) {
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) out.v[i] = fn(X.v[i], Y.v[i]);
        } else {
            // the rolled loop indexes a scratch array, not `out`, so that
            // `out` itself can stay in registers
            float tmp[kNumLambda];
#pragma unroll 1
            for (int i = 0; i < kNumLambda; ++i) tmp[i] = fn(X.v[i], Y.v[i]);
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) out.v[i] = tmp[i];
        }
        return;
    }
    float val[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 1
    for (uint32_t j = 0; j < n; ++j) {
        float x = B.iorX[0], y = B.iorY[0];
#pragma unroll
        for (int k = 1; k < kIorPairSlots; ++k)
            if (j == (uint32_t)k) { x = B.iorX[k]; y = B.iorY[k]; }
        const float v = fn(x, y);
#pragma unroll
        for (int k = 0; k < kIorPairSlots; ++k)
            if (j == (uint32_t)k) val[k] = v;
    }
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) {
        const uint32_t s = (B.iorSlots >> (2 * i)) & 3u;
        out.v[i] = s == 0 ? val[0] : s == 1 ? val[1] : s == 2 ? val[2] : val[3];
    }
}

// Whether material kind KIND looks for index pairs (compile time).
template <uint32_t KIND>
constexpr bool kIorPairsFor = SLRGPU_IOR_PAIRS != 0 && ((SLRGPU_IOR_PAIR_KINDS >> KIND) & 1u) != 0;

// fresnelConductor / fresnelDielectric over the pair spectra of B.
__device__ __forceinline__ void fresnelConductorPairs(const Bsdf &B, const Spec &eta, const Spec &k, float cosEnter,
                                                      Spec &F) {
    evalIorPairs<true>(B, eta, k, [cosEnter](float e, float kk) { return fresnelConductor1(e, kk, cosEnter); }, F);
}

__device__ __forceinline__ void fresnelDielectricPairs(const Bsdf &B, const Spec &etaExt, const Spec &etaInt,
                                                       float cosEnter, Spec &F) {
    evalIorPairs<SLRGPU_IOR_FRESNEL_UNROLL != 0>(
        B, etaExt, etaInt, [cosEnter](float eExt, float eInt) { return fresnelDielectric1(eExt, eInt, cosEnter); }, F);
}

// ---- GGX (directional_distribution_functions.cpp:247-315) ----
__device__ __forceinline__ float ggxD(float ax, float ay, V3 m) {
    if (m.z <= 0) return 0.0f;
    float temp = m.x * m.x / (ax * ax) + m.y * m.y / (ay * ay) + m.z * m.z;
    return 1.0f / (kPiF * ax * ay * temp * temp);
}

__device__ __forceinline__ float ggxG1(float ax, float ay, V3 v, V3 m) {
    float chi = (dot(v, m) / v.z) > 0 ? 1.0f : 0.0f;
    float tan2 = (v.x * v.x * ax * ax + v.y * v.y * ay * ay) / (v.z * v.z);
    return chi * 2 / (1 + sqrtf(1 + tan2));
}

__device__ __forceinline__ float ggxPdf(float ax, float ay, V3 v, V3 m) {
    return ggxG1(ax, ay, v, m) * absDot(v, m) * ggxD(ax, ay, m) / fabsf(v.z);
}

// The Fresnel spectra of a BSDF of kind KIND: once per index pair for the
// kinds that look for pairs, else per wavelength (no pair code compiled in).
template <uint32_t KIND>
__device__ __forceinline__ void fresnelConductorFor(const Bsdf &B, const Spec &eta, const Spec &k, float cosEnter,
                                                    Spec &F) {
    if constexpr (kIorPairsFor<KIND>) fresnelConductorPairs(B, eta, k, cosEnter, F);
    else fresnelConductor(eta, k, cosEnter, F);
}

template <uint32_t KIND>
__device__ __forceinline__ void fresnelDielectricFor(const Bsdf &B, const Spec &etaExt, const Spec &etaInt,
                                                     float cosEnter, Spec &F) {
    if constexpr (kIorPairsFor<KIND>) fresnelDielectricPairs(B, etaExt, etaInt, cosEnter, F);
    else fresnelDielectric(etaExt, etaInt, cosEnter, F);
}

// Transmission term of the rough dielectric B between v and l at every
// wavelength, with each wavelength's own half vector
// (microfacet_bsdfs.cpp:187-199, :239-250); r = 1 / |v.z l.z|; an adjoint
// query scales by the exit index squared instead of the entry index's.
// Rolled when evaluated per wavelength: 16 copies of the half-vector math
// overflow the instruction cache of the shading kernel.
__device__ __forceinline__ void ggxTransmitPairs(const Bsdf &B, bool entering, V3 v, V3 l, float r, Spec &fs,
                                                 bool adjoint = false) {
    const float ax = B.ax, ay = B.ay;
    evalIorPairs<false>(B, B.a, B.b, [=](float eExt, float eInt) {
        float eEnter = entering ? eExt : eInt;
        float eExit = entering ? eInt : eExt;
        V3 mw = normalize(-(eEnter * v + eExit * l));
        float dHV = dot(v, mw), dHL = dot(l, mw);
        float Fw = fresnelDielectric1(eExt, eInt, dHV);
        float Gw = ggxG1(ax, ay, v, mw) * ggxG1(ax, ay, l, mw);
        float Dw = ggxD(ax, ay, mw);
        float dd = eEnter * dHV + eExit * dHL;
        float val = fabsf(dHV * dHL) * (1 - Fw) * Gw * Dw / (dd * dd);
        return (val * r) * (adjoint ? eExit * eExit : eEnter * eEnter);
    }, fs);
}

// Visible-normal sampling (Heitz 2017, "A Simpler and Exact Sampling Routine
// for the GGX Distribution of Visible Normals").
__device__ __forceinline__ float ggxSample(float ax, float ay, V3 v, float u0, float u1, V3* m, float* pdf) {
    V3 sv = normalize(V3{ax * v.x, ay * v.y, v.z});
    float dist2D = sqrtf(sv.x * sv.x + sv.y * sv.y);
    float rec = 1.0f / dist2D;
    V3 T1 = (sv.z < 0.9999f) ? V3{sv.y * rec, -sv.x * rec, 0} : V3{1, 0, 0};
    V3 T2 = V3{T1.y * sv.z, -T1.x * sv.z, dist2D};
    float a = 1.0f / (1.0f + sv.z);
    float r = sqrtf(u0);
    float phi = kPiF * ((u1 < a) ? u1 / a : 1 + (u1 - a) / (1.0f - a));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float P1 = r * cp;
    float P2 = r * sp * ((u1 < a) ? 1.0f : sv.z);
    V3 mm = P1 * T1 + P2 * T2 + sqrtf(1.0f - P1 * P1 - P2 * P2) * sv;
    mm = normalize(V3{ax * mm.x, ay * mm.y, mm.z});
    *m = mm;
    float D = ggxD(ax, ay, mm);
    *pdf = ggxG1(ax, ay, v, mm) * absDot(v, mm) * D / fabsf(v.z);
    return D;
}

// ---- per-BSDF internals ----
__device__ __forceinline__ void specScale(const Spec &a, float s, Spec &out) {
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) out.v[i] = a.v[i] * s;
}

// The BSDF bodies are templates over the material kind: K >= 0 fixes the
// kind at compile time (the switch folds to one case inside a kernel that
// shades a single material), K < 0 dispatches on B.kind at run time.

// Returns fs (without the shading-normal correction); res->pdf == 0 on failure.
template <int K>
__device__ __forceinline__ void bsdfSampleBody(const Bsdf &B, const BsdfQuery &q, float uc, float u0, float u1,
                                               BsdfSample* res, Spec &fs) {
    res->pdf = 0.0f;
    res->type = 0;
    res->dir = V3{0, 0, 1};
    fs = specConst(0.0f);
    const uint32_t kind = K < 0 ? B.kind : (uint32_t)K;
    switch (kind) {
    case kMatMatte: {  // basic_bsdfs.cpp:13-27
        V3 d = cosineSampleHemisphere(u0, u1);
        res->pdf = d.z * kInvPiF;
        res->type = kDirReflection | kDirLowFreq;
        d.z *= q.dir.z > 0 ? 1.0f : -1.0f;
        res->dir = d;
        specScale(B.a, 1.0f / kPiF, fs);
        return;
    }
    case kMatSpecularReflection: {  // basic_bsdfs.cpp:62-72
        res->dir = V3{-q.dir.x, -q.dir.y, q.dir.z};
        res->pdf = 1.0f;
        res->type = kDirReflection | kDirDelta0D;
        Spec F;
        fresnelConductorFor<kMatSpecularReflection>(B, B.b, B.c, q.dir.z, F);
        float r = 1.0f / fabsf(q.dir.z);
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) fs.v[i] = (B.a.v[i] * F.v[i]) * r;
        return;
    }
    case kMatSpecularScattering: {  // basic_bsdfs.cpp:99-150
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
            return;
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
        val *= (eEnter * eEnter) / (eExit * eExit);
        float r = 1.0f / fabsf(cosExit);
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) fs.v[i] = (i == q.wl) ? val * r : 0.0f;
        return;
    }
    case kMatGGXReflection: {  // microfacet_bsdfs.cpp:11-40
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
        return;
    }
    case kMatGGXScattering: {  // microfacet_bsdfs.cpp:116-215
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
            return;
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
        ggxTransmitPairs(B, entering, q.dir, d, r, fs);
        return;
    }
    default:
        return;
    }
}

template <int K>
__device__ __forceinline__ void bsdfEvalBody(const Bsdf &B, const BsdfQuery &q, V3 dir, Spec &fs) {
    fs = specConst(0.0f);
    const uint32_t kind = K < 0 ? B.kind : (uint32_t)K;
    switch (kind) {
    case kMatMatte:
        if (q.dir.z * dir.z <= 0.0f) return;
        specScale(B.a, 1.0f / kPiF, fs);
        return;
    case kMatGGXReflection: {
        if (dir.z * q.dir.z <= 0) return;
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
        return;
    }
    case kMatGGXScattering: {  // microfacet_bsdfs.cpp:217-263
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
            ggxTransmitPairs(B, entering, q.dir, dir, r, fs);
        }
        return;
    }
    default:  // delta BSDFs evaluate to zero
        return;
    }
}

template <int K>
__device__ __forceinline__ float bsdfPdfBody(const Bsdf &B, const BsdfQuery &q, V3 dir) {
    const uint32_t kind = K < 0 ? B.kind : (uint32_t)K;
    switch (kind) {
    case kMatMatte:
        if (q.dir.z * dir.z <= 0.0f) return 0.0f;
        return fabsf(dir.z) * kInvPiF;
    case kMatGGXReflection: {
        if (dir.z * q.dir.z <= 0) return 0.0f;
        float sign = q.dir.z >= 0.0f ? 1.0f : -1.0f;
        V3 m = sign * normalize(q.dir + dir);
        float dotHV = dot(q.dir, m);
        if (dotHV * sign <= 0) return 0.0f;
        float mPdf = ggxPdf(B.ax, B.ay, sign * q.dir, m);
        float common = 1.0f / (4 * dotHV * sign);
        return common * mPdf;
    }
    case kMatGGXScattering: {  // microfacet_bsdfs.cpp:265-318
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
            return common * mPdf;
        }
        float dotHL = dot(dir, m);
        float den = eEnterW * dotHV + eExitW * dotHL;
        float common = (1 - reflectProb) / (den * den);
        return common * mPdf * eExitW * eExitW * fabsf(dotHL);
    }
    default:
        return 0.0f;
    }
}

// Run-time dispatch, kept out of line so that kernels shading any material
// carry one copy of every BSDF.
static __device__ __noinline__ void bsdfSampleInternal(const Bsdf &B, const BsdfQuery &q, float uc, float u0, float u1,
                                                BsdfSample* res, Spec &fs) {
    bsdfSampleBody<-1>(B, q, uc, u0, u1, res, fs);
}
static __device__ __noinline__ void bsdfEvalInternal(const Bsdf &B, const BsdfQuery &q, V3 dir, Spec &fs) {
    bsdfEvalBody<-1>(B, q, dir, fs);
}
static __device__ __noinline__ float bsdfPdfInternal(const Bsdf &B, const BsdfQuery &q, V3 dir) {
    return bsdfPdfBody<-1>(B, q, dir);
}

// ---- the BSDF wrapper: shading-normal correction |d.z / dot(d, n_g)| ----
// K < 0: any material (run-time dispatch); K >= 0: that material kind only.
template <int K = -1>
__device__ __forceinline__ void bsdfSample(const Bsdf &B, const BsdfQuery &q, float uc, float u0, float u1,
                                           BsdfSample* res, Spec &fs) {
    if (K < 0) bsdfSampleInternal(B, q, uc, u0, u1, res, fs);
    else bsdfSampleBody<K>(B, q, uc, u0, u1, res, fs);
    if (res->pdf == 0.0f) return;
    float sn = fabsf(res->dir.z / dot(res->dir, q.gn));
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) fs.v[i] *= sn;
}

template <int K = -1>
__device__ __forceinline__ void bsdfEval(const Bsdf &B, const BsdfQuery &q, V3 dir, Spec &fs) {
    if (K < 0) bsdfEvalInternal(B, q, dir, fs);
    else bsdfEvalBody<K>(B, q, dir, fs);
    float sn = fabsf(dir.z / dot(dir, q.gn));
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) fs.v[i] *= sn;
}

template <int K = -1>
__device__ __forceinline__ float bsdfPdf(const Bsdf &B, const BsdfQuery &q, V3 dir) {
    if (K < 0) return bsdfPdfInternal(B, q, dir);
    return bsdfPdfBody<K>(B, q, dir);
}

}  // namespace slrgpu
