// Device helpers: vector math, counter-based RNG, spectral evaluation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "slrgpu_types.h"

namespace slrgpu {

constexpr float kPiF = 3.14159265358979323846f;
constexpr float kInvPiF = 0.318309886183790671538f;

struct V3 { float x, y, z; };

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float absDot(V3 a, V3 b) { return fabsf(dot(a, b)); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float sqLength(V3 a) { return dot(a, a); }
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
// v / |v| as v * (1 / |v|) (Vector3D.h:115-118, :31).
__device__ __forceinline__ V3 normalize(V3 a) { float r = 1.0f / length(a); return a * r; }

// Exactly rounded forms (no contraction) for the parity-critical ray tests.
__device__ __forceinline__ float rn_dot(V3 a, V3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 rn_cross(V3 a, V3 b) {
    return V3{__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
              __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ V3 rn_sub(V3 a, V3 b) { return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
// org + dir * t, each product and sum rounded on its own.  Points on a light
// (hit points, sampled light positions) must round as the reference does:
// whether a point on an emitter lands exactly in the emitter's plane decides
// whether next-event estimation from it divides zero by zero, and a fused
// multiply-add lands there more often.
__device__ __forceinline__ V3 rn_ray_point(V3 org, V3 dir, float t) {
    return V3{__fadd_rn(org.x, __fmul_rn(dir.x, t)), __fadd_rn(org.y, __fmul_rn(dir.y, t)),
              __fadd_rn(org.z, __fmul_rn(dir.z, t))};
}
// b0 * p0 + b1 * p1 + b2 * p2, left to right, without contraction.
__device__ __forceinline__ V3 rn_bary(float b0, V3 p0, float b1, V3 p1, float b2, V3 p2) {
    return V3{__fadd_rn(__fadd_rn(__fmul_rn(b0, p0.x), __fmul_rn(b1, p1.x)), __fmul_rn(b2, p2.x)),
              __fadd_rn(__fadd_rn(__fmul_rn(b0, p0.y), __fmul_rn(b1, p1.y)), __fmul_rn(b2, p2.y)),
              __fadd_rn(__fadd_rn(__fmul_rn(b0, p0.z), __fmul_rn(b1, p1.z)), __fmul_rn(b2, p2.z))};
}

struct Frame {
    V3 x, y, z;
    __device__ V3 toLocal(V3 v) const { return V3{dot(x, v), dot(y, v), dot(z, v)}; }
    __device__ V3 fromLocal(V3 v) const {
        return V3{dot(V3{x.x, y.x, z.x}, v), dot(V3{x.y, y.y, z.y}, v), dot(V3{x.z, y.z, z.z}, v)};
    }
};

// ---------------------------------------------------------------------------
// RNG: counter-based.  Each path owns a 64-bit key derived from (seed, global
// sample index); draw i is the SplitMix64 finaliser of key + i * golden
// gamma.  Floats use the reference's construction: the top 23 bits as the
// mantissa of [1, 2), minus 1 (random_number_generator.cpp:12-15).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t pathKey(uint32_t seed, uint64_t sampleIndex) {
    return mix64(((uint64_t)seed << 32) ^ mix64(sampleIndex + 0x632be59bd9b4e019ull));
}
__device__ __forceinline__ float uniformFloat(uint64_t key, uint32_t counter) {
    uint32_t u = (uint32_t)(mix64(key + (uint64_t)(counter + 1) * 0x9e3779b97f4a7c15ull) >> 32);
    return __uint_as_float((u >> 9) | 0x3f800000u) - 1.0f;
}

// Path-level replay: a path draws its uniforms from tape[key .. key +
// kRngTapeStride) (a recorded reference path) instead of the counter-based
// generator; draws past the stride return 0.5.
constexpr uint32_t kRngTapeStride = 256;   // kRngTapeFloats of render_api.h
struct Rng {
    uint64_t key;
    uint32_t counter;
    const float* tape = nullptr;
    __device__ float next() {
        if (tape) {
            const uint32_t c = counter++;
            return c < kRngTapeStride ? tape[key + c] : 0.5f;
        }
        return uniformFloat(key, counter++);
    }
};

// ---------------------------------------------------------------------------
// Spectra: 16 sampled values.
// ---------------------------------------------------------------------------
struct Spec {
    float v[kNumLambda];
};

__device__ __forceinline__ Spec specConst(float c) {
    Spec s;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) s.v[i] = c;
    return s;
}

// lambda_i = 360 + 470 (i + offset) / 16 (spectrum_types.h:59-68).  The
// division by 16 is a multiplication by 2^-4, exact for the (non-negative,
// normal or zero) dividends that occur, so the IEEE quotient is kept.
static_assert(kNumLambda == 16, "the scale 2^-4 below is 1 / kNumLambda");
__device__ __forceinline__ float lambdaAt(int i, float offset) {
    return __fadd_rn(kWavelengthLow, __fmul_rn(__fmul_rn(kWavelengthHigh - kWavelengthLow, __fadd_rn((float)i, offset)),
                                               0.0625f));
}

// SampledSpectrum::importance (spectrum_types.h:473-486).
__device__ __forceinline__ float importance(const Spec &s, int sel) {
    float sum = 0;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) sum += s.v[i];
    const float primary = 0.9f;
    const float marginal = (1 - primary) / (kNumLambda - 1);
    float vs = 0;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) vs = (i == sel) ? s.v[i] : vs;
    return sum * marginal + vs * (primary - marginal);
}

__device__ __forceinline__ float specAt(const Spec &s, int idx) {
    float r = 0;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) r = (i == idx) ? s.v[i] : r;
    return r;
}

__device__ __forceinline__ bool specIsZero(const Spec &s) {
    bool z = true;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) z &= (s.v[i] == 0.0f);
    return z;
}

__device__ __forceinline__ bool specAllFinite(const Spec &s) {
    bool f = true;
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) f &= isfinite(s.v[i]);
    return f;
}

// Upsampled spectrum value at one wavelength: sum_j w_j lerp(basis_j, lambda),
// in the reference's operation order (spectrum_types.cpp:610-650).
__device__ __forceinline__ void upsWeights(uint32_t adj, float s, float t, int idx[4], float w[4], int* n) {
    idx[0] = adj & 0xff; idx[1] = (adj >> 8) & 0xff; idx[2] = (adj >> 16) & 0xff; idx[3] = adj >> 24;
    if (idx[3] != 0xff) {
        w[0] = __fmul_rn(__fsub_rn(1.0f, s), __fsub_rn(1.0f, t));
        w[1] = __fmul_rn(s, __fsub_rn(1.0f, t));
        w[2] = __fmul_rn(__fsub_rn(1.0f, s), t);
        w[3] = __fmul_rn(s, t);
        *n = 4;
    } else {
        w[0] = s; w[1] = t; w[2] = __fsub_rn(__fsub_rn(1.0f, s), t); w[3] = 0.0f;
        idx[3] = idx[0];
        *n = 3;
    }
}

// x / 470 (the width of the wavelength range) correctly rounded, by the FMA
// method of Brisebarre, Muller and Raina ("Accelerating correctly rounded
// floating-point division when the divisor is known in advance", IEEE Trans.
// Computers 53(8), 2004): with z = RN(1/470), q = RN(x z) and the exact
// remainder r = x - q 470 (one FMA), RN(q + r z) is the correctly rounded
// quotient.  Checked against IEEE division for every float of [2^-20, 2048]
// (tests/test_division_by_range.py); the inputs here are wavelength offsets,
// 0 or at least 2^-15.
__device__ __forceinline__ float divRange(float x) {
    constexpr float z = 1.0f / 470.0f;
    const float q = __fmul_rn(x, z);
    const float r = __fmaf_rn(-q, 470.0f, x);
    return __fmaf_rn(r, z, q);
}
static_assert(kWavelengthHigh - kWavelengthLow == 470.0f, "divRange divides by the wavelength range");

// The 16 wavelengths of a path computed from its offset where they are
// used (lambdaAt, the same numbers as a stored array), so that no array of
// them needs registers or local memory; spectrum functions take either this
// or a plain array (const float*).
struct OffsetLambdas {
    float off;
    __device__ __forceinline__ float operator[](int i) const { return lambdaAt(i, off); }
};

template <class LAM>
__device__ __forceinline__ void evalUpsampled(const float* __restrict__ basis, uint32_t adj, float s, float t, float scale,
                                              LAM lambdas, Spec &out) {
    int idx[4]; float w[4]; int n;
    upsWeights(adj, s, t, idx, w, &n);
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) {
        float p = divRange(__fsub_rn(lambdas[i], 360.0f));
        p = fminf(fmaxf(p, 0.0f), 1.0f);
        float sBinF = __fmul_rn(p, (float)(kUpsNumSamples - 1));
        uint32_t sBin = min((uint32_t)sBinF, (uint32_t)(kUpsNumSamples - 1));
        uint32_t sBinNext = min(sBin + 1, (uint32_t)(kUpsNumSamples - 1));
        float tt = __fsub_rn(sBinF, (float)sBin);
        float omt = __fsub_rn(1.0f, tt);
        float acc = 0.0f;
        for (int j = 0; j < n; ++j) {
            const float* sp = basis + idx[j] * kUpsNumSamples;
            float lerp = __fadd_rn(__fmul_rn(__ldg(sp + sBin), omt), __fmul_rn(__ldg(sp + sBinNext), tt));
            acc = __fadd_rn(acc, __fmul_rn(w[j], lerp));
        }
        out.v[i] = __fmul_rn(acc, scale);
    }
}

template <class LAM>
static __device__ __noinline__ void evalSpectrum(const DevScene &sc, int id, LAM lambdas, Spec &out) {
    const DevSpectrum sp = sc.spectra[id];
    if (sp.kind == kSpecUpsampled) {
        evalUpsampled(sc.upsSpectra, sp.adj, sp.p0, sp.p1, sp.scale, lambdas, out);
    } else if (sp.kind == kSpecRegular) {
        const float* v = sc.specValues + sp.offset;
        const float nm1 = (float)(sp.count - 1);
        // over the wavelength range itself the quotient is divRange's, the
        // correctly rounded one, in three operations instead of a division
        const bool fullRange = sp.p0 == kWavelengthLow && sp.p1 == kWavelengthHigh;
#pragma unroll
        for (int i = 0; i < kNumLambda; ++i) {
            const float x = __fsub_rn(lambdas[i], sp.p0);
            float binF = __fmul_rn(fullRange ? divRange(x) : __fdiv_rn(x, __fsub_rn(sp.p1, sp.p0)), nm1);
            float r;
            if (binF <= 0.0f) r = v[0];
            else if (binF >= nm1) r = v[sp.count - 1];
            else {
                int bin = (int)binF;
                float t = __fsub_rn(binF, (float)bin);
                r = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, t), v[bin]), __fmul_rn(t, v[bin + 1]));
            }
            out.v[i] = r;
        }
    } else {
        const float* wl = sc.specValues + sp.offset;
        const float* v = wl + sp.count;
        uint32_t base = 0;
        for (int i = 0; i < kNumLambda; ++i) {
            // lower_bound over [base, count)
            uint32_t lo = base, hi = sp.count;
            while (lo < hi) {
                uint32_t mid = (lo + hi) >> 1;
                if (wl[mid] < lambdas[i]) lo = mid + 1; else hi = mid;
            }
            int low = max((int)lo - 1, 0);
            base = (uint32_t)low;
            float r;
            if (low >= (int)sp.count - 1) r = v[sp.count - 1];
            else {
                float t = __fdiv_rn(__fsub_rn(lambdas[i], wl[low]), __fsub_rn(wl[low + 1], wl[low]));
                if (t <= 0.0f) r = v[0];
                else r = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, t), v[low]), __fmul_rn(t, v[low + 1]));
            }
            out.v[i] = r;
        }
    }
}

// One wavelength of evalSpectrum: the same arithmetic for that wavelength
// (every wavelength of evalSpectrum is computed on its own; the irregular
// search from the previous wavelength's bracket finds the same bracket as a
// search from the start), for threads that need a single wavelength.
static __device__ __noinline__ float evalSpectrumAt(const DevScene &sc, int id, float lambda) {
    const DevSpectrum sp = sc.spectra[id];
    if (sp.kind == kSpecUpsampled) {
        int idx[4]; float w[4]; int n;
        upsWeights(sp.adj, sp.p0, sp.p1, idx, w, &n);
        float p = divRange(__fsub_rn(lambda, 360.0f));
        p = fminf(fmaxf(p, 0.0f), 1.0f);
        const float sBinF = __fmul_rn(p, (float)(kUpsNumSamples - 1));
        const uint32_t sBin = min((uint32_t)sBinF, (uint32_t)(kUpsNumSamples - 1));
        const uint32_t sBinNext = min(sBin + 1, (uint32_t)(kUpsNumSamples - 1));
        const float tt = __fsub_rn(sBinF, (float)sBin);
        const float omt = __fsub_rn(1.0f, tt);
        float acc = 0.0f;
        for (int j = 0; j < n; ++j) {
            const float* b = sc.upsSpectra + idx[j] * kUpsNumSamples;
            const float lerp = __fadd_rn(__fmul_rn(__ldg(b + sBin), omt), __fmul_rn(__ldg(b + sBinNext), tt));
            acc = __fadd_rn(acc, __fmul_rn(w[j], lerp));
        }
        return __fmul_rn(acc, sp.scale);
    }
    if (sp.kind == kSpecRegular) {
        const float* v = sc.specValues + sp.offset;
        const float nm1 = (float)(sp.count - 1);
        const float binF = __fmul_rn(__fdiv_rn(__fsub_rn(lambda, sp.p0), __fsub_rn(sp.p1, sp.p0)), nm1);
        if (binF <= 0.0f) return v[0];
        if (binF >= nm1) return v[sp.count - 1];
        const int bin = (int)binF;
        const float t = __fsub_rn(binF, (float)bin);
        return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, t), v[bin]), __fmul_rn(t, v[bin + 1]));
    }
    const float* wl = sc.specValues + sp.offset;
    const float* v = wl + sp.count;
    uint32_t lo = 0, hi = sp.count;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (wl[mid] < lambda) lo = mid + 1; else hi = mid;
    }
    const int low = max((int)lo - 1, 0);
    if (low >= (int)sp.count - 1) return v[sp.count - 1];
    const float t = __fdiv_rn(__fsub_rn(lambda, wl[low]), __fsub_rn(wl[low + 1], wl[low]));
    if (t <= 0.0f) return v[0];
    return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, t), v[low]), __fmul_rn(t, v[low + 1]));
}

}  // namespace slrgpu
