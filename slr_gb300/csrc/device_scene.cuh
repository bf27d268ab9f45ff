// Scene-level device helpers shared by the path tracers (render.cu) and the
// bidirectional path tracer (bpt.cu): spectral SoA access, queue pushes,
// cameras, the environment light, alias-table sampling, material -> BSDF,
// triangle surface points and light selection.
#pragma once
#include "device_bsdf.cuh"
#include "device_trace.cuh"

namespace slrgpu {

// Spectra in the path state (throughput, radiance, shadow contribution):
// the 16 values of a path are contiguous, 64 bytes or two whole 32-byte
// sectors, so a thread's access costs two sectors wherever the compacted
// queues have scattered its path (16 planes of [16][N] would cost 16).
__device__ __forceinline__ void loadSpec(const float* base, uint32_t p, Spec &s) {
    const float4* b = reinterpret_cast<const float4*>(base) + (size_t)p * (kNumLambda / 4);
#pragma unroll
    for (int k = 0; k < kNumLambda / 4; ++k) {
        const float4 v = b[k];
        s.v[4 * k] = v.x; s.v[4 * k + 1] = v.y; s.v[4 * k + 2] = v.z; s.v[4 * k + 3] = v.w;
    }
}
__device__ __forceinline__ void storeSpec(float* base, uint32_t p, const Spec &s) {
    float4* b = reinterpret_cast<float4*>(base) + (size_t)p * (kNumLambda / 4);
#pragma unroll
    for (int k = 0; k < kNumLambda / 4; ++k)
        b[k] = make_float4(s.v[4 * k], s.v[4 * k + 1], s.v[4 * k + 2], s.v[4 * k + 3]);
}
__device__ __forceinline__ void addSpec(float* base, uint32_t p, const Spec &s) {
    float4* b = reinterpret_cast<float4*>(base) + (size_t)p * (kNumLambda / 4);
#pragma unroll
    for (int k = 0; k < kNumLambda / 4; ++k) {
        float4 v = b[k];
        v.x += s.v[4 * k]; v.y += s.v[4 * k + 1]; v.z += s.v[4 * k + 2]; v.w += s.v[4 * k + 3];
        b[k] = v;
    }
}

// Warp-aggregated queue push.
__device__ __forceinline__ void queuePush(uint32_t* queue, uint32_t* count, uint32_t value, bool pred) {
    unsigned mask = __ballot_sync(__activemask(), pred);
    if (!pred) return;
    int leader = __ffs(mask) - 1;
    int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    queue[base + __popc(mask & ((1u << lane) - 1))] = value;
}

// ---------------------------------------------------------------------------
// Camera
// ---------------------------------------------------------------------------
// Thin-lens perspective camera (PerspectiveCamera.cpp:31-83) and
// equirectangular camera (EquirectangularCamera.cpp:25-69): ray and the
// sample weight We0 We1 cos / (areaPDF dirPDF).
__device__ __forceinline__ void cameraRay(const DevCamera &c, float lu0, float lu1, float px, float py,
                                          V3* org, V3* dir, float* weight) {
    V3 ex = V3{c.ex[0], c.ex[1], c.ex[2]}, ey = V3{c.ey[0], c.ey[1], c.ey[2]}, ez = V3{c.ez[0], c.ez[1], c.ez[2]};
    Frame fr{ex, ey, ez};
    if (c.kind == 0) {
        float lx, ly;
        concentricSampleDisk(lu0, lu1, &lx, &ly);
        V3 orgLocal = V3{c.lensRadius * lx, c.lensRadius * ly, 0.0f};
        *org = V3{c.org[0], c.org[1], c.org[2]} + orgLocal.x * ex + orgLocal.y * ey;
        V3 pFocus = V3{c.opWidth * (0.5f - px), c.opHeight * (0.5f - py), c.objPlaneDist};
        V3 dl = normalize(pFocus - orgLocal);
        float dirPDF = c.imgPlaneDist * c.imgPlaneDist / ((dl.z * dl.z * dl.z) * c.imgPlaneArea);
        float areaPDF = c.lensRadius > 0.0f ? 1.0f / (kPiF * c.lensRadius * c.lensRadius) : 1.0f;
        *dir = fr.fromLocal(dl);
        float cosT = absDot(*dir, ez);
        *weight = cosT / (areaPDF * dirPDF);
    } else {
        *org = V3{c.org[0], c.org[1], c.org[2]};
        float phi = c.phiAngle * (px - 0.5f);
        float theta = 0.5f * kPiF + c.thetaAngle * (py - 0.5f);
        float sp, cp, st, ct;
        sincosf(phi, &sp, &cp);
        sincosf(theta, &st, &ct);
        V3 dl = V3{-sp * st, ct, cp * st};
        float sinTheta = sqrtf(1.0f - dl.y * dl.y);
        float dirPDF = 1.0f / (c.phiAngle * c.thetaAngle * sinTheta);
        *dir = fr.fromLocal(dl);
        // We0 We1 |cos| / (areaPDF dirPDF) with areaPDF = 1 (EquirectangularCamera.cpp:25-69).
        *weight = absDot(*dir, ez) / dirPDF;
    }
}

// ---------------------------------------------------------------------------
// Environment
// ---------------------------------------------------------------------------
__device__ __forceinline__ void toPolarYUp(V3 d, float* theta, float* phi) {
    *theta = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f));
    const float twoPi = 6.28318530717958647692f;
    *phi = fmodf(atan2f(-d.x, d.z) + twoPi, twoPi);
}

// Emitted radiance of the environment at texture coordinate (tu, tv):
// (pi * texel * scale) * (1 / pi) (IBLEmitterSurfaceProperty.cpp:16-18, IBLEDF.cpp:18-21).
template <class LAM>
__device__ __forceinline__ void envRadiance(const DevScene &sc, float tu, float tv, LAM lambdas, Spec &Le) {
    float u = fmodf(tu, 1.0f), v = fmodf(tv, 1.0f);
    u += u < 0 ? 1.0f : 0.0f;
    v += v < 0 ? 1.0f : 0.0f;
    uint32_t px = min((uint32_t)(sc.envWidth * u), sc.envWidth - 1);
    uint32_t py = min((uint32_t)(sc.envHeight * v), sc.envHeight - 1);
    EnvTexel tx = sc.envTexels[(size_t)py * sc.envWidth + px];
    evalUpsampled(sc.upsSpectra, tx.adj, tx.s, tx.t, tx.scale, lambdas, Le);
#pragma unroll
    for (int i = 0; i < kNumLambda; ++i) Le.v[i] = ((Le.v[i] * kPiF) * sc.envScale) * kInvPiF;
}

// RegularConstantContinuousDistribution1D::sample (distributions.cpp:205-214).
__device__ __forceinline__ uint32_t prevPow2(uint32_t x) {
    x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
    return x - (x >> 1);
}
// Alias-table sampling (Vose; O(1) instead of the CDF's binary search) of a
// piecewise-constant distribution over [0, 1) with n bins: the bin is the
// alias pick of u, the position inside it the leftover fraction of u
// rescaled to [0, 1), the density that of the bin.  The tables hold the
// PMF of the reference's CDFs, so the sampled distribution is the same.
__device__ __forceinline__ uint32_t aliasPick(const AliasEntry* __restrict__ t, uint32_t n, float u, float* frac) {
    const float x = u * (float)n;
    const uint32_t i = min((uint32_t)x, n - 1);
    const float f = fminf(x - (float)i, 0x1.fffffep-1f);
    const AliasEntry e = t[i];
    if (f < e.prob) {
        *frac = f / e.prob;
        return i;
    }
    *frac = (f - e.prob) / (1.0f - e.prob);
    return e.alias;
}

__device__ __forceinline__ float sampleAlias(const AliasEntry* __restrict__ t, const float* __restrict__ pdf, uint32_t n,
                                             float u, float* outPdf, uint32_t* bin) {
    float frac;
    const uint32_t k = aliasPick(t, n, u, &frac);
    *outPdf = pdf[k];
    *bin = k;
    return fminf(((float)k + fminf(frac, 0x1.fffffep-1f)) / (float)n, 0x1.fffffep-1f);
}


__device__ __forceinline__ float envUVPdf(const DevScene &sc, float d0, float d1) {
    uint32_t row = min((uint32_t)(sc.envMapH * d1), sc.envMapH - 1);
    float top = sc.envTopPDF[min((int)(d1 * sc.envMapH), (int)sc.envMapH - 1)];
    return top * sc.envRowPDF[(size_t)row * sc.envMapW + min((int)(d0 * sc.envMapW), (int)sc.envMapW - 1)];
}

// Area pdf of the environment at (phi, theta) (surface_object.cpp:281-286).
__device__ __forceinline__ float envAreaPdf(const DevScene &sc, float phi, float theta) {
    const float twoPi = 6.28318530717958647692f;
    float uvPdf = envUVPdf(sc, phi / twoPi, theta / kPiF);
    return uvPdf / (2.0f * kPiF * kPiF * sinf(theta));
}

// ---------------------------------------------------------------------------
// Material -> BSDF (SurfaceMaterial::getBSDF)
// ---------------------------------------------------------------------------
template <class LAM>
static __device__ __noinline__ void makeBsdf(const DevScene &sc, const DevMaterial &m, LAM lambdas,
                                      bool wlSelected, Bsdf &B) {
    B.kind = m.kind;
    B.ax = m.alphaX;
    B.ay = m.alphaY;
    B.dispersive = !wlSelected;
    switch (m.kind) {
    case kMatMatte:
        evalSpectrum(sc, m.spec[0], lambdas, B.a);
        break;
    case kMatSpecularReflection:
    case kMatSpecularScattering:
        evalSpectrum(sc, m.spec[0], lambdas, B.a);
        evalSpectrum(sc, m.spec[1], lambdas, B.b);
        evalSpectrum(sc, m.spec[2], lambdas, B.c);
        break;
    case kMatGGXReflection:
    case kMatGGXScattering:
        evalSpectrum(sc, m.spec[0], lambdas, B.a);
        evalSpectrum(sc, m.spec[1], lambdas, B.b);
        break;
    default:
        break;
    }
    prepareIorPairs(B);
}

struct SurfPoint {
    V3 p;
    Frame frame;
    V3 gn;
};

// Surface point of a hit (TriangleSurfaceShape.cpp:301-346): interpolated
// shading normal, tangent made orthogonal to it, geometric normal.
__device__ __forceinline__ void surfacePoint(const DevScene &sc, const DevPrim &pr, V3 org, V3 dir, float t, float mb1,
                                             float mb2, SurfPoint &sp) {
    sp.p = rn_ray_point(org, dir, t);   // TriangleSurfaceShape.cpp:250
    float b0 = 1.0f - mb1 - mb2;
    float b1 = mb1;
    float b2 = 1.0f - b0 - b1;
    float4 n0 = sc.vnrm[pr.v0], n1 = sc.vnrm[pr.v1], n2 = sc.vnrm[pr.v2];
    float4 t0 = sc.vtan[pr.v0], t1 = sc.vtan[pr.v1], t2 = sc.vtan[pr.v2];
    V3 z = normalize(b0 * V3{n0.x, n0.y, n0.z} + b1 * V3{n1.x, n1.y, n1.z} + b2 * V3{n2.x, n2.y, n2.z});
    V3 x = b0 * V3{t0.x, t0.y, t0.z} + b1 * V3{t1.x, t1.y, t1.z} + b2 * V3{t2.x, t2.y, t2.z};
    float dnt = dot(z, x);
    x = normalize(x - dnt * z);
    sp.frame = Frame{x, cross(z, x), z};
    sp.gn = V3{pr.ngx, pr.ngy, pr.ngz};
}

// Light selection (Scene::selectSurfaceLight, Scene.cpp:137-155).  Returns
// -1 for the environment, else the light index; *prob = selection probability.
__device__ __forceinline__ int selectLight(const DevScene &sc, float u, float* prob) {
    auto surf = [&](float uu, float* pr) -> int {
        float frac;
        const int idx = (int)aliasPick(sc.lightAlias, sc.numLights, uu, &frac);
        *pr = sc.lightPMF[idx];
        return idx;
    };
    if (sc.envPresent) {
        float sumImps = sc.surfImportance + sc.envImportance;
        float su = sumImps * u;
        if (su < sc.surfImportance) {
            float uu = u / (sc.surfImportance / sumImps);
            int idx = surf(uu, prob);
            *prob *= sc.surfImportance / sumImps;
            return idx;
        }
        *prob = 1.0f * (sc.envImportance / sumImps);
        return -1;
    }
    return surf(u, prob);
}


// Scene::selectLight (Scene.cpp:157-188) with sampleDiscrete
// (distributions.cpp:16-36) over {surfaces, media, environment}.  Returns 0
// surface (light index in *li), 2 environment; *prob = selection probability.
__device__ __forceinline__ int selectLight3(const DevScene &sc, float u, int* li, float* prob) {
    float imps[3] = {sc.surfImportance, sc.medium.importance, sc.envImportance};
    // compensated sums as in the reference
    float sum = 0.0f, c = 0.0f;
    for (int i = 0; i < 3; ++i) {
        float y = imps[i] - c, t = sum + y;
        c = (t - sum) - y;
        sum = t;
    }
    float su = u * sum;
    float cum = 0.0f, cc = 0.0f, base = 0.0f;
    int idx = 0;
    float prob1st = imps[0] / sum, remapped = u;
    bool found = false;
    for (int i = 0; i < 3; ++i) {
        base = cum;
        float y = imps[i] - cc, t = cum + y;
        cc = (t - cum) - y;
        cum = t;
        if (!found && su < cum) {
            idx = i;
            prob1st = imps[i] / sum;
            remapped = (su - base) / imps[i];
            found = true;
        }
    }
    if (idx == 0) {
        float frac;
        const int j = (int)aliasPick(sc.lightAlias, sc.numLights, remapped, &frac);
        *li = j;
        *prob = sc.lightPMF[j] * prob1st;
    } else {
        *li = -1;
        *prob = 1.0f * prob1st;
    }
    return idx;
}

template <int K, class LAM>
__device__ __forceinline__ void makeBsdfK(const DevScene &sc, const DevMaterial &m, LAM lambdas,
                                          bool wlSelected, Bsdf &B) {
    B.kind = (uint32_t)K;
    B.ax = m.alphaX;
    B.ay = m.alphaY;
    B.dispersive = !wlSelected;
    evalSpectrum(sc, m.spec[0], lambdas, B.a);
    if (K != kMatMatte) evalSpectrum(sc, m.spec[1], lambdas, B.b);
    if (K == kMatSpecularReflection || K == kMatSpecularScattering) evalSpectrum(sc, m.spec[2], lambdas, B.c);
    if constexpr (((SLRGPU_IOR_PAIR_KINDS >> K) & 1u) != 0) {
        if (K == kMatGGXReflection || K == kMatGGXScattering) prepareIorPairs(B, B.a, B.b);
        else prepareIorPairs(B, B.b, B.c);
    } else {
        B.iorCount = 0u;
    }
}

}  // namespace slrgpu
