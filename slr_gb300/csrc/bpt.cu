// Bidirectional path tracing (BPTRenderer semantics) on the GPU.
//
// The estimator is the reference's BPTRenderer::Job (libSLR/Renderer/
// BPTRenderer.cpp:103-431): per sample a light subpath (light vertex, then
// vertices traced with adjoint BSDFs) and an eye subpath (lens vertex, then
// vertices traced with radiance BSDFs, adding the implicit paths that hit an
// emitter), then every connection of an eye vertex with a light vertex,
// weighted by the power heuristic over all strategies of the same path.
// Connections through the lens vertex (t = 1) land on another pixel and go
// to a splat film, the counterpart of the reference's separated sensor
// buffers (ImageSensor.cpp:132-137).  Only the random numbers differ
// (counter-based, one stream per subpath).
//
// GPU structure, one wave at a time:
//   kBptInit     one thread per path: pixel and wavelengths, the light vertex
//                and the lens vertex, the first ray of each subpath;
//   kBptBounce   per bounce, over the queue of live subpaths (both kinds
//                mixed): closest hit, vertex creation, implicit emission,
//                BSDF sampling with reverse densities, Russian roulette;
//   kBptConnect  one thread per eye vertex: the connections with every light
//                vertex of its path (shadow ray, MIS weight, contribution);
//   kBptAccumulate  per pixel: the wave's per-path sums and the splat film
//                into the compensated 16-bin film.
// Vertices live in HBM as [depth][subpath] arrays of 64-byte geometry,
// 32-byte density and 64-byte throughput records.
#include "render_api.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>

#include "device_bsdf_rev.cuh"
#include "device_medium.cuh"
#include "device_scene.cuh"

namespace slrgpu {

// Resident blocks per SM the traversal kernels are compiled for (the path
// tracer's tuned value).
#ifndef SLRGPU_TRACE_MIN_BLOCKS
#define SLRGPU_TRACE_MIN_BLOCKS 4
#endif
#ifndef SLRGPU_MEDIUM_MIN_BLOCKS
#define SLRGPU_MEDIUM_MIN_BLOCKS 4
#endif

namespace {

// Vertex kinds.
constexpr uint32_t kVtxLens = 0;
constexpr uint32_t kVtxLight = 1;
constexpr uint32_t kVtxSurface = 2;
constexpr uint32_t kVtxMedium = 3;       // a scattering point in the medium (volumetric BPT)
// BptPdf::flags
constexpr uint32_t kVfDelta = 1u;        // reached by a delta distribution (position or direction)
constexpr uint32_t kVfWlSelected = 2u;   // the subpath's wavelength was selected when the vertex was made
constexpr int kVfKindShift = 4;         // vertex kind, 2 bits
constexpr int kVfMatShift = 8;          // material kind of a surface vertex, 4 bits
constexpr uint32_t kVfAtInf = 1u << 12;  // the light vertex on the environment (position = direction)

// Geometry of a vertex (64 B).
//   surface: pg.w = material index bits; ng.w, nz.w, tx.w = query direction
//            (toward the previous vertex) z, x, y in the shading frame
//   lens:    nz.w, tx.w = lens position in the lens frame (x, y)
struct __align__(16) BptGeom {
    float4 pg;   // position
    float4 ng;   // geometric normal
    float4 nz;   // shading normal
    float4 tx;   // shading tangent
};

// Densities of a vertex (32 B), BPTRenderer.h:66-86.
struct __align__(16) BptPdf {
    float cosIn;        // |cos| at this vertex toward the previous one
    float areaPdf;      // area density of this vertex, sampled from the previous one
    float rrProb;       // Russian roulette probability that led here
    float revAreaPdf;   // area density of this vertex, sampled from the next one
    float revRRProb;
    uint32_t flags;
    float pad0, pad1;
};

// Per-subpath state (S = 2N subpaths: light subpaths [0, N), eye [N, 2N)).
struct BptState {
    uint32_t N;           // paths per wave
    uint32_t S;           // 2N
    uint32_t D;           // vertex capacity per subpath - 1
    BptGeom* geom;        // [(D + 1) * S]
    BptPdf* pdf;          // [(D + 1) * S]
    float4* alpha;        // [(D + 1) * S * 4]
    float4* bsdfA;        // [(D + 1) * S * 4] first spectrum of a surface vertex's BSDF
    float4* rayOrg;       // [S] xyz, tmin
    float4* rayDir;       // [S]
    float4* alphaPend;    // [S * 4] throughput arriving at the next vertex
    float4* aux;          // [S] dirPdf, cosLast, rrPend, info bits
    uint32_t* rngCounter; // [S]
    uint32_t* numVerts;   // [S]
    // per path
    uint2* rngKey;        // [N]
    float2* pix;          // [N] film position
    float* wlOffset;      // [N]
    uint32_t* sel;        // [N]
    float* L;             // [N][16] contributions at the path's own pixel
    float* splat;         // [pixels][16] contributions through the lens vertex (film bins)
    uint32_t splatPixels;
    uint32_t* queue[2];   // [S]
    uint32_t* connQueue;  // [N * (D + 1)] eye vertex indices
    // connections that contribute, waiting for their shadow ray
    uint32_t connCap;
    float4* cRay;         // [connCap * 2] origin + tmin, direction + tmax
    float4* cContrib;     // [connCap * 4] contribution (film bins when splatted)
    uint32_t* cTarget;    // [connCap] path index, or pixel | kTargetSplat
    uint32_t* cPath;      // [connCap] path of the connection (volumetric: wavelengths, RNG key)
    uint32_t* cMeta;      // [connCap] eye vertex index << 8 | light vertex number (volumetric RNG stream)
    uint32_t* mQueue;     // [connCap] unoccluded connections whose transmittance is due (volumetric)
    uint32_t* counters;   // [D + 5] queue sizes per bounce, eye vertices to connect, queued
                          // connections, connections waiting for their transmittance, the
                          // transmittance kernel's work counter
    unsigned long long* stats;   // 0 extension rays, 1 shadow rays, 2 dropped contributions
};

// aux.w info bits
constexpr uint32_t kAuxDelta = 1u;        // the pending direction was sampled by a delta distribution
constexpr uint32_t kAuxWlSelected = 2u;
constexpr uint32_t kAuxPrevAtInf = 4u;    // the ray leaves the vertex at infinity (squared distance 1)


struct BptWave {
    uint32_t width, height, gridW, gridH, gridPositions;
    uint32_t sampleBase, samples, seed, numPaths;
};

constexpr uint32_t kLightStream = 1u << 30;   // counter offset of the light subpath's random numbers

__device__ __forceinline__ uint64_t keyOf(const BptState &st, uint32_t p) {
    uint2 k = st.rngKey[p];
    return ((uint64_t)k.y << 32) | k.x;
}
__device__ __forceinline__ V3 xyz(float4 v) { return V3{v.x, v.y, v.z}; }
// std::min(a, b) as the reference evaluates it: b < a ? b : a (a NaN first
// argument stays NaN, unlike fminf).
__device__ __forceinline__ float stdMin(float a, float b) { return (b < a) ? b : a; }

__device__ __forceinline__ void storeAlpha(float4* a, size_t i, const Spec &s) {
#pragma unroll
    for (int k = 0; k < 4; ++k) a[i * 4 + k] = make_float4(s.v[4 * k], s.v[4 * k + 1], s.v[4 * k + 2], s.v[4 * k + 3]);
}
__device__ __forceinline__ void loadAlpha(const float4* a, size_t i, Spec &s) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float4 v = a[i * 4 + k];
        s.v[4 * k] = v.x; s.v[4 * k + 1] = v.y; s.v[4 * k + 2] = v.z; s.v[4 * k + 3] = v.w;
    }
}

__device__ __forceinline__ Frame cameraFrame(const DevCamera &c) {
    return Frame{V3{c.ex[0], c.ex[1], c.ex[2]}, V3{c.ey[0], c.ey[1], c.ey[2]}, V3{c.ez[0], c.ez[1], c.ez[2]}};
}

// ---- the camera as a vertex (PerspectiveCamera.cpp:31-107, EquirectangularCamera.cpp:24-109) ----
// Importance of the lens vertex toward dirIn (lens frame): 1 inside the view, else 0.
__device__ __forceinline__ bool idfInside(const DevCamera &c, V3 d, float lu, float lv) {
    if (c.kind == 0) {
        float s = c.objPlaneDist / d.z;
        float fx = d.x * s + lu, fy = d.y * s + lv;
        return fx >= -c.opWidth * 0.5f && fx <= c.opWidth * 0.5f && fy >= -c.opHeight * 0.5f &&
               fy <= c.opHeight * 0.5f && d.z >= 0;
    }
    float theta, phi;
    toPolarYUp(d, &theta, &phi);
    if (phi > kPiF) phi -= 2 * kPiF;
    theta -= 0.5f * kPiF;
    return phi >= -c.phiAngle * 0.5f && phi < c.phiAngle * 0.5f && theta >= -c.thetaAngle * 0.5f &&
           theta < c.thetaAngle * 0.5f;
}
__device__ __forceinline__ float idfPdf(const DevCamera &c, V3 d, float lu, float lv) {
    if (!idfInside(c, d, lu, lv)) return 0.0f;
    if (c.kind == 0) return c.imgPlaneDist * c.imgPlaneDist / ((d.z * d.z * d.z) * c.imgPlaneArea);
    // EquirectangularIDF::evaluatePDF takes 1 - y^2 for the sine (no root).
    float sinTheta = 1.0f - d.y * d.y;
    return 1.0f / (c.phiAngle * c.thetaAngle * sinTheta);
}
__device__ __forceinline__ void idfPixel(const DevCamera &c, V3 d, float lu, float lv, uint32_t w, uint32_t h,
                                         float* px, float* py) {
    if (c.kind == 0) {
        float s = c.objPlaneDist / d.z;
        float fx = d.x * s + lu, fy = d.y * s + lv;
        *px = w * (0.5f - fx / c.opWidth);
        *py = h * (0.5f - fy / c.opHeight);
        return;
    }
    float theta, phi;
    toPolarYUp(d, &theta, &phi);
    if (phi > kPiF) phi -= 2 * kPiF;
    theta -= 0.5f * kPiF;
    *px = (phi / c.phiAngle + 0.5f) * w;
    *py = (theta / c.thetaAngle + 0.5f) * h;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// Job::kernel up to the two subpath generations (BPTRenderer.cpp:107-172,
// VolumetricBPTRenderer.cpp:107-174).
template <bool VOL>
__global__ void kBptInit(DevScene sc, BptState st, BptWave wv) {
    const float selectWLPDF = kNumLambda / (kWavelengthHigh - kWavelengthLow);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < wv.numPaths; p += gridDim.x * blockDim.x) {
        const uint32_t s = p / wv.gridPositions;
        const uint32_t pos = p - s * wv.gridPositions;
        const uint32_t ix = pos % wv.gridW, iy = pos / wv.gridW;
        const uint64_t key = pathKey(wv.seed, (uint64_t)(wv.sampleBase + s) * wv.gridPositions + pos);
        st.rngKey[p] = make_uint2((uint32_t)key, (uint32_t)(key >> 32));
        Rng er{key, 0};
        (void)er.next();   // time
        const float pxf = ix + er.next();
        const float pyf = iy + er.next();
        const float wlOff = er.next();
        const uint32_t sel = min((uint32_t)(kNumLambda * er.next()), (uint32_t)(kNumLambda - 1));
        st.pix[p] = make_float2(pxf, pyf);
        st.wlOffset[p] = wlOff;
        st.sel[p] = sel;
        float lambdas[kNumLambda];
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) {
            lambdas[k] = lambdaAt(k, wlOff);
            st.L[(size_t)p * kNumLambda + k] = 0.0f;
        }

        // Light subpath: light vertex and its ray (BPTRenderer.cpp:122-149).
        {
            const uint32_t sp = p;
            Rng lr{key, kLightStream};
            float lightProb;
            int li;
            if (VOL) {   // Scene::selectLight over surfaces, media and the environment
                const int kind = selectLight3(sc, lr.next(), &li, &lightProb);
                if (kind != 0) li = -1;
            } else {     // Scene::selectSurfaceLight
                li = selectLight(sc, lr.next(), &lightProb);
            }
            const float u0 = lr.next(), u1 = lr.next();
            (void)lr.next();   // EDFSample::uComponent
            const float e0 = lr.next(), e1 = lr.next();
            BptGeom g;
            BptPdf pd;
            pd.cosIn = 0.0f;
            pd.rrProb = 1.0f;
            pd.revAreaPdf = 0.0f;
            pd.revRRProb = 0.0f;
            pd.pad0 = pd.pad1 = 0.0f;
            Spec a0, a;
            V3 org, dir;
            float dirPdf, cosLast, tmin;
            uint32_t info = 0;
            if (li >= 0) {
                // a point on an emitting triangle (surface_object.cpp:65-90,
                // TriangleSurfaceShape.cpp:357-406), a cosine direction from
                // its DiffuseEDF (basic_edfs.cpp:13-18)
                const DevPrim lpr = sc.prims[sc.lightPrims[li]];
                const float su = sqrtf(u0);
                const float b0 = 1.0f - su, b1 = u1 * su, b2 = 1.0f - b0 - b1;
                const float4 p0 = sc.vpos[lpr.v0], p1 = sc.vpos[lpr.v1], p2 = sc.vpos[lpr.v2];
                const V3 lp = rn_bary(b0, xyz(p0), b1, xyz(p1), b2, xyz(p2));
                const float4 n0 = sc.vnrm[lpr.v0], n1 = sc.vnrm[lpr.v1], n2 = sc.vnrm[lpr.v2];
                const float4 t0 = sc.vtan[lpr.v0], t1 = sc.vtan[lpr.v1], t2 = sc.vtan[lpr.v2];
                const V3 z = normalize(b0 * xyz(n0) + b1 * xyz(n1) + b2 * xyz(n2));
                V3 x = normalize(b0 * xyz(t0) + b1 * xyz(t1) + b2 * xyz(t2));
                const float dotNT = dot(z, x);
                if (fabsf(dotNT) >= 0.01f) x = normalize(x - dotNT * z);
                const Frame fr{x, cross(z, x), z};
                const V3 gn = V3{lpr.ngx, lpr.ngy, lpr.ngz};
                Spec Le0;
                evalSpectrum(sc, sc.materials[lpr.material].emit, lambdas, Le0);
                pd.areaPdf = lightProb * lpr.invArea;
                pd.flags = kVtxLight << kVfKindShift;   // LowFreq position
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) a0.v[k] = Le0.v[k] / pd.areaPdf;
                g.pg = make_float4(lp.x, lp.y, lp.z, 0.0f);
                g.ng = make_float4(gn.x, gn.y, gn.z, 0.0f);
                g.nz = make_float4(z.x, z.y, z.z, 0.0f);
                g.tx = make_float4(x.x, x.y, x.z, 0.0f);
                const V3 dl = cosineSampleHemisphere(e0, e1);
                dirPdf = dl.z * kInvPiF;
                dir = fr.fromLocal(dl);
                const float cosG = absDot(dir, gn);
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) a.v[k] = a0.v[k] * kInvPiF * (cosG / dirPdf);
                org = lp;
                tmin = kRayEpsilon;
                cosLast = dl.z;
            } else {
                // a point on the environment at infinity
                // (InfiniteSphereSurfaceObject::sample/sampleRay,
                // surface_object.cpp:201-272) and IBLEDF::sample (IBLEDF.cpp:11-16):
                // the direction is the inward normal, the origin a point of
                // the world disc facing it, outside the world sphere
                const float twoPi = 6.28318530717958647692f;
                float uvPdf, topPdf;
                uint32_t row, col;
                const float d1 = sampleAlias(sc.envTopAlias, sc.envTopPDF, sc.envMapH, u1, &topPdf, &row);
                const float d0 = sampleAlias(sc.envRowAlias + (size_t)row * sc.envMapW,
                                             sc.envRowPDF + (size_t)row * sc.envMapW, sc.envMapW, u0, &uvPdf, &col);
                uvPdf *= topPdf;
                const float phi = d0 * twoPi, theta = d1 * kPiF;
                float sph, cph, sth, cth;
                sincosf(phi, &sph, &cph);
                sincosf(theta, &sth, &cth);
                const V3 pos = V3{-sph * sth, cth, cph * sth};
                const V3 x = normalize(V3{-cph, 0.0f, -sph});
                const V3 gn = -pos;
                pd.areaPdf = lightProb * (uvPdf / (2.0f * kPiF * kPiF * sth));
                pd.flags = (kVtxLight << kVfKindShift) | kVfAtInf;
                Spec Le;   // emittance x EDF value (1 / pi)
                envRadiance(sc, phi / twoPi, theta / kPiF, lambdas, Le);
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) a0.v[k] = (Le.v[k] * kPiF) / pd.areaPdf;
                g.pg = make_float4(pos.x, pos.y, pos.z, 0.0f);
                g.ng = make_float4(gn.x, gn.y, gn.z, 0.0f);
                g.nz = make_float4(gn.x, gn.y, gn.z, 0.0f);
                g.tx = make_float4(x.x, x.y, x.z, 0.0f);
                dirPdf = 1.0f / sc.worldDiscArea;
                dir = gn;
                float dx, dy;
                concentricSampleDisk(e0, e1, &dx, &dy);
                // Vector3D::makeCoordinateSystem (Vector3D.h:61-67)
                const Frame db = frameFromZ(dir);
                const V3 vx = db.x, vy = db.y;
                const V3 wc = V3{sc.worldCenter[0], sc.worldCenter[1], sc.worldCenter[2]};
                org = wc + (1.1f * sc.worldRadius) * pos + sc.worldRadius * (dx * vx + dy * vy);
                const float cosG = absDot(dir, gn);
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) a.v[k] = a0.v[k] * kInvPiF * (cosG / dirPdf);
                tmin = 0.0f;
                cosLast = 1.0f;
                info = kAuxPrevAtInf;
            }
            st.geom[sp] = g;
            st.pdf[sp] = pd;
            storeAlpha(st.alpha, sp, a0);
            storeAlpha(st.alphaPend, sp, a);
            st.rayOrg[sp] = make_float4(org.x, org.y, org.z, tmin);
            st.rayDir[sp] = make_float4(dir.x, dir.y, dir.z, 0.0f);
            st.aux[sp] = make_float4(dirPdf, cosLast, 1.0f, __uint_as_float(info));
            st.rngCounter[sp] = lr.counter;
            st.numVerts[sp] = 1;
            queuePush(st.queue[0], st.counters + 0, sp, dirPdf != 0.0f);
        }

        // Eye subpath: lens vertex and its ray (BPTRenderer.cpp:151-172, camera.h:49-63).
        {
            const uint32_t sp = st.N + p;
            const DevCamera &c = sc.camera;
            const Frame fr = cameraFrame(c);
            const float l0 = er.next(), l1 = er.next();
            V3 orgLocal = V3{0.0f, 0.0f, 0.0f};
            float areaPdf = 1.0f;
            bool deltaPos = true;
            V3 dl;
            float dirPdf;
            const float u = pxf / wv.width, v = pyf / wv.height;
            if (c.kind == 0) {
                float lx, ly;
                concentricSampleDisk(l0, l1, &lx, &ly);
                orgLocal = V3{c.lensRadius * lx, c.lensRadius * ly, 0.0f};
                if (c.lensRadius > 0.0f) {
                    areaPdf = 1.0f / (kPiF * c.lensRadius * c.lensRadius);
                    deltaPos = false;
                }
                V3 pFocus = V3{c.opWidth * (0.5f - u), c.opHeight * (0.5f - v), c.objPlaneDist};
                dl = normalize(pFocus - orgLocal);
                dirPdf = c.imgPlaneDist * c.imgPlaneDist / ((dl.z * dl.z * dl.z) * c.imgPlaneArea);
            } else {
                float phi = c.phiAngle * (u - 0.5f);
                float theta = 0.5f * kPiF + c.thetaAngle * (v - 0.5f);
                float sp_, cp, st_, ct;
                sincosf(phi, &sp_, &cp);
                sincosf(theta, &st_, &ct);
                dl = V3{-sp_ * st_, ct, cp * st_};
                float sinTheta = sqrtf(1.0f - dl.y * dl.y);
                dirPdf = 1.0f / (c.phiAngle * c.thetaAngle * sinTheta);
            }
            const V3 org = V3{c.org[0], c.org[1], c.org[2]} + orgLocal.x * fr.x + orgLocal.y * fr.y;
            const float a0 = 1.0f / (areaPdf * selectWLPDF);
            BptGeom g;
            g.pg = make_float4(org.x, org.y, org.z, 0.0f);
            g.ng = make_float4(fr.z.x, fr.z.y, fr.z.z, 0.0f);
            g.nz = make_float4(fr.z.x, fr.z.y, fr.z.z, orgLocal.x);
            g.tx = make_float4(fr.x.x, fr.x.y, fr.x.z, orgLocal.y);
            st.geom[sp] = g;
            BptPdf pd;
            pd.cosIn = 0.0f;
            pd.areaPdf = areaPdf;
            pd.rrProb = 1.0f;
            pd.revAreaPdf = 0.0f;
            pd.revRRProb = 0.0f;
            pd.flags = (kVtxLens << kVfKindShift) | (deltaPos ? kVfDelta : 0u);
            pd.pad0 = pd.pad1 = 0.0f;
            st.pdf[sp] = pd;
            storeAlpha(st.alpha, sp, specConst(a0));
            const V3 dir = fr.fromLocal(dl);
            const float cosG = absDot(dir, fr.z);
            storeAlpha(st.alphaPend, sp, specConst(a0 * (cosG / dirPdf)));
            st.rayOrg[sp] = make_float4(org.x, org.y, org.z, 0.0f);
            st.rayDir[sp] = make_float4(dir.x, dir.y, dir.z, 0.0f);
            st.aux[sp] = make_float4(dirPdf, dl.z, 1.0f, __uint_as_float(0u));
            st.rngCounter[sp] = er.counter;
            st.numVerts[sp] = 1;
            queuePush(st.queue[0], st.counters + 0, sp, dirPdf != 0.0f);
            queuePush(st.connQueue, st.counters + st.D + 1, sp, true);   // t = 1
        }
    }
}

// Power-heuristic MIS weight (BPTRenderer.cpp:383-431) over the density
// records of one eye subpath and one light subpath.
struct MisSide {
    const BptPdf* pdf;
    uint32_t S, sp, n, minN;
    float e1, r1, e2, r2;   // densities of extending the other subpath by one and two vertices
};
__device__ __forceinline__ void kahanAdd(float &sum, float &comp, float v) {
    float cin = v - comp;
    float t = sum + cin;
    comp = (t - sum) - cin;
    sum = t;
}
__device__ void extendAndShorten(const MisSide &m, float &sum, float &comp) {
    if (m.n <= m.minN) return;
    const BptPdf end = m.pdf[(size_t)(m.n - 1) * m.S + m.sp];
    float ratio = m.e1 * m.r1 / (end.areaPdf * end.rrProb);
    bool sd = (end.flags & kVfDelta) != 0;
    if (!sd) kahanAdd(sum, comp, ratio * ratio);
    bool prev = sd;
    if (m.n - 1 > m.minN) {
        const BptPdf nv = m.pdf[(size_t)(m.n - 2) * m.S + m.sp];
        ratio *= m.e2 * m.r2 / (nv.areaPdf * nv.rrProb);
        sd = (nv.flags & kVfDelta) != 0;
        if (!sd && !prev) kahanAdd(sum, comp, ratio * ratio);
        prev = sd;
        for (int i = (int)m.n - 2; i > (int)m.minN; --i) {
            const BptPdf v = m.pdf[(size_t)(i - 1) * m.S + m.sp];
            ratio *= v.revAreaPdf * v.revRRProb / (v.areaPdf * v.rrProb);
            sd = (v.flags & kVfDelta) != 0;
            if (!sd && !prev) kahanAdd(sum, comp, ratio * ratio);
            prev = sd;
        }
    }
}
__device__ __forceinline__ float misWeight(const MisSide &eye, const MisSide &light) {
    float sum = 1.0f, comp = 0.0f;
    extendAndShorten(eye, sum, comp);     // shorten the eye subpath, not down to the lens
    extendAndShorten(light, sum, comp);   // shorten the light subpath, down to the implicit path
    return 1.0f / sum;
}

// Target of a contribution: the path's own sum, or a pixel of the splat film.
constexpr uint32_t kTargetSplat = 0x80000000u;

// Adds an unoccluded connection to the path's sum or, through the lens,
// to the splat film (both [.][16], four 16-byte atomic additions).
__device__ __forceinline__ void addConnection(const BptState &st, uint32_t target, const Spec &c) {
    float4* dst = reinterpret_cast<float4*>((target & kTargetSplat) ? st.splat : st.L) +
                  (size_t)(target & ~kTargetSplat) * (kNumLambda / 4);
#pragma unroll
    for (int k = 0; k < kNumLambda / 4; ++k) {
        const float4 v = make_float4(c.v[4 * k], c.v[4 * k + 1], c.v[4 * k + 2], c.v[4 * k + 3]);
        if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f) atomicAdd(dst + k, v);
    }
}

__device__ __forceinline__ Frame vertexFrame(const BptGeom &g) {
    V3 z = xyz(g.nz), x = xyz(g.tx);
    return Frame{x, cross(z, x), z};
}

// Film bin of a wavelength (SpectrumStorage::add, spectrum_types.h:729).
__device__ __forceinline__ uint32_t filmBin(float lambda) {
    const float f = __fmul_rn(divRange(__fsub_rn(lambda, kWavelengthLow)),
                              (float)kNumLambda);
    return min((uint32_t)f, (uint32_t)(kNumLambda - 1));
}

// Cosine factor of a vertex toward a direction: |cos| against the
// geometric normal, 1 for a point in the medium (MediumPoint::calcCosTerm,
// geometry.h:281-283).
__device__ __forceinline__ float vertexCos(const BptGeom &g, uint32_t flags, V3 d) {
    return ((flags >> kVfKindShift) & 3u) == kVtxMedium ? 1.0f : absDot(d, xyz(g.ng));
}

// One bounce of every live subpath: generateSubPath's loop body
// (BPTRenderer.cpp:304-379; VOL: VolumetricBPTRenderer.cpp:311-391, where
// Scene::interact may stop the ray at a scattering point in the medium).  A
// subpath holds at most D + 1 vertices.
template <bool VOL>
__global__ void __launch_bounds__(256, 2) kBptBounce(DevScene sc, BptState st, const uint32_t* __restrict__ inQueue,
                                                     const uint32_t* __restrict__ inCount, uint32_t* outQueue,
                                                     uint32_t* outCount) {
    const uint32_t n = *inCount;
    const float inf = __int_as_float(0x7f800000);
    const float twoPi = 6.28318530717958647692f;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        bool extend = false, conn = false;
        uint32_t sp = active ? inQueue[i] : 0;
        if (active) {
            const bool adjoint = sp < st.N;
            const uint32_t p = adjoint ? sp : sp - st.N;
            const float4 ro = st.rayOrg[sp], rd = st.rayDir[sp];
            const V3 org = xyz(ro), dir = xyz(rd);
            const float4 ax = st.aux[sp];
            const float dirPdf = ax.x, cosLast = ax.y, rrPend = ax.z;
            uint32_t info = __float_as_uint(ax.w);
            bool wlSelected = (info & kAuxWlSelected) != 0;
            const uint32_t k = st.numVerts[sp];   // index of the new vertex
            const float wlOff = st.wlOffset[p];
            const int sel = (int)st.sel[p];
            float lambdas[kNumLambda];
#pragma unroll
            for (int q = 0; q < kNumLambda; ++q) lambdas[q] = lambdaAt(q, wlOff);
            Rng rng{keyOf(st, p), st.rngCounter[sp]};
            Spec alpha;
            loadAlpha(st.alphaPend, sp, alpha);
            Hit h;
            traceClosest(sc, org, dir, ro.w, inf, &h);
            // Scene::interact (Scene.cpp:66-94): a collision in the medium
            // before the surface, with the medium throughput on the way.
            bool medHit = false;
            float tMed = 0.0f;
            V3 mparam = V3{0, 0, 0};
            Spec sigmaE;
            if (VOL && sc.medium.present) {
                evalSpectrum(sc, sc.medium.sigmaE, lambdas, sigmaE);
                Spec thr;
                medHit = mediumInteract(sc.medium, org, dir, ro.w, h.prim == kNoHit ? inf : h.t, sigmaE, sel,
                                        wlSelected, rng, &tMed, &mparam, thr);
#pragma unroll
                for (int q = 0; q < kNumLambda; ++q) alpha.v[q] *= thr.v[q];
            }
            if (!medHit && h.prim == kNoHit) {
                if (!adjoint && sc.envPresent) {
                    // The eye subpath reaches the environment: a vertex at
                    // infinity (InfiniteSphereSurfaceShape.cpp:50-80) whose
                    // implicit path is weighted against the light subpaths
                    // that start there (BPTRenderer.cpp:318-345); the vertex
                    // is then dropped and the subpath ends.
                    const float cosOut = absDot(-dir, -dir);
                    const BptPdf pd{cosOut, dirPdf * cosOut, rrPend, 0.0f, 0.0f,
                                    (kVtxSurface << kVfKindShift) | ((info & kAuxDelta) ? kVfDelta : 0u), 0.0f, 0.0f};
                    st.pdf[(size_t)k * st.S + sp] = pd;   // read by the MIS weight only
                    float theta, phi;
                    toPolarYUp(dir, &theta, &phi);
                    Spec Le;   // emittance x IBLEDF value
                    envRadiance(sc, phi / twoPi, theta / kPiF, lambdas, Le);
                    // the light probability Scene::intersect gives the
                    // environment; Scene::interact leaves the sphere's own 1
                    const float envProb = VOL ? 1.0f : sc.envImportance / (sc.surfImportance + sc.envImportance);
                    const float e1 = envProb * envAreaPdf(sc, phi, theta);
                    const float e2 = (1.0f / sc.worldDiscArea) * cosLast;
                    MisSide eye{st.pdf, st.S, sp, k + 1, 1, e1, 1.0f, e2, 1.0f};
                    MisSide light{st.pdf, st.S, p, 0, 0, 0.0f, 0.0f, 0.0f, 0.0f};
                    const float mis = misWeight(eye, light);
                    if (!isinf(mis) && !isnan(mis)) {
                        Spec c;
                        bool finite = true;
#pragma unroll
                        for (int q = 0; q < kNumLambda; ++q) {
                            c.v[q] = (mis * alpha.v[q]) * Le.v[q];
                            if (wlSelected && q == sel) c.v[q] *= kNumLambda;
                            finite &= isfinite(c.v[q]);
                        }
                        if (finite) addConnection(st, p, c);
                        else atomicAdd(&st.stats[2], 1ull);
                    }
                }
            } else {
                // the new vertex: a surface point or a scattering point in the medium
                V3 P, gn;
                Frame fr;
                DevMaterial mat;
                float invArea = 0.0f;
                if (medHit) {
                    P = rn_ray_point(org, dir, tMed);
                    fr = frameFromZ(normalize(dir));
                    gn = V3{0.0f, 0.0f, 0.0f};
                    const float dens = mediumDensity(sc.medium, mparam);
                    // alpha *= the extinction coefficient at the point
#pragma unroll
                    for (int q = 0; q < kNumLambda; ++q) alpha.v[q] *= dens * sigmaE.v[q];
                    mat.kind = kMatNull;
                    mat.emit = -1;
                } else {
                    const DevPrim pr = sc.prims[h.prim];
                    SurfPoint spt;
                    surfacePoint(sc, pr, org, dir, h.t, h.b1, h.b2, spt);
                    P = spt.p;
                    fr = spt.frame;
                    gn = spt.gn;
                    mat = sc.materials[pr.material];
                    invArea = pr.invArea;
                }
                const float dist2 = (info & kAuxPrevAtInf) ? 1.0f : sqLength(P - org);
                const V3 dirOut = fr.toLocal(-dir);
                const V3 gnl = fr.toLocal(gn);
                const float cosOut = medHit ? 1.0f : absDot(-dir, gn);
                const float areaPdf = dirPdf * cosOut / dist2;
                const size_t vi = (size_t)k * st.S + sp;
                BptGeom g;
                g.pg = make_float4(P.x, P.y, P.z, __uint_as_float(medHit ? 0u : sc.prims[h.prim].material));
                g.ng = make_float4(gn.x, gn.y, gn.z, dirOut.z);
                g.nz = make_float4(fr.z.x, fr.z.y, fr.z.z, dirOut.x);
                g.tx = make_float4(fr.x.x, fr.x.y, fr.x.z, dirOut.y);
                st.geom[vi] = g;
                BptPdf pd;
                pd.cosIn = cosOut;
                pd.areaPdf = areaPdf;
                pd.rrProb = rrPend;
                pd.revAreaPdf = 0.0f;
                pd.revRRProb = 0.0f;
                pd.flags = ((medHit ? kVtxMedium : kVtxSurface) << kVfKindShift) | (mat.kind << kVfMatShift) |
                           ((info & kAuxDelta) ? kVfDelta : 0u) | (wlSelected ? kVfWlSelected : 0u);
                pd.pad0 = pd.pad1 = 0.0f;
                st.pdf[vi] = pd;
                storeAlpha(st.alpha, vi, alpha);
                st.numVerts[sp] = k + 1;
                conn = !adjoint;

                // the vertex's BSDF: the material's, or the medium's
                // VolumetricBSDF (albedo x Henyey-Greenstein,
                // directional_distribution_functions.cpp:78-104,
                // medium_object.cpp:106-112)
                Bsdf B;
                if (medHit) {
                    B.kind = kMatNull;
                    B.ax = B.ay = 0.0f;
                    B.dispersive = false;
                    Spec sigmaS;
                    evalSpectrum(sc, sc.medium.sigmaS, lambdas, sigmaS);
                    const bool in = !outsideUnit(mparam);
#pragma unroll
                    for (int q = 0; q < kNumLambda; ++q)
                        B.a.v[q] = (in && sigmaE.v[q] > 0) ? sigmaS.v[q] / sigmaE.v[q] : 0.0f;
                } else {
                    makeBsdf(sc, mat, lambdas, wlSelected, B);
                }
                storeAlpha(st.bsdfA, vi, B.a);   // the connections reuse it (Lambert reflectance, albedo)
                // Implicit path, no light subpath vertex (BPTRenderer.cpp:318-340).
                if (!adjoint && !medHit && mat.emit >= 0) {
                    Spec Le0;
                    evalSpectrum(sc, mat.emit, lambdas, Le0);
                    const float Le1 = dirOut.z > 0.0f ? kInvPiF : 0.0f;
                    // The light probability of the hit: Scene::intersect gives
                    // the emitter's share of the surface aggregate times the
                    // surfaces' share of all lights (all emitting triangles
                    // weigh 1); Scene::interact (volumetric) leaves the
                    // surfaces' share out (Scene.cpp:80-84).
                    const float surfShare = VOL ? 1.0f : sc.surfImportance / (sc.surfImportance + sc.envImportance);
                    const float e1 = surfShare * sc.lightPMF[0] * invArea;
                    const float e2 = (dirOut.z > 0.0f ? dirOut.z * kInvPiF : 0.0f) * cosLast / dist2;
                    MisSide eye{st.pdf, st.S, sp, k + 1, 1, e1, 1.0f, e2, 1.0f};
                    MisSide light{st.pdf, st.S, p, 0, 0, 0.0f, 0.0f, 0.0f, 0.0f};
                    const float mis = misWeight(eye, light);
                    if (!isinf(mis) && !isnan(mis)) {
                        Spec c;
                        bool finite = true;
#pragma unroll
                        for (int q = 0; q < kNumLambda; ++q) {
                            c.v[q] = ((mis * alpha.v[q]) * Le0.v[q]) * Le1;
                            if (wlSelected && q == sel) c.v[q] *= kNumLambda;
                            finite &= isfinite(c.v[q]);
                        }
                        if (finite) addConnection(st, p, c);
                        else atomicAdd(&st.stats[2], 1ull);
                    }
                }
                if (k < st.D) {
                    BsdfSample bs;
                    Spec fs, revFs;
                    float revPdf;
                    if (medHit) {
                        // PhaseFunction sample (basic_phase_functions.cpp:38-52)
                        const float u0 = rng.next(), u1 = rng.next();
                        bs.dir = hgSample(sc.medium.g, u0, u1, &bs.pdf);
                        bs.type = kDirLowFreq;
                        revPdf = bs.pdf;
#pragma unroll
                        for (int q = 0; q < kNumLambda; ++q) fs.v[q] = B.a.v[q] * bs.pdf;
                        revFs = fs;
                    } else {
                        RevQuery q{dirOut, gnl, sel, adjoint};
                        const float uc = rng.next(), u0 = rng.next(), u1 = rng.next();
                        bsdfSampleRev(B, q, uc, u0, u1, &bs, fs, &revPdf, revFs);
                    }
                    if (bs.pdf != 0.0f && !specIsZero(fs)) {
                        if ((bs.type & kDirDispersive) && !wlSelected) wlSelected = true;
                        const V3 vecIn = fr.fromLocal(bs.dir);
                        const float cosIn = medHit ? 1.0f : absDot(vecIn, gn);
                        Spec weight;
#pragma unroll
                        for (int c = 0; c < kNumLambda; ++c) weight.v[c] = fs.v[c] * (cosIn / bs.pdf);
                        const float rr = stdMin(importance(weight, sel), 1.0f);
                        if (rng.next() < rr) {
#pragma unroll
                            for (int c = 0; c < kNumLambda; ++c) alpha.v[c] *= weight.v[c] / rr;
                            // reverse densities of the previous vertex
                            BptPdf* prev = &st.pdf[(size_t)(k - 1) * st.S + sp];
                            prev->revAreaPdf = revPdf * cosLast / dist2;
                            Spec rv;
#pragma unroll
                            for (int c = 0; c < kNumLambda; ++c) rv.v[c] = revFs.v[c] * cosOut / revPdf;
                            prev->revRRProb = stdMin(importance(rv, sel), 1.0f);
                            storeAlpha(st.alphaPend, sp, alpha);
                            st.rayOrg[sp] = make_float4(P.x, P.y, P.z, kRayEpsilon);
                            st.rayDir[sp] = make_float4(vecIn.x, vecIn.y, vecIn.z, 0.0f);
                            info = (dirIsDelta(bs.type) ? kAuxDelta : 0u) | (wlSelected ? kAuxWlSelected : 0u);
                            st.aux[sp] = make_float4(bs.pdf, cosIn, rr, __uint_as_float(info));
                            extend = true;
                        }
                    }
                }
            }
            st.rngCounter[sp] = rng.counter;
        }
        queuePush(outQueue, outCount, sp, active && extend);
        queuePush(st.connQueue, st.counters + st.D + 1, sp + (uint32_t)(st.numVerts[sp] - 1) * st.S,
                  active && conn);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st.stats[0], (unsigned long long)n);
}

// The BSDF of a surface vertex for its connections: Lambert from the
// reflectance cached at the vertex, other kinds evaluated again.
__device__ __forceinline__ void vertexBsdf(const DevScene &sc, const BptState &st, size_t vi, uint32_t material,
                                           uint32_t flags, const float* lambdas, Bsdf &B) {
    if (((flags >> kVfMatShift) & 0xfu) == kMatMatte) {
        B.kind = kMatMatte;
        B.ax = B.ay = 0.0f;
        B.dispersive = (flags & kVfWlSelected) == 0;
        loadAlpha(st.bsdfA, vi, B.a);
    } else {
        makeBsdf(sc, sc.materials[material], lambdas, (flags & kVfWlSelected) != 0, B);
    }
}

// One connection (BPTRenderer.cpp:174-280; VOL: VolumetricBPTRenderer.cpp:
// 174-286): eye vertex evi (t = its index + 1) with light vertex s of the
// same path.  Returns false when the connection adds nothing (zero
// connection term, invalid MIS weight) or is dropped as non-finite
// (*dropped set); else the shadow ray and the contribution, *target = path,
// or pixel | kTargetSplat when it lands through the lens (t = 1).  Without
// a medium the splat contribution comes binned into film bins; VOL leaves it
// per wavelength for the transmittance.
template <bool VOL>
__device__ bool connectOne(const DevScene &sc, const BptState &st, uint32_t evi, uint32_t s, uint32_t width,
                           uint32_t height, float4* rayOrg, float4* rayDir, Spec &c, uint32_t* target,
                           bool* dropped) {
    *dropped = false;
    const uint32_t k = evi / st.S;            // eye vertex index, t = k + 1
    const uint32_t esp = evi - k * st.S;
    const uint32_t p = esp - st.N;
    const uint32_t t = k + 1;
    const int sel = (int)st.sel[p];
    const float wlOff = st.wlOffset[p];
    float lambdas[kNumLambda];
#pragma unroll
    for (int q = 0; q < kNumLambda; ++q) lambdas[q] = lambdaAt(q, wlOff);
    const BptGeom eg = st.geom[evi];
    const BptPdf ep = st.pdf[evi];
    const V3 eP = xyz(eg.pg);
    const Frame eF = vertexFrame(eg);
    const uint32_t eKind = ep.flags >> kVfKindShift & 3u;
    const size_t lvi = (size_t)(s - 1) * st.S + p;
    const BptGeom lg = st.geom[lvi];
    const BptPdf lpd = st.pdf[lvi];
    const uint32_t lKind = lpd.flags >> kVfKindShift & 3u;
    const V3 lP = xyz(lg.pg);
    const Frame lF = vertexFrame(lg);
    // InteractionPoint::getDirectionFrom (geometry.h:147-157): a vertex at
    // infinity is a direction at squared distance 1
    const bool lInf = (lpd.flags & kVfAtInf) != 0;
    V3 cv = lInf ? lP : lP - eP;
    const float dist2 = lInf ? 1.0f : sqLength(cv);
    cv = lInf ? normalize(cv) : cv * (1.0f / sqrtf(dist2));
    const float cosLightEnd = vertexCos(lg, lpd.flags, cv);
    const float cosEyeEnd = vertexCos(eg, ep.flags, cv);
    const float G = cosEyeEnd * cosLightEnd / dist2;
    // light end: EDF of the light vertex, the adjoint BSDF or the medium's
    const V3 lc = lF.toLocal(-cv);
    Spec lDDF, lRev;
    float lExt1DirPdf, eExt2DirPdf = 0.0f;
    if (lInf) {   // IBLEDF (IBLEDF.cpp:18-30)
        lDDF = specConst(kInvPiF);
        lRev = lDDF;
        lExt1DirPdf = 1.0f / sc.worldDiscArea;
    } else if (s == 1) {   // DiffuseEDF (basic_edfs.cpp:20-30)
        lDDF = specConst(lc.z > 0.0f ? kInvPiF : 0.0f);
        lRev = lDDF;
        lExt1DirPdf = lc.z > 0.0f ? lc.z * kInvPiF : 0.0f;
    } else if (VOL && lKind == kVtxMedium) {   // albedo x Henyey-Greenstein, symmetric
        Spec albedo;
        loadAlpha(st.bsdfA, lvi, albedo);
        lExt1DirPdf = hgValue(sc.medium.g, lc.z);
        eExt2DirPdf = lExt1DirPdf;
#pragma unroll
        for (int q = 0; q < kNumLambda; ++q) lDDF.v[q] = albedo.v[q] * lExt1DirPdf;
        lRev = lDDF;
    } else {
        Bsdf lB;
        vertexBsdf(sc, st, lvi, __float_as_uint(lg.pg.w), lpd.flags, lambdas, lB);
        RevQuery lq{V3{lg.nz.w, lg.tx.w, lg.ng.w}, lF.toLocal(xyz(lg.ng)), sel, true};
        bsdfEvalRev(lB, lq, lc, lDDF, lRev);
        lExt1DirPdf = bsdfPdfRev(lB, lq, lc, &eExt2DirPdf);
    }
    // eye end: importance of the lens, the BSDF or the medium's
    const V3 ec = eF.toLocal(cv);
    Spec eDDF, eRev;
    float eExt1DirPdf, lExt2DirPdf = 0.0f;
    if (eKind == kVtxLens) {
        eDDF = specConst(idfInside(sc.camera, ec, eg.nz.w, eg.tx.w) ? 1.0f : 0.0f);
        eRev = eDDF;
        eExt1DirPdf = idfPdf(sc.camera, ec, eg.nz.w, eg.tx.w);
    } else if (VOL && eKind == kVtxMedium) {
        Spec albedo;
        loadAlpha(st.bsdfA, evi, albedo);
        eExt1DirPdf = hgValue(sc.medium.g, ec.z);
        lExt2DirPdf = eExt1DirPdf;
#pragma unroll
        for (int q = 0; q < kNumLambda; ++q) eDDF.v[q] = albedo.v[q] * eExt1DirPdf;
        eRev = eDDF;
    } else {
        Bsdf eB;
        vertexBsdf(sc, st, evi, __float_as_uint(eg.pg.w), ep.flags, lambdas, eB);
        RevQuery eq{V3{eg.nz.w, eg.tx.w, eg.ng.w}, eF.toLocal(xyz(eg.ng)), sel, false};
        bsdfEvalRev(eB, eq, ec, eDDF, eRev);
        eExt1DirPdf = bsdfPdfRev(eB, eq, ec, &lExt2DirPdf);
    }
    Spec ct;
    bool nz = false;
#pragma unroll
    for (int q = 0; q < kNumLambda; ++q) {
        ct.v[q] = lDDF.v[q] * G * eDDF.v[q];
        nz |= ct.v[q] != 0.0f;
    }
    if (!nz) return false;
    if ((lpd.flags & kVfWlSelected) || (ep.flags & kVfWlSelected)) {
#pragma unroll
        for (int q = 0; q < kNumLambda; ++q)
            if (q == sel) ct.v[q] *= kNumLambda;
    }
    // densities of the two subpaths' first and second extensions
    const float lExt1Area = lExt1DirPdf * cosEyeEnd / dist2;
    Spec tmp;
#pragma unroll
    for (int q = 0; q < kNumLambda; ++q) tmp.v[q] = lDDF.v[q] * cosLightEnd / lExt1DirPdf;
    const float lExt1RR = s > 1 ? stdMin(importance(tmp, sel), 1.0f) : 1.0f;
    float lExt2Area = 0.0f, lExt2RR = 0.0f;
    if (t > 1) {
        const BptGeom g2 = st.geom[evi - st.S];
        const uint32_t f2 = st.pdf[evi - st.S].flags;
        V3 d2 = eP - xyz(g2.pg);
        const float dd2 = sqLength(d2);
        d2 = d2 * (1.0f / sqrtf(dd2));
        lExt2Area = lExt2DirPdf * vertexCos(g2, f2, d2) / dd2;
#pragma unroll
        for (int q = 0; q < kNumLambda; ++q) tmp.v[q] = eRev.v[q] * ep.cosIn / lExt2DirPdf;
        lExt2RR = stdMin(importance(tmp, sel), 1.0f);
    }
    const float eExt1Area = eExt1DirPdf * cosLightEnd / dist2;
#pragma unroll
    for (int q = 0; q < kNumLambda; ++q) tmp.v[q] = eDDF.v[q] * cosEyeEnd / eExt1DirPdf;
    const float eExt1RR = t > 1 ? stdMin(importance(tmp, sel), 1.0f) : 1.0f;
    float eExt2Area = 0.0f, eExt2RR = 0.0f;
    if (s > 1) {
        const BptGeom l2 = st.geom[lvi - st.S];
        const uint32_t f2 = st.pdf[lvi - st.S].flags;
        const bool l2Inf = (f2 & kVfAtInf) != 0;
        V3 d2 = l2Inf ? xyz(l2.pg) : xyz(l2.pg) - lP;
        const float dd2 = l2Inf ? 1.0f : sqLength(d2);
        d2 = l2Inf ? normalize(d2) : d2 * (1.0f / sqrtf(dd2));
        eExt2Area = eExt2DirPdf * vertexCos(l2, f2, d2) / dd2;
#pragma unroll
        for (int q = 0; q < kNumLambda; ++q) tmp.v[q] = lRev.v[q] * lpd.cosIn / eExt2DirPdf;
        eExt2RR = stdMin(importance(tmp, sel), 1.0f);
    }
    MisSide eyeSide{st.pdf, st.S, esp, t, 1, lExt1Area, lExt1RR, lExt2Area, lExt2RR};
    MisSide lightSide{st.pdf, st.S, p, s, 0, eExt1Area, eExt1RR, eExt2Area, eExt2RR};
    const float mis = misWeight(eyeSide, lightSide);
    if (isinf(mis) || isnan(mis)) return false;
    Spec lAlpha, eAlpha;
    loadAlpha(st.alpha, lvi, lAlpha);
    loadAlpha(st.alpha, evi, eAlpha);
    bool finite = true;
#pragma unroll
    for (int q = 0; q < kNumLambda; ++q) {
        c.v[q] = ((mis * lAlpha.v[q]) * ct.v[q]) * eAlpha.v[q];
        finite &= isfinite(c.v[q]);
    }
    if (!finite) {
        *dropped = true;
        return false;
    }
    // Scene::testVisibility (Scene.cpp:96-135)
    *rayOrg = make_float4(eP.x, eP.y, eP.z, kRayEpsilon);
    if (lInf) {
        *rayDir = make_float4(cv.x, cv.y, cv.z, 3.402823466e+38f);
    } else {
        const float dist = length(lP - eP);
        const V3 sd = (lP - eP) * (1.0f / dist);
        *rayDir = make_float4(sd.x, sd.y, sd.z, dist * (1 - kRayEpsilon));
    }
    if (t > 1) {
        *target = p;
        return true;
    }
    float hx, hy;
    idfPixel(sc.camera, ec, eg.nz.w, eg.tx.w, width, height, &hx, &hy);
    const uint32_t ipx = min((uint32_t)fmaxf(hx, 0.0f), width - 1);
    const uint32_t ipy = min((uint32_t)fmaxf(hy, 0.0f), height - 1);
    *target = (ipy * width + ipx) | kTargetSplat;
    if (VOL) return true;
    // SpectrumStorage::add (spectrum_types.h:725-734): wavelength -> film bin
    const float recBinWidth = kNumLambda / (kWavelengthHigh - kWavelengthLow);
    Spec binned = specConst(0.0f);
#pragma unroll
    for (int q = 0; q < kNumLambda; ++q) {
        const uint32_t bin = filmBin(lambdas[q]);
#pragma unroll
        for (int b = 0; b < kNumLambda; ++b)
            if (b == (int)bin) binned.v[b] += c.v[q] * recBinWidth;
    }
    c = binned;
    return true;
}

// Adds one wavelength of a volumetric connection (film bin for a splat).
__device__ __forceinline__ void addConnectionWl(const BptState &st, uint32_t target, uint32_t p, int wl, float v) {
    if (v == 0.0f) return;
    if (target & kTargetSplat) {
        const float recBinWidth = kNumLambda / (kWavelengthHigh - kWavelengthLow);
        const uint32_t bin = filmBin(lambdaAt(wl, st.wlOffset[p]));
        atomicAdd(&st.splat[(size_t)(target & ~kTargetSplat) * kNumLambda + bin], v * recBinWidth);
    } else {
        atomicAdd(&st.L[(size_t)target * kNumLambda + wl], v);
    }
}

// Connections of the queued eye vertices [first, first + count) with every
// light vertex of their paths, spread over the lanes of a warp: a warp takes
// 32 eye vertices, prefix-sums their light-subpath lengths and gives each
// lane one (eye vertex, light vertex) pair per round, so lanes stay busy
// whatever the subpath lengths.  Connections that contribute go to the
// shadow queue.
template <bool VOL>
__global__ void __launch_bounds__(256, 2) kBptConnect(DevScene sc, BptState st, uint32_t width, uint32_t height,
                                                      const uint32_t* __restrict__ queue,
                                                      const uint32_t* __restrict__ count, uint32_t first,
                                                      uint32_t maxItems, uint32_t* shCount) {
    const uint32_t total0 = *count;
    const uint32_t end = total0 > first ? min(total0, first + maxItems) : first;
    const uint32_t n = end - first;
    queue += first;
    const uint32_t lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    unsigned long long dropped = 0;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t item = base + lane;
        uint32_t evi = 0, nL = 0;
        if (item < n) {
            evi = queue[item];
            const uint32_t p = evi % st.S - st.N;
            nL = st.numVerts[p];
        }
        uint32_t incl = nL;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(full, incl, d);
            if (lane >= (uint32_t)d) incl += v;
        }
        const uint32_t total = __shfl_sync(full, incl, 31);
        for (uint32_t j0 = 0; j0 < total; j0 += 32) {
            const uint32_t j = j0 + lane;
            // owner lane: the number of lanes whose inclusive sum is <= j
            uint32_t o = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
                const uint32_t v = __shfl_sync(full, incl, o + step - 1);
                if (v <= j) o += step;
            }
            o = min(o, 31u);
            const uint32_t ev = __shfl_sync(full, evi, o);
            const uint32_t first = __shfl_sync(full, incl, o) - __shfl_sync(full, nL, o);
            const uint32_t sIdx = j - first + 1;
            bool push = false;
            float4 ro, rd;
            Spec c;
            uint32_t target = 0;
            if (j < total) {
                bool drop;
                push = connectOne<VOL>(sc, st, ev, sIdx, width, height, &ro, &rd, c, &target, &drop);
                dropped += drop ? 1 : 0;
            }
            const unsigned mask = __ballot_sync(full, push);
            uint32_t slot = 0;
            if (lane == 0 && mask) slot = atomicAdd(shCount, (uint32_t)__popc(mask));
            slot = __shfl_sync(full, slot, 0) + __popc(mask & ((1u << lane) - 1));
            if (push) {
                const uint32_t p = ev % st.S - st.N;
                const uint32_t meta = (ev / st.S) << 8 | sIdx;
                // a pass never holds more connections than the queue (see renderBpt)
                st.cRay[2 * (size_t)slot] = ro;
                st.cRay[2 * (size_t)slot + 1] = rd;
                storeAlpha(st.cContrib, slot, c);
                st.cTarget[slot] = target;
                if (VOL) {
                    st.cPath[slot] = p;
                    st.cMeta[slot] = meta;
                }
            }
        }
    }
    if (dropped) atomicAdd(&st.stats[2], dropped);
}

// Shadow rays of the queued connections; unoccluded ones add their
// contribution, or (VOL) wait for their medium transmittance.
template <bool VOL>
__global__ void __launch_bounds__(256, SLRGPU_TRACE_MIN_BLOCKS) kBptShadow(DevScene sc, BptState st,
                                                                         const uint32_t* __restrict__ shCount,
                                                                         uint32_t* medCount) {
    const uint32_t n = min(*shCount, st.connCap);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool pushMedium = false;
        if (i < n) {
            const float4 o = st.cRay[2 * (size_t)i], d = st.cRay[2 * (size_t)i + 1];
            if (!traceAny(sc, xyz(o), xyz(d), o.w, d.w)) {
                if (VOL) {
                    pushMedium = true;
                } else {
                    Spec c;
                    loadAlpha(st.cContrib, i, c);
                    addConnection(st, st.cTarget[i], c);
                }
            }
        }
        if (VOL) queuePush(st.mQueue, medCount, i, pushMedium);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st.stats[1], (unsigned long long)n);
}

// Medium transmittance of the unoccluded volumetric connections
// (Scene::testVisibility, Scene.cpp:114-135, with
// MediumObjectAggregate::evaluateTransmittance), one walk per (connection,
// wavelength) as the path tracer's shadow rays do: the kernel's wavelengths
// are never selected there, so every wavelength is tracked, each from its own
// counter range of a stream of the connection; lanes take the next walk as
// soon as theirs ends (TrWalk).
__global__ void __launch_bounds__(256, SLRGPU_MEDIUM_MIN_BLOCKS) kVbptMedium(DevScene sc, BptState st,
                                                                           const uint32_t* __restrict__ medCount,
                                                                           uint32_t* take) {
    const uint32_t n = *medCount * kNumLambda;
    uint32_t poolNext = 0, poolEnd = 0;
    TrWalk q;
    uint32_t slot = 0;
    int wl = 0;
    float cw = 0.0f;
    bool walking = false, exhausted = false;
    for (;;) {
        for (;;) {
            const bool need = !walking && !exhausted;
            if (!__any_sync(0xffffffffu, need)) break;
            const uint32_t item = trTake(need, take, poolNext, poolEnd);
            if (!need) continue;
            if (item >= n) {
                exhausted = true;
                continue;
            }
            slot = st.mQueue[item / kNumLambda];
            wl = (int)(item % kNumLambda);
            cw = reinterpret_cast<const float*>(st.cContrib)[(size_t)slot * kNumLambda + wl];
            if (cw == 0.0f) continue;
            const uint32_t p = st.cPath[slot];
            if (!sc.medium.present) {
                addConnectionWl(st, st.cTarget[slot], p, wl, cw);
                continue;
            }
            const float4 o = st.cRay[2 * (size_t)slot], d = st.cRay[2 * (size_t)slot + 1];
            const Rng rng{mix64(keyOf(st, p) ^ (0x9e3779b97f4a7c15ull * (st.cMeta[slot] + 1))), (uint32_t)wl << 24};
            const float sig = evalSpectrumAt(sc, sc.medium.sigmaE, lambdaAt(wl, st.wlOffset[p]));
            walking = trBegin(sc.medium, q, xyz(o), xyz(d), o.w, d.w, sig, true, rng);
            if (!walking) addConnectionWl(st, st.cTarget[slot], p, wl, cw * q.T);
        }
        if (!__any_sync(0xffffffffu, walking)) break;
        if (walking) {
            walking = trStep(sc.medium, q);
            if (!walking) addConnectionWl(st, st.cTarget[slot], st.cPath[slot], wl, cw * q.T);
        }
    }
}

// The wave's contributions into the compensated film: per pixel, the sums of
// its paths in sample order (grid positions clamped into the last row /
// column as ImageSensor::add does), then the splat film, which is cleared.
__global__ void kBptAccumulate(BptState st, BptWave wv, float* filmSum, float* filmComp) {
    const float recBinWidth = kNumLambda / (kWavelengthHigh - kWavelengthLow);
    const uint32_t P = wv.width * wv.height;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < P; pix += gridDim.x * blockDim.x) {
        float sum[kNumLambda], comp[kNumLambda];
#pragma unroll
        for (int b = 0; b < kNumLambda; ++b) {
            sum[b] = filmSum[(size_t)b * P + pix];
            comp[b] = filmComp[(size_t)b * P + pix];
        }
        const uint32_t x = pix % wv.width, y = pix / wv.width;
        const uint32_t xEnd = x + 1 == wv.width ? wv.gridW : x + 1;
        const uint32_t yEnd = y + 1 == wv.height ? wv.gridH : y + 1;
        for (uint32_t s = 0; s < wv.samples; ++s)
        for (uint32_t gy = y; gy < yEnd; ++gy)
        for (uint32_t gx = x; gx < xEnd; ++gx) {
            const uint32_t p = s * wv.gridPositions + gy * wv.gridW + gx;
            const float wlOff = st.wlOffset[p];
            float addend[kNumLambda];
#pragma unroll
            for (int b = 0; b < kNumLambda; ++b) addend[b] = 0.0f;
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) {
                const float c = st.L[(size_t)p * kNumLambda + i];
                const float lam = lambdaAt(i, wlOff);
                const float f = __fmul_rn(divRange(__fsub_rn(lam, kWavelengthLow)),
                                          (float)kNumLambda);
                const uint32_t bin = min((uint32_t)f, (uint32_t)(kNumLambda - 1));
#pragma unroll
                for (int b = 0; b < kNumLambda; ++b)
                    if (b == (int)bin) addend[b] += c * recBinWidth;
            }
#pragma unroll
            for (int b = 0; b < kNumLambda; ++b) kahanAdd(sum[b], comp[b], addend[b]);
        }
#pragma unroll
        for (int b = 0; b < kNumLambda; ++b) {
            float* sp = &st.splat[(size_t)pix * kNumLambda + b];
            kahanAdd(sum[b], comp[b], *sp);
            *sp = 0.0f;
            filmSum[(size_t)b * P + pix] = sum[b];
            filmComp[(size_t)b * P + pix] = comp[b];
        }
    }
}

int gridFor(const void* kernel, int block) {
    int dev = 0, sms = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, block, 0);
    return std::max(1, sms * std::max(1, perSM));
}

struct BptGrids {
    int init[2], bounce[2], connect[2], shadow[2], medium, accumulate;
};
const BptGrids &bptGrids() {
    static BptGrids g;
    static std::once_flag once;
    std::call_once(once, [&]() {
        g.init[0] = gridFor((const void*)kBptInit<false>, 256);
        g.init[1] = gridFor((const void*)kBptInit<true>, 256);
        g.bounce[0] = gridFor((const void*)kBptBounce<false>, 256);
        g.bounce[1] = gridFor((const void*)kBptBounce<true>, 256);
        g.connect[0] = gridFor((const void*)kBptConnect<false>, 256);
        g.connect[1] = gridFor((const void*)kBptConnect<true>, 256);
        g.shadow[0] = gridFor((const void*)kBptShadow<false>, 256);
        g.shadow[1] = gridFor((const void*)kBptShadow<true>, 256);
        g.medium = gridFor((const void*)kVbptMedium, 256);
        g.accumulate = gridFor((const void*)kBptAccumulate, 256);
    });
    return g;
}

}  // namespace

// Paths per wave of the bidirectional tracer when samples_per_wave is 0,
// and the device memory its path state may take (about 9.5 KB per path at
// 16 vertices per subpath).  Measured on the 512 x 512, 16 spp box: 1 Mi
// paths in 8 GB 121.8 M path samples/s, 2 Mi in 24 GB 141.2 M, 4 Mi (the
// whole frame) in 48 GB 145.9 M.
#ifndef SLRGPU_BPT_WAVE_PATHS
#define SLRGPU_BPT_WAVE_PATHS (1u << 22)
#endif
#ifndef SLRGPU_BPT_STATE_GB
#define SLRGPU_BPT_STATE_GB 48
#endif
constexpr uint64_t kBptStateBudget = (uint64_t)SLRGPU_BPT_STATE_GB << 30;
// Connections the shadow queue holds per path of a wave; the connection
// passes take kConnPerPath / (max_depth + 1) paths' worth of eye vertices.
constexpr uint32_t kConnPerPath = 16;

struct BptEngine {
    BptState st{};
    std::vector<void*> allocs;
    uint32_t capN = 0, capD = 0, capPixels = 0;
    ~BptEngine() { release(); }
    void release() {
        for (void* p : allocs) cudaFree(p);
        allocs.clear();
        st = BptState{};
        capN = capD = capPixels = 0;
    }
    template <typename T>
    T* alloc(size_t n, cudaError_t* e) {
        void* p = nullptr;
        *e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (*e != cudaSuccess) return nullptr;
        allocs.push_back(p);
        return (T*)p;
    }
    int ensure(uint32_t N, uint32_t D, uint32_t pixels) {
        if (N <= capN && D <= capD && pixels <= capPixels && !allocs.empty()) return SLRGPU_OK;
        release();
        cudaError_t e = cudaSuccess;
        const size_t S = 2ull * N, V = (size_t)(D + 1) * S;
        BptState s{};
        s.N = N;
        s.S = (uint32_t)S;
        s.D = D;
        bool ok = (s.geom = alloc<BptGeom>(V, &e)) && (s.pdf = alloc<BptPdf>(V, &e)) &&
                  (s.alpha = alloc<float4>(V * 4, &e)) && (s.bsdfA = alloc<float4>(V * 4, &e)) &&
                  (s.rayOrg = alloc<float4>(S, &e)) &&
                  (s.rayDir = alloc<float4>(S, &e)) && (s.alphaPend = alloc<float4>(S * 4, &e)) &&
                  (s.aux = alloc<float4>(S, &e)) && (s.rngCounter = alloc<uint32_t>(S, &e)) &&
                  (s.numVerts = alloc<uint32_t>(S, &e)) && (s.rngKey = alloc<uint2>(N, &e)) &&
                  (s.pix = alloc<float2>(N, &e)) && (s.wlOffset = alloc<float>(N, &e)) &&
                  (s.sel = alloc<uint32_t>(N, &e)) && (s.L = alloc<float>((size_t)N * kNumLambda, &e)) &&
                  (s.splat = alloc<float>((size_t)pixels * kNumLambda, &e)) &&
                  (s.queue[0] = alloc<uint32_t>(S, &e)) && (s.queue[1] = alloc<uint32_t>(S, &e)) &&
                  (s.connQueue = alloc<uint32_t>((size_t)N * (D + 1), &e)) &&
                  (s.cRay = alloc<float4>((size_t)kConnPerPath * N * 2, &e)) &&
                  (s.cContrib = alloc<float4>((size_t)kConnPerPath * N * 4, &e)) &&
                  (s.cTarget = alloc<uint32_t>((size_t)kConnPerPath * N, &e)) &&
                  (s.cPath = alloc<uint32_t>((size_t)kConnPerPath * N, &e)) &&
                  (s.cMeta = alloc<uint32_t>((size_t)kConnPerPath * N, &e)) &&
                  (s.mQueue = alloc<uint32_t>((size_t)kConnPerPath * N, &e)) &&
                  (s.counters = alloc<uint32_t>(D + 5, &e)) && (s.stats = alloc<unsigned long long>(4, &e));
        if (!ok) {
            release();
            setError(std::string("bidirectional path state allocation failed: ") + cudaGetErrorString(e));
            return SLRGPU_ERR_OUT_OF_MEMORY;
        }
        s.splatPixels = pixels;
        s.connCap = kConnPerPath * N;
        if (cudaMemset(s.splat, 0, (size_t)pixels * kNumLambda * sizeof(float)) != cudaSuccess) {
            release();
            setError("bidirectional path state initialisation failed");
            return SLRGPU_ERR_CUDA;
        }
        st = s;
        capN = N;
        capD = D;
        capPixels = pixels;
        return SLRGPU_OK;
    }
};

BptEngine* bptEngineCreate() { return new BptEngine(); }
void bptEngineDestroy(BptEngine* e) { delete e; }

uint64_t bptStateBytesPerPath(uint32_t maxDepth) {
    const uint64_t V = 2ull * (maxDepth + 1);
    return V * (sizeof(BptGeom) + sizeof(BptPdf) + 128) + 2 * (16 + 16 + 64 + 16 + 4 + 4) + 8 + 8 + 4 + 4 +
           4 * kNumLambda + 8 + 4ull * (maxDepth + 1) + kConnPerPath * (32 + 64 + 16);
}

int renderBpt(BptEngine &eng, const DeviceScene &ds, const slrgpu_settings &s, float* filmSum, float* filmComp,
              cudaStream_t stream, uint64_t* launches, std::vector<cudaEvent_t>* eventPool,
              slrgpu_render_stats* stats) {
    const bool vol = s.volumetric != 0;
    if (ds.sc.numLights == 0 && !ds.sc.envPresent) {
        setError("bidirectional path tracing needs a light (an emitting surface or an environment)");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (s.max_depth < 1 || s.max_depth > 63) {
        setError("bidirectional path tracing takes max_depth in [1, 63] (vertices per subpath after the first)");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const uint32_t D = s.max_depth;
    const uint32_t gridW = (s.width + 7) / 8 * 8, gridH = (s.height + 7) / 8 * 8;
    const uint32_t G = gridW * gridH;
    const uint64_t perPath = bptStateBytesPerPath(D);
    uint64_t want = s.samples_per_wave ? (uint64_t)s.samples_per_wave * G
                                       : std::max<uint64_t>(G, (uint64_t)SLRGPU_BPT_WAVE_PATHS / G * G);
    const uint64_t budgetPaths = std::max<uint64_t>(G, kBptStateBudget / perPath / G * G);
    if (!s.samples_per_wave) want = std::min(want, budgetPaths);
    uint32_t S = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1, want / G), s.spp);
    const uint64_t N64 = (uint64_t)S * G;
    if (N64 * (D + 1) * 2 >= (1ull << 32)) {
        setError("bidirectional wave too large (paths x vertices exceed 2^32)");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const uint32_t N = (uint32_t)N64;
    const uint32_t P = s.width * s.height;
    int rc = eng.ensure(N, D, P);
    if (rc != SLRGPU_OK) return rc;
    BptState st = eng.st;
    st.D = D;
    st.splatPixels = P;
    const BptGrids &g = bptGrids();
    if (cudaMemsetAsync(st.stats, 0, 4 * sizeof(unsigned long long), stream) != cudaSuccess) {
        setError("cudaMemsetAsync failed");
        return SLRGPU_ERR_CUDA;
    }
    struct Mark { int cls; size_t ev; };
    std::vector<Mark> marks;
    size_t used = 0;
    auto mark = [&](int cls) {
        if (!eventPool) return;
        if (used == eventPool->size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            eventPool->push_back(e);
        }
        marks.push_back(Mark{cls, used});
        cudaEventRecord((*eventPool)[used++], stream);
    };
    auto markEnd = [&]() {
        if (!eventPool) return;
        if (used == eventPool->size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            eventPool->push_back(e);
        }
        cudaEventRecord((*eventPool)[used++], stream);
    };
    uint64_t nl = 0;
    for (uint32_t base = 0; base < s.spp; base += S) {
        BptWave wv;
        wv.width = s.width;
        wv.height = s.height;
        wv.gridW = gridW;
        wv.gridH = gridH;
        wv.gridPositions = G;
        wv.sampleBase = s.sample_base + base;
        wv.samples = std::min(S, s.spp - base);
        wv.seed = s.seed;
        wv.numPaths = wv.samples * G;
        cudaMemsetAsync(st.counters, 0, (D + 5) * sizeof(uint32_t), stream);
        mark(SLRGPU_KERNEL_RAYGEN);
        if (vol) kBptInit<true><<<g.init[1], 256, 0, stream>>>(ds.sc, st, wv);
        else kBptInit<false><<<g.init[0], 256, 0, stream>>>(ds.sc, st, wv);
        markEnd();
        ++nl;
        for (uint32_t b = 0; b < D; ++b) {
            mark(SLRGPU_KERNEL_EXTEND);
            if (vol)
                kBptBounce<true><<<g.bounce[1], 256, 0, stream>>>(ds.sc, st, st.queue[b & 1], st.counters + b,
                                                                   st.queue[(b + 1) & 1], st.counters + b + 1);
            else
                kBptBounce<false><<<g.bounce[0], 256, 0, stream>>>(ds.sc, st, st.queue[b & 1], st.counters + b,
                                                                    st.queue[(b + 1) & 1], st.counters + b + 1);
            markEnd();
            ++nl;
        }
        // Connections in passes of at most connCap / (D + 1) eye vertices:
        // each has at most D + 1 light vertices to connect to, so a pass
        // never overfills the shadow queue.  The number of eye vertices is
        // read back once per wave.
        uint32_t items = 0;
        if (cudaMemcpyAsync(&items, st.counters + D + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess) {
            setError("bidirectional connection count readback failed");
            return SLRGPU_ERR_CUDA;
        }
        const uint32_t perPass = std::max(1u, st.connCap / (D + 1));
        for (uint32_t first = 0; first < items; first += perPass) {
            cudaMemsetAsync(st.counters + D + 2, 0, 3 * sizeof(uint32_t), stream);
            mark(SLRGPU_KERNEL_SHADE);
            if (vol)
                kBptConnect<true><<<g.connect[1], 256, 0, stream>>>(ds.sc, st, s.width, s.height, st.connQueue,
                                                                     st.counters + D + 1, first, perPass,
                                                                     st.counters + D + 2);
            else
                kBptConnect<false><<<g.connect[0], 256, 0, stream>>>(ds.sc, st, s.width, s.height, st.connQueue,
                                                                      st.counters + D + 1, first, perPass,
                                                                      st.counters + D + 2);
            markEnd();
            mark(SLRGPU_KERNEL_SHADOW);
            if (vol)
                kBptShadow<true><<<g.shadow[1], 256, 0, stream>>>(ds.sc, st, st.counters + D + 2,
                                                                   st.counters + D + 3);
            else
                kBptShadow<false><<<g.shadow[0], 256, 0, stream>>>(ds.sc, st, st.counters + D + 2,
                                                                    st.counters + D + 3);
            markEnd();
            nl += 2;
            if (vol) {
                mark(SLRGPU_KERNEL_SHADOW);
                kVbptMedium<<<g.medium, 256, 0, stream>>>(ds.sc, st, st.counters + D + 3, st.counters + D + 4);
                markEnd();
                ++nl;
            }
        }
        mark(SLRGPU_KERNEL_ACCUMULATE);
        kBptAccumulate<<<g.accumulate, 256, 0, stream>>>(st, wv, filmSum, filmComp);
        markEnd();
        ++nl;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        setError(std::string("bidirectional kernels: ") + cudaGetErrorString(e));
        return SLRGPU_ERR_CUDA;
    }
    if (launches) *launches += nl;
    if (stats) {
        unsigned long long h[4] = {0, 0, 0, 0};
        if (cudaMemcpyAsync(h, st.stats, sizeof(h), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess) {
            setError("bidirectional statistics readback failed");
            return SLRGPU_ERR_CUDA;
        }
        stats->extension_rays = h[0];
        stats->shadow_rays = h[1];
        stats->dropped_samples = h[2];
        for (const Mark &m : marks) {
            float kms = 0;
            cudaEventElapsedTime(&kms, (*eventPool)[m.ev], (*eventPool)[m.ev + 1]);
            stats->kernel_ms[m.cls] += kms;
            stats->kernel_count[m.cls] += 1;
        }
    }
    return SLRGPU_OK;
}

}  // namespace slrgpu
