// Closest-hit and any-hit traversal of the 4-wide BVH.
//
// By default the box and triangle tests repeat the reference's arithmetic
// exactly (no fused multiply-add): the slab test of BoundingBox3D::intersect
// (libSLR/BasicTypes/BoundingBox3D.h:100-116) on the SBVH's own boxes, and
// the Moller-Trumbore test of TriangleSurfaceShape::intersect
// (libSLR/SurfaceShape/TriangleSurfaceShape.cpp:205-257), including its
// inclusive [tmin, tmax] acceptance.  The wide nodes only skip the SBVH's
// intermediate boxes, which contain their children's boxes, so every
// triangle the reference would test is still tested.  With
// DevScene::watertight the triangle test is the watertight one below.
#pragma once
#include "device_common.cuh"

namespace slrgpu {

struct Hit {
    float t, b1, b2;
    uint32_t prim;
};

constexpr uint32_t kNoHit = 0xffffffffu;
constexpr int kTraceStack = 96;

// Moller-Trumbore; returns true and t/b1/b2 when the triangle is hit within [tmin, tmax].
__device__ __forceinline__ bool mtIntersect(const TriFrag &f, V3 org, V3 dir, float tmin, float tmax,
                                            float* tOut, float* b1Out, float* b2Out) {
    V3 e1 = V3{f.e1x, f.e1y, f.e1z};
    V3 e2 = V3{f.e2x, f.e2y, f.e2z};
    V3 p = rn_cross(dir, e2);
    float det = rn_dot(e1, p);
    if (det == 0.0f) return false;
    float invDet = __fdiv_rn(1.0f, det);
    V3 d = rn_sub(org, V3{f.v0x, f.v0y, f.v0z});
    float b1 = __fmul_rn(rn_dot(d, p), invDet);
    if (b1 < 0.0f || b1 > 1.0f) return false;
    V3 q = rn_cross(d, e1);
    float b2 = __fmul_rn(rn_dot(dir, q), invDet);
    if (b2 < 0.0f || __fadd_rn(b1, b2) > 1.0f) return false;
    float tt = __fmul_rn(rn_dot(e2, q), invDet);
    if (tt < tmin || tt > tmax) return false;
    *tOut = tt;
    *b1Out = b1;
    *b2Out = b2;
    return true;
}

// Watertight ray-triangle test (Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2013): vertices translated to the ray
// origin and sheared so the ray runs along +z; the 2-D edge functions are
// exact in sign for edges shared by two triangles (recomputed in double when
// one is zero), so a ray never slips between adjacent triangles.  Uses the
// vertices as given (not v0 + edge).  b1, b2 are the weights of v1 and v2, t
// is accepted in [tmin, tmax] as the reference's test does.
struct WtRay {
    int kx, ky, kz;
    float sx, sy, sz;
    V3 org;
};

__device__ __forceinline__ WtRay wtSetup(V3 org, V3 dir) {
    const float d[3] = {dir.x, dir.y, dir.z};
    const float ax = fabsf(dir.x), ay = fabsf(dir.y), az = fabsf(dir.z);
    int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dz = kz == 0 ? d[0] : (kz == 1 ? d[1] : d[2]);
    if (dz < 0.0f) { int tmp = kx; kx = ky; ky = tmp; }
    const float dx = kx == 0 ? d[0] : (kx == 1 ? d[1] : d[2]);
    const float dy = ky == 0 ? d[0] : (ky == 1 ? d[1] : d[2]);
    WtRay r;
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = dx / dz;
    r.sy = dy / dz;
    r.sz = 1.0f / dz;
    r.org = org;
    return r;
}

__device__ __forceinline__ float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ bool wtIntersect(const float4* __restrict__ wv, uint32_t i, const WtRay &r, float tmin,
                                            float tmax, float* tOut, float* b1Out, float* b2Out, uint32_t* prim) {
    const float4 p0 = __ldg(wv + 3 * (size_t)i), p1 = __ldg(wv + 3 * (size_t)i + 1), p2 = __ldg(wv + 3 * (size_t)i + 2);
    const V3 A = V3{p0.x, p0.y, p0.z} - r.org, B = V3{p1.x, p1.y, p1.z} - r.org, C = V3{p2.x, p2.y, p2.z} - r.org;
    const float Az = comp(A, r.kz), Bz = comp(B, r.kz), Cz = comp(C, r.kz);
    const float Ax = comp(A, r.kx) - r.sx * Az, Ay = comp(A, r.ky) - r.sy * Az;
    const float Bx = comp(B, r.kx) - r.sx * Bz, By = comp(B, r.ky) - r.sy * Bz;
    const float Cx = comp(C, r.kx) - r.sx * Cz, Cy = comp(C, r.ky) - r.sy * Cz;
    // Each product rounded on its own (no fused multiply-add): the edge
    // function of an edge shared by two triangles must come out exactly
    // negated in the neighbour, which a contraction would break.
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)__dsub_rn(__dmul_rn(Cx, By), __dmul_rn(Cy, Bx));
        V = (float)__dsub_rn(__dmul_rn(Ax, Cy), __dmul_rn(Ay, Cx));
        W = (float)__dsub_rn(__dmul_rn(Bx, Ay), __dmul_rn(By, Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float T = U * (r.sz * Az) + V * (r.sz * Bz) + W * (r.sz * Cz);
    const float inv = 1.0f / det;
    const float t = T * inv;
    if (!(t >= tmin && t <= tmax)) return false;
    *tOut = t;
    *b1Out = V * inv;
    *b2Out = W * inv;
    *prim = __float_as_uint(p0.w);
    return true;
}

// Slab test; returns the entry distance (dist0) or +inf when rejected.
// `robust` widens each slab's exit distance by 1 + 2 gamma_3 (Ize, "Robust
// BVH Ray Traversal", JCGT 2013) so that rounding cannot reject a box the
// ray only grazes at a face, edge or corner; the watertight triangle test
// needs it, the reference's arithmetic does not have it.
template <bool ROBUST>
__device__ __forceinline__ float slabTest(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                          V3 org, V3 inv, float tmin, float tmax) {
    float d0 = tmin, d1 = tmax;
    float tn = __fmul_rn(__fsub_rn(lox, org.x), inv.x), tf = __fmul_rn(__fsub_rn(hix, org.x), inv.x);
    if (tn > tf) { float s = tn; tn = tf; tf = s; }
    if (ROBUST) tf = __fmul_rn(tf, 1.0000008f);
    d0 = tn > d0 ? tn : d0;
    d1 = tf < d1 ? tf : d1;
    tn = __fmul_rn(__fsub_rn(loy, org.y), inv.y); tf = __fmul_rn(__fsub_rn(hiy, org.y), inv.y);
    if (tn > tf) { float s = tn; tn = tf; tf = s; }
    if (ROBUST) tf = __fmul_rn(tf, 1.0000008f);
    d0 = tn > d0 ? tn : d0;
    d1 = tf < d1 ? tf : d1;
    tn = __fmul_rn(__fsub_rn(loz, org.z), inv.z); tf = __fmul_rn(__fsub_rn(hiz, org.z), inv.z);
    if (tn > tf) { float s = tn; tn = tf; tf = s; }
    if (ROBUST) tf = __fmul_rn(tf, 1.0000008f);
    d0 = tn > d0 ? tn : d0;
    d1 = tf < d1 ? tf : d1;
    return (d0 > d1) ? __int_as_float(0x7f800000) : d0;
}

// The same slab test as min/max operations, for rays whose inverse direction
// is finite in every axis: then no product is NaN, the compare-and-swap of
// each slab's two distances is their min and max, and the running entry and
// exit distances are a max and a min (the order of the axes does not
// change a max or a min), so every distance and decision equals slabTest's
// (up to the sign of a zero, which no comparison sees).  A zero direction
// component makes (plane - origin) * inv NaN on a plane through the origin,
// where slabTest's comparisons decide differently from min/max; such rays
// take slabTest.
template <bool ROBUST>
__device__ __forceinline__ float slabTestMinMax(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                                V3 org, V3 inv, float tmin, float tmax) {
    const float ax = __fmul_rn(__fsub_rn(lox, org.x), inv.x), bx = __fmul_rn(__fsub_rn(hix, org.x), inv.x);
    const float ay = __fmul_rn(__fsub_rn(loy, org.y), inv.y), by = __fmul_rn(__fsub_rn(hiy, org.y), inv.y);
    const float az = __fmul_rn(__fsub_rn(loz, org.z), inv.z), bz = __fmul_rn(__fsub_rn(hiz, org.z), inv.z);
    float fx = fmaxf(ax, bx), fy = fmaxf(ay, by), fz = fmaxf(az, bz);
    if (ROBUST) {
        fx = __fmul_rn(fx, 1.0000008f);
        fy = __fmul_rn(fy, 1.0000008f);
        fz = __fmul_rn(fz, 1.0000008f);
    }
    const float d0 = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), tmin));
    const float d1 = fminf(fminf(fx, fy), fminf(fz, tmax));
    return (d0 > d1) ? __int_as_float(0x7f800000) : d0;
}

#ifndef SLRGPU_MINMAX_SLABS
#define SLRGPU_MINMAX_SLABS 1
#endif

struct StackEntry {
    uint32_t node;
    float tnear;
};

// Box test of the 4 children of a node; returns the hit mask and entry distances.
template <bool ROBUST>
__device__ __forceinline__ uint32_t testChildren(const BvhNode* __restrict__ nodes, uint32_t ni, V3 org, V3 inv,
                                                 float tmin, float tmax, float tn[kBvhWidth],
                                                 uint32_t ch[kBvhWidth], bool minmax = false) {
    // 128-bit loads: Q float4 per coordinate array, then the child words
    constexpr int Q = kBvhWidth / 4;
    const float4* np = reinterpret_cast<const float4*>(nodes + ni);
    uint32_t mask = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float4 lx = __ldg(np + 0 * Q + q), hx = __ldg(np + 1 * Q + q), ly = __ldg(np + 2 * Q + q);
        const float4 hy = __ldg(np + 3 * Q + q), lz = __ldg(np + 4 * Q + q), hz = __ldg(np + 5 * Q + q);
        const uint4 c = __ldg(reinterpret_cast<const uint4*>(np + 6 * Q) + q);
        const float lxa[4] = {lx.x, lx.y, lx.z, lx.w}, hxa[4] = {hx.x, hx.y, hx.z, hx.w};
        const float lya[4] = {ly.x, ly.y, ly.z, ly.w}, hya[4] = {hy.x, hy.y, hy.z, hy.w};
        const float lza[4] = {lz.x, lz.y, lz.z, lz.w}, hza[4] = {hz.x, hz.y, hz.z, hz.w};
        const uint32_t ca[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = 4 * q + k;
            ch[i] = ca[k];
            tn[i] = (SLRGPU_MINMAX_SLABS && minmax)
                        ? slabTestMinMax<ROBUST>(lxa[k], hxa[k], lya[k], hya[k], lza[k], hza[k], org, inv, tmin, tmax)
                        : slabTest<ROBUST>(lxa[k], hxa[k], lya[k], hya[k], lza[k], hza[k], org, inv, tmin, tmax);
            if (ch[i] != kChildEmpty && tn[i] != __int_as_float(0x7f800000)) mask |= 1u << i;
        }
    }
    return mask;
}

// Orders the hit children of a node near to far (ties in child order) with a
// sorting network on registers (5 comparators for 4 children, Batcher's 19
// for 8); missed children sort last at +inf.  Pushes all but the nearest,
// far to near, and returns the nearest.
__device__ __forceinline__ uint32_t orderChildren(uint32_t mask, const float tn[kBvhWidth],
                                                  const uint32_t ch[kBvhWidth], StackEntry* stack, int &sp,
                                                  bool &ok) {
    float t[kBvhWidth];
    uint32_t c[kBvhWidth], k[kBvhWidth];
#pragma unroll
    for (int i = 0; i < kBvhWidth; ++i) {
        t[i] = ((mask >> i) & 1u) ? tn[i] : __int_as_float(0x7f800000);
        c[i] = ch[i];
        k[i] = (uint32_t)i;
    }
#define SLRGPU_CSWAP(a, b)                                                           \
    if (t[b] < t[a] || (t[b] == t[a] && k[b] < k[a])) {                              \
        float tt = t[a]; t[a] = t[b]; t[b] = tt;                                     \
        uint32_t cc = c[a]; c[a] = c[b]; c[b] = cc;                                  \
        uint32_t kk = k[a]; k[a] = k[b]; k[b] = kk;                                  \
    }
    if constexpr (kBvhWidth == 4) {
        SLRGPU_CSWAP(0, 1) SLRGPU_CSWAP(2, 3) SLRGPU_CSWAP(0, 2) SLRGPU_CSWAP(1, 3) SLRGPU_CSWAP(1, 2)
    } else {
        SLRGPU_CSWAP(0, 1) SLRGPU_CSWAP(2, 3) SLRGPU_CSWAP(4, 5) SLRGPU_CSWAP(6, 7)
        SLRGPU_CSWAP(0, 2) SLRGPU_CSWAP(1, 3) SLRGPU_CSWAP(4, 6) SLRGPU_CSWAP(5, 7)
        SLRGPU_CSWAP(1, 2) SLRGPU_CSWAP(5, 6)
        SLRGPU_CSWAP(0, 4) SLRGPU_CSWAP(1, 5) SLRGPU_CSWAP(2, 6) SLRGPU_CSWAP(3, 7)
        SLRGPU_CSWAP(2, 4) SLRGPU_CSWAP(3, 5)
        SLRGPU_CSWAP(1, 2) SLRGPU_CSWAP(3, 4) SLRGPU_CSWAP(5, 6)
    }
#undef SLRGPU_CSWAP
    const int n = __popc(mask);
#pragma unroll
    for (int i = kBvhWidth - 1; i >= 1; --i) {
        if (i < n) {
            if (sp < kTraceStack) stack[sp++] = StackEntry{c[i], t[i]};
            else ok = false;
        }
    }
    return c[0];
}

__device__ __forceinline__ TriFrag loadFrag(const TriFrag* __restrict__ frags, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(frags + i);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    TriFrag f;
    f.v0x = a.x; f.v0y = a.y; f.v0z = a.z; f.prim = __float_as_uint(a.w);
    f.e1x = b.x; f.e1y = b.y; f.e1z = b.z; f.pad0 = 0;
    f.e2x = c.x; f.e2y = c.y; f.e2z = c.z; f.pad1 = 0;
    return f;
}

// A closest-hit walk over [tmin, tmax] that can stop after a number of node
// or leaf visits and resume later: the wave kernels give a lane a new ray as
// soon as its walk ends, instead of leaving it idle until the longest walk of
// its warp is done.  Nodes and triangles are visited in the order of an
// uninterrupted walk, so the hit is the same.  WT: the watertight triangle
// test with conservative box tests.
template <bool WT>
struct ClosestWalk {
    V3 org, dir, inv;
    WtRay wr;
    float tmin, tmax;
    Hit hit;
    uint32_t cur;
    int sp;
    bool ok;   // false after a stack overflow (the hit found so far is kept)
    bool minmax;   // finite inverse direction: slabTestMinMax

    // Returns true when the walk has already ended (an empty scene).
    __device__ __forceinline__ bool begin(const DevScene &sc, V3 o, V3 d, float t0, float t1) {
        hit.prim = kNoHit;
        hit.t = __int_as_float(0x7f800000);
        hit.b1 = hit.b2 = 0.0f;
        org = o;
        dir = d;
        inv = V3{__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z)};
        minmax = isfinite(inv.x) && isfinite(inv.y) && isfinite(inv.z);
        if (WT) wr = wtSetup(o, d);
        tmin = t0;
        tmax = t1;
        cur = 0;
        sp = 0;
        ok = true;
        return sc.numPrims == 0;
    }

    // At most `visits` node or leaf visits; returns true when the walk has ended.
    __device__ __forceinline__ bool advance(const DevScene &sc, StackEntry* stack, int visits) {
        for (int v = 0; v < visits; ++v) {
            if (!(cur & kLeafBit)) {
                float tn[kBvhWidth];
                uint32_t ch[kBvhWidth];
                const uint32_t mask = testChildren<WT>(sc.nodes, cur, org, inv, tmin, tmax, tn, ch, minmax);
                if (mask != 0) {
                    cur = orderChildren(mask, tn, ch, stack, sp, ok);
                    continue;
                }
            } else {
                const uint32_t first = cur & kLeafFirstMask;
                const uint32_t count = ((cur >> kLeafCountShift) & 0x1f) + 1;
                for (uint32_t i = 0; i < count; ++i) {
                    float t, b1, b2;
                    uint32_t prim;
                    bool h;
                    if (WT) {
                        h = wtIntersect(sc.wtVerts, first + i, wr, tmin, tmax, &t, &b1, &b2, &prim);
                    } else {
                        TriFrag f = loadFrag(sc.frags, first + i);
                        h = mtIntersect(f, org, dir, tmin, tmax, &t, &b1, &b2);
                        prim = f.prim;
                    }
                    if (h) {
                        tmax = t;
                        hit.t = t;
                        hit.b1 = b1;
                        hit.b2 = b2;
                        hit.prim = prim;
                    }
                }
            }
            // the nearest pushed node the ray can still reach
            for (;;) {
                if (sp == 0) return true;
                const StackEntry e = stack[--sp];
                if (e.tnear <= tmax) {
                    cur = e.node;
                    break;
                }
            }
        }
        return false;
    }
};

// Closest hit over [tmin, tmax] in one go.  Returns false on stack overflow
// (the hit found so far is still reported).
template <bool WT>
__device__ __forceinline__ bool traceClosestT(const DevScene &sc, V3 org, V3 dir, float tmin, float tmax, Hit* hit) {
    StackEntry stack[kTraceStack];
    ClosestWalk<WT> w;
    if (!w.begin(sc, org, dir, tmin, tmax))
        while (!w.advance(sc, stack, 1 << 30)) {
        }
    *hit = w.hit;
    return w.ok;
}

__device__ __forceinline__ bool traceClosest(const DevScene &sc, V3 org, V3 dir, float tmin, float tmax, Hit* hit) {
    return sc.watertight ? traceClosestT<true>(sc, org, dir, tmin, tmax, hit)
                         : traceClosestT<false>(sc, org, dir, tmin, tmax, hit);
}

// An any-hit walk over [tmin, tmax] that can stop and resume like
// ClosestWalk; `occluded` holds the answer once the walk has ended.
template <bool WT>
struct AnyWalk {
    V3 org, dir, inv;
    WtRay wr;
    float tmin, tmax;
    uint32_t cur;
    int sp;
    bool occluded;
    bool minmax;

    __device__ __forceinline__ bool begin(const DevScene &sc, V3 o, V3 d, float t0, float t1) {
        org = o;
        dir = d;
        inv = V3{__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z)};
        minmax = isfinite(inv.x) && isfinite(inv.y) && isfinite(inv.z);
        if (WT) wr = wtSetup(o, d);
        tmin = t0;
        tmax = t1;
        cur = 0;
        sp = 0;
        occluded = false;
        return sc.numPrims == 0;
    }

    __device__ __forceinline__ bool advance(const DevScene &sc, uint32_t* stack, int visits) {
        for (int v = 0; v < visits; ++v) {
            if (!(cur & kLeafBit)) {
                float tn[kBvhWidth];
                uint32_t ch[kBvhWidth];
                const uint32_t mask = testChildren<WT>(sc.nodes, cur, org, inv, tmin, tmax, tn, ch, minmax);
                bool have = false;
                uint32_t next = 0;
#pragma unroll
                for (int k = 0; k < kBvhWidth; ++k) {
                    if (mask & (1u << k)) {
                        if (!have) { next = ch[k]; have = true; }
                        else if (sp < kTraceStack) stack[sp++] = ch[k];
                    }
                }
                if (have) {
                    cur = next;
                    continue;
                }
            } else {
                const uint32_t first = cur & kLeafFirstMask;
                const uint32_t count = ((cur >> kLeafCountShift) & 0x1f) + 1;
                for (uint32_t i = 0; i < count; ++i) {
                    float t, b1, b2;
                    bool h;
                    if (WT) {
                        uint32_t prim;
                        h = wtIntersect(sc.wtVerts, first + i, wr, tmin, tmax, &t, &b1, &b2, &prim);
                    } else {
                        TriFrag f = loadFrag(sc.frags, first + i);
                        h = mtIntersect(f, org, dir, tmin, tmax, &t, &b1, &b2);
                    }
                    if (h) {
                        occluded = true;
                        return true;
                    }
                }
            }
            if (sp == 0) return true;
            cur = stack[--sp];
        }
        return false;
    }
};

// Any hit over [tmin, tmax]: true when the segment is occluded.
template <bool WT>
__device__ __forceinline__ bool traceAnyT(const DevScene &sc, V3 org, V3 dir, float tmin, float tmax) {
    uint32_t stack[kTraceStack];
    AnyWalk<WT> w;
    if (w.begin(sc, org, dir, tmin, tmax)) return false;
    while (!w.advance(sc, stack, 1 << 30)) {
    }
    return w.occluded;
}

__device__ __forceinline__ bool traceAny(const DevScene &sc, V3 org, V3 dir, float tmin, float tmax) {
    return sc.watertight ? traceAnyT<true>(sc, org, dir, tmin, tmax) : traceAnyT<false>(sc, org, dir, tmin, tmax);
}

}  // namespace slrgpu
