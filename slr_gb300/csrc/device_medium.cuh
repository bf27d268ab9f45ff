// Heterogeneous medium on the device: density-grid lookups, the super-voxel
// 3-D DDA with a cubic majorant per cell and regula-falsi free-path solve,
// delta tracking for scattering and ratio tracking for transmittance.  The
// arithmetic follows DensityGridMediumDistribution
// (libSLR/MediumDistribution/DensityGridMediumDistribution.cpp:16-744) and the
// single-medium case of MediumObjectAggregate::interact / evaluateTransmittance
// (libSLR/Core/medium_object.cpp:287-402).
#pragma once
#include "device_common.cuh"

namespace slrgpu {

__device__ __forceinline__ bool outsideUnit(V3 p) {
    return p.x < 0 || p.y < 0 || p.z < 0 || p.x > 1 || p.y > 1 || p.z > 1;
}

__device__ __forceinline__ float trilinearGrid(const float* __restrict__ g, uint32_t nx, uint32_t ny, uint32_t nz, V3 p) {
    uint32_t lx = min((uint32_t)(p.x * (nx - 1)), nx - 1), ux = min(lx + 1, nx - 1);
    uint32_t ly = min((uint32_t)(p.y * (ny - 1)), ny - 1), uy = min(ly + 1, ny - 1);
    uint32_t lz = min((uint32_t)(p.z * (nz - 1)), nz - 1), uz = min(lz + 1, nz - 1);
    float wux = p.x * (nx - 1) - lx, wlx = 1 - wux;
    float wuy = p.y * (ny - 1) - ly, wly = 1 - wuy;
    float wuz = p.z * (nz - 1) - lz, wlz = 1 - wuz;
    const size_t sl = (size_t)nx * ny;
    const float* zl = g + sl * lz;
    const float* zu = g + sl * uz;
    return __ldg(zl + nx * ly + lx) * wlz * wly * wlx + __ldg(zl + nx * ly + ux) * wlz * wly * wux +
           __ldg(zl + nx * uy + lx) * wlz * wuy * wlx + __ldg(zl + nx * uy + ux) * wlz * wuy * wux +
           __ldg(zu + nx * ly + lx) * wuz * wly * wlx + __ldg(zu + nx * ly + ux) * wuz * wly * wux +
           __ldg(zu + nx * uy + lx) * wuz * wuy * wlx + __ldg(zu + nx * uy + ux) * wuz * wuy * wux;
}

// calcDensity (DensityGridMediumDistribution.cpp:369-395).
__device__ __forceinline__ float mediumDensity(const DevMedium &m, V3 param) {
    if (outsideUnit(param)) return 0.0f;
    return trilinearGrid(m.density, m.nx, m.ny, m.nz, param);
}

// calcDensityInSuperVoxels (DensityGridMediumDistribution.cpp:16-43).
__device__ __forceinline__ float mediumCoarseDensity(const DevMedium &m, V3 param) {
    if (outsideUnit(param)) return 0.0f;
    float d = trilinearGrid(m.superVoxels, m.svx, m.svy, m.svz, param);
    uint32_t lx = min((uint32_t)(param.x * (m.svx - 1)), m.svx - 1);
    uint32_t ly = min((uint32_t)(param.y * (m.svy - 1)), m.svy - 1);
    uint32_t lz = min((uint32_t)(param.z * (m.svz - 1)), m.svz - 1);
    uint32_t cell = (m.svx - 1) * (m.svy - 1) * min(lz, m.svz - 2) + (m.svx - 1) * min(ly, m.svy - 2) + min(lx, m.svx - 2);
    return d + m.maxDiff[cell];
}

// Position in the medium's unit cube.  The divisions of the reference become
// multiplications by reciprocals computed once on the host (results differ
// in the last bit; the walks are issue-bound and an IEEE division is a
// sequence of instructions).
__device__ __forceinline__ V3 mediumLocal(const DevMedium &m, V3 p) {
    return V3{(p.x - m.bmin[0]) * m.invExtent[0], (p.y - m.bmin[1]) * m.invExtent[1],
              (p.z - m.bmin[2]) * m.invExtent[2]};
}

constexpr float kThird = 1.0f / 3.0f;

__device__ __forceinline__ bool mediumContains(const DevMedium &m, V3 p) {
    return p.x >= m.bmin[0] && p.x < m.bmax[0] && p.y >= m.bmin[1] && p.y < m.bmax[1] && p.z >= m.bmin[2] &&
           p.z < m.bmax[2];
}

// BoundingBox3D::intersectBoundary (BoundingBox3D.h:119-144).
__device__ __forceinline__ bool mediumIntersectBoundary(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax,
                                                       float* dist, bool* enter) {
    float d0 = -__int_as_float(0x7f800000), d1 = __int_as_float(0x7f800000);
    const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float inv = 1.0f / d[i];
        float tn = (m.bmin[i] - o[i]) * inv, tf = (m.bmax[i] - o[i]) * inv;
        if (tn > tf) { float s = tn; tn = tf; tf = s; }
        d0 = tn > d0 ? tn : d0;
        d1 = tf < d1 ? tf : d1;
        if (d0 > d1) return false;
    }
    if (mediumContains(m, org + dmin * dir)) {
        *dist = d1;
        *enter = false;
        return d1 >= dmin && d1 < dmax;
    }
    *dist = d0;
    *enter = true;
    return d0 >= dmin && d0 < dmax;
}

// ---- super-voxel traversal -------------------------------------------------
struct SvWalk {
    int sv[3];
    float maxt[3];
};

struct SvSetup {
    int step[3];
    int outside[3];
    float invD[3];      // 1 / direction: the plane distances are multiplications
    SvWalk init;
};

__device__ __forceinline__ void svSetup(const DevMedium &m, V3 org, V3 dir, float dmin, SvSetup &s) {
    V3 p = mediumLocal(m, org + dmin * dir);
    p = V3{fminf(fmaxf(p.x, 0.0f), 1.0f), fminf(fmaxf(p.y, 0.0f), 1.0f), fminf(fmaxf(p.z, 0.0f), 1.0f)};
    const uint32_t n[3] = {m.svx, m.svy, m.svz};
    const float lp[3] = {p.x, p.y, p.z}, o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        s.init.sv[i] = min((int)(lp[i] * (n[i] - 1)), (int)n[i] - 2);
        s.invD[i] = 1.0f / d[i];
        if (d[i] > 0) {
            s.step[i] = 1;
            s.outside[i] = (int)n[i] - 1;
            float plane = m.bmin[i] + m.svWidth[i] * (s.init.sv[i] + 1);
            s.init.maxt[i] = (plane - o[i]) * s.invD[i];
        } else {
            s.step[i] = -1;
            s.outside[i] = -1;
            float plane = m.bmin[i] + m.svWidth[i] * (s.init.sv[i] + 0);
            s.init.maxt[i] = (plane - o[i]) * s.invD[i];
        }
    }
}

// Cubic in the segment parameter of the trilinear super-voxel majorant
// between entry and exit (plus the cell's maximum difference).
__device__ __forceinline__ void svPolyCoeffs(const DevMedium &m, V3 entry, V3 exit, const int cell[3], float c[4]) {
    const uint32_t sx = m.svx, sxy = m.svx * m.svy;
    const float* s = m.superVoxels;
    const int i0 = sxy * cell[2] + sx * cell[1] + cell[0];
    float d000 = __ldg(s + i0), d100 = __ldg(s + i0 + 1), d010 = __ldg(s + i0 + sx), d110 = __ldg(s + i0 + sx + 1);
    float d001 = __ldg(s + i0 + sxy), d101 = __ldg(s + i0 + sxy + 1), d011 = __ldg(s + i0 + sxy + sx),
          d111 = __ldg(s + i0 + sxy + sx + 1);
    V3 base = V3{m.bmin[0] + cell[0] * m.svWidth[0], m.bmin[1] + cell[1] * m.svWidth[1],
                 m.bmin[2] + cell[2] * m.svWidth[2]};
    V3 ep = V3{(entry.x - base.x) * m.invSvWidth[0], (entry.y - base.y) * m.invSvWidth[1],
               (entry.z - base.z) * m.invSvWidth[2]};
    V3 op = V3{(exit.x - base.x) * m.invSvWidth[0], (exit.y - base.y) * m.invSvWidth[1],
               (exit.z - base.z) * m.invSvWidth[2]};
    V3 dl = op - ep;
    float dxyz = d111 - d011 - d101 - d110 + d001 + d010 + d100 - d000;
    float dxy = d000 - d100 - d010 + d110;
    float dxz = d000 - d100 - d001 + d101;
    float dyz = d000 - d010 - d001 + d011;
    float dx = d100 - d000, dy = d010 - d000, dz = d001 - d000;
    c[3] = dxyz * dl.x * dl.y * dl.z;
    c[2] = ((ep.z * dl.x * dl.y + ep.y * dl.x * dl.z + ep.x * dl.y * dl.z) * dxyz + dxy * dl.x * dl.y +
            dxz * dl.x * dl.z + dyz * dl.y * dl.z);
    c[1] = ((ep.y * ep.z * dl.x + ep.x * ep.z * dl.y + ep.x * ep.y * dl.z) * dxyz + dx * dl.x + dy * dl.y +
            dz * dl.z + (ep.y * dl.x + ep.x * dl.y) * dxy + (ep.z * dl.x + ep.x * dl.z) * dxz +
            (ep.z * dl.y + ep.y * dl.z) * dyz);
    c[0] = (ep.x * ep.y * ep.z * dxyz + ep.x * ep.y * dxy + ep.x * ep.z * dxz + ep.y * ep.z * dyz + ep.x * dx +
            ep.y * dy + ep.z * dz + d000);
    c[0] += __ldg(m.maxDiff + (m.svx - 1) * (m.svy - 1) * cell[2] + (m.svx - 1) * cell[1] + cell[0]);
}

// traverseSuperVoxels (DensityGridMediumDistribution.cpp:208-367): samples a
// tentative collision of the majorant process along [dmin, dmax).  Returns
// false (and *dist = dmax) when the walk leaves the segment.
constexpr int kMaxSvSteps = 4096;

static __device__ __noinline__ bool svTraverse(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax, float u,
                                        float sigma, const SvSetup &s, SvWalk &w, float* dist, float* majorant) {
    float sampledOD = -logf(1 - u);
    if (sampledOD == 0.0f) {
        V3 q = org + (*dist) * dir;
        *majorant = sigma * mediumCoarseDensity(m, mediumLocal(m, q));
        return true;
    }
    float entryDist = 0.0f, exitDist = dmin;
    V3 entryP, exitP = org + exitDist * dir;
    float entryOD = 0.0f, exitOD = 0.0f;
    float c[4];
    int steps = 0;
    for (;;) {
        entryP = exitP;
        entryDist = exitDist;
        entryOD = exitOD;
        const uint32_t cond = (uint32_t)(w.maxt[0] < w.maxt[1]) | ((uint32_t)(w.maxt[0] < w.maxt[2]) << 1) |
                              ((uint32_t)(w.maxt[1] < w.maxt[2]) << 2);
        // axisMap[cond] = {2, 2, 2, 0, 1, 2, 1, 0}, one nibble per entry
        const int axis = (0x01210222u >> (4 * cond)) & 0xf;
        exitDist = w.maxt[axis];
        exitP = org + exitDist * dir;
        svPolyCoeffs(m, entryP, exitP, w.sv, c);
        exitOD += (exitDist - entryDist) * sigma * (c[0] + c[1] * 0.5f + c[2] * kThird + c[3] * 0.25f);
        if (exitOD >= sampledOD) break;
        w.sv[axis] += s.step[axis];
        if (w.sv[axis] == s.outside[axis] || exitDist >= dmax || ++steps > kMaxSvSteps) {
            *dist = dmax;
            *majorant = __int_as_float(0x7fc00000);
            return false;
        }
        float plane = m.bmin[axis] + m.svWidth[axis] * (w.sv[axis] + (s.step[axis] == 1 ? 1 : 0));
        const float oa = axis == 0 ? org.x : (axis == 1 ? org.y : org.z);
        w.maxt[axis] = (plane - oa) * s.invD[axis];
    }
    // Regula falsi on the integrated majorant.
    float pLow = 0.0f, pHigh = 1.0f, odLow = entryOD, odHigh = exitOD;
    float prev = -__int_as_float(0x7f800000), cur = pHigh;
    int iters = 0;
    while (fabsf(cur - prev) >= 1e-3f * fabsf(cur) && iters < 100) {
        prev = cur;
        cur = pLow + (pHigh - pLow) * __fdividef(sampledOD - odLow, odHigh - odLow);
        float temp = sigma * (c[0] * cur + c[1] * cur * cur * 0.5f + c[2] * cur * cur * cur * kThird +
                              c[3] * cur * cur * cur * cur * 0.25f);
        float od = entryOD + (exitDist - entryDist) * temp;
        ++iters;
        if (od < sampledOD) { pLow = cur; odLow = od; }
        else if (od > sampledOD) { pHigh = cur; odHigh = od; }
        else break;
    }
    *dist = entryDist + (exitDist - entryDist) * cur;
    if (*dist >= dmax) {
        *dist = dmax;
        *majorant = __int_as_float(0x7fc00000);
        return false;
    }
    *majorant = sigma * (c[0] + c[1] * cur + c[2] * cur * cur + c[3] * cur * cur * cur);
    return true;
}

// DensityGridMediumDistribution::interact (:402-575): delta tracking at the
// selected wavelength; spectral throughput for the others by the ratio
// estimator.  Returns true on a real collision at *tHit (param = normalised
// position).  thr receives the medium throughput (already divided by the
// extinction coefficient at the collision).
template <class R>
__device__ __noinline__ bool mediumInteractSegment(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax,
                                                   const Spec &sigmaE, int sel, bool wlSelected, R &rng,
                                                   float* tHit, V3* param, Spec &thr) {
    SvSetup s;
    svSetup(m, org, dir, dmin, s);
    SvWalk w = s.init;
    bool hit = false;
    float extAt = 0.0f;
    float sd = dmin;
    const float sigSel = specAt(sigmaE, sel);
    while (sd < dmax) {
        float maj;
        bool tent = svTraverse(m, org, dir, sd, dmax, rng.next(), sigSel, s, w, &sd, &maj);
        if (!tent) { hit = false; break; }
        V3 q = org + sd * dir;
        V3 pr = mediumLocal(m, q);
        float ext = sigSel * mediumDensity(m, pr);
        float prob = ext / maj;
        if (rng.next() < prob) {
            hit = true;
            *tHit = sd;
            *param = pr;
            extAt = ext;
            break;
        }
    }
    if (wlSelected) {
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) thr.v[k] = (k == sel) ? 1.0f : 0.0f;
    } else {
        const float hitDist = fminf(sd, dmax);
        sd = dmin;
        w = s.init;
        Spec mc = specConst(1.0f);
        // The walk state is shared across the wavelengths, so only the first
        // wavelength other than the selected one takes steps (the reference's
        // loop at DensityGridMediumDistribution.cpp:487-510 never resets it).
        for (int wl = 0; wl < kNumLambda; ++wl) {
            if (wl == sel) continue;
            const float sigWl = specAt(sigmaE, wl);
            while (sd < hitDist) {
                float maj;
                bool tent = svTraverse(m, org, dir, sd, hitDist, rng.next(), sigWl, s, w, &sd, &maj);
                if (tent) {
                    V3 q = org + sd * dir;
                    float dens = mediumDensity(m, mediumLocal(m, q));
                    float prob = (sigWl * dens - sigSel * dens) / maj;
                    if (maj != 0.0f) mc.v[wl] *= (1.0f - prob);
                }
            }
        }
        thr = mc;
    }
    if (hit) {
        float r = 1.0f / extAt;
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) thr.v[k] *= r;
    }
    return hit;
}

// Ratio-tracking estimate of one wavelength's transmittance over [dmin, dmax)
// inside the medium, with Russian roulette below 0.1
// (DensityGridMediumDistribution.cpp:618-651); s is the DDA set-up at dmin.
template <class R>
__device__ __forceinline__ float ratioTrackSegment(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax,
                                                   const SvSetup &s, float sig, R &rng) {
    float t = 1.0f;
    SvWalk w = s.init;
    float sd = dmin;
    while (sd < dmax) {
        float maj;
        bool tent = svTraverse(m, org, dir, sd, dmax, rng.next(), sig, s, w, &sd, &maj);
        if (tent) {
            float ext = sig * mediumDensity(m, mediumLocal(m, org + sd * dir));
            float prob = ext / maj;
            if (maj != 0.0f) t *= (1.0f - prob);
            if (t < 0.1f) {
                if (rng.next() < t) t = 1.0f;
                else return 0.0f;
            }
        }
    }
    return t;
}

// Spectral transmittance of one segment inside the medium
// (DensityGridMediumDistribution::evaluateTransmittance, :577-744): every
// wavelength, or only the selected one once a wavelength is selected.
template <class R>
__device__ __noinline__ void mediumTransmittanceSegment(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax,
                                                        const Spec &sigmaE, int sel, bool wlSelected, R &rng,
                                                        Spec &T) {
    SvSetup s;
    svSetup(m, org, dir, dmin, s);
    T = specConst(0.0f);
    for (int wl = 0; wl < kNumLambda; ++wl) {
        if (wlSelected && wl != sel) continue;
        const float t = ratioTrackSegment(m, org, dir, dmin, dmax, s, specAt(sigmaE, wl), rng);
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k)
            if (k == wl) T.v[k] = t;
    }
}

// MediumObjectAggregate::interact for one medium (medium_object.cpp:287-348):
// walks boundary crossings of the medium box within [dmin, dmax).
template <class R>
__device__ __forceinline__ bool mediumInteract(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax,
                                               const Spec &sigmaE, int sel, bool wlSelected, R &rng, float* tHit,
                                               V3* param, Spec &thr) {
    thr = specConst(1.0f);
    float rmin = dmin;
    bool inside = mediumContains(m, org + rmin * dir);
    for (int guard = 0; guard < 8; ++guard) {
        float dist;
        bool enter;
        bool nextInside = false;
        float distNext = __int_as_float(0x7f800000);
        if (mediumIntersectBoundary(m, org, dir, rmin, dmax, &dist, &enter) && dist < distNext) {
            distNext = dist;
            nextInside = enter;
        }
        if (inside && nextInside) inside = false;
        distNext = fminf(distNext, dmax);
        if (isinf(distNext)) return false;
        if (inside) {
            Spec t;
            bool hit = mediumInteractSegment(m, org, dir, rmin, distNext, sigmaE, sel, wlSelected, rng, tHit, param, t);
#pragma unroll
            for (int k = 0; k < kNumLambda; ++k) thr.v[k] *= t.v[k];
            if (hit) return true;
        }
        if (distNext == dmax) return false;
        rmin = distNext * (1.0f + kRayEpsilon);
        inside = nextInside;
    }
    return false;
}

// MediumObjectAggregate::evaluateTransmittance for one medium (:350-402).
template <class R>
__device__ __forceinline__ void mediumTransmittance(const DevMedium &m, V3 org, V3 dir, float dmin, float dmax,
                                                    const Spec &sigmaE, int sel, bool wlSelected, R &rng, Spec &T) {
    T = specConst(1.0f);
    float rmin = dmin;
    bool inside = mediumContains(m, org + rmin * dir);
    for (int guard = 0; guard < 8; ++guard) {
        float dist;
        bool enter;
        bool nextInside = false;
        float distNext = __int_as_float(0x7f800000);
        if (mediumIntersectBoundary(m, org, dir, rmin, dmax, &dist, &enter) && dist < distNext) {
            distNext = dist;
            nextInside = enter;
        }
        if (inside && nextInside) inside = false;
        distNext = fminf(distNext, dmax);
        if (isinf(distNext)) return;
        if (inside) {
            Spec t;
            mediumTransmittanceSegment(m, org, dir, rmin, distNext, sigmaE, sel, wlSelected, rng, t);
#pragma unroll
            for (int k = 0; k < kNumLambda; ++k) T.v[k] *= t.v[k];
        }
        if (distNext == dmax) return;
        rmin = distNext * (1.0f + kRayEpsilon);
        inside = nextInside;
    }
}

// One wavelength of mediumTransmittance as a resumable walk, for one lane per
// (ray, wavelength): the same boundary crossings and per-segment ratio
// tracking, with the state kept between two tentative collisions so that a
// lane whose walk has ended can start the next (ray, wavelength) while the
// other lanes of its warp go on.  `evaluate` false (a wavelength other than
// the selected one) gives 0 once the ray crosses the medium and 1 otherwise,
// as the spectral version does.
struct TrWalk {
    V3 org, dir;
    float dmax, sig;
    Rng rng;
    float T;            // product of the finished segments
    float t;            // the current segment's ratio-tracking estimate
    float rmin, segEnd, sd;
    int guard;
    bool inside, nextInside, evaluate;
    SvSetup s;
    SvWalk w;
};

// Runs the boundary loop until a segment inside the medium is ready to walk
// (true) or the estimate q.T is final (false).
__device__ __forceinline__ bool trAdvance(const DevMedium &m, TrWalk &q) {
    for (; q.guard < 8; ++q.guard) {
        float dist;
        bool enter;
        q.nextInside = false;
        float distNext = __int_as_float(0x7f800000);
        if (mediumIntersectBoundary(m, q.org, q.dir, q.rmin, q.dmax, &dist, &enter) && dist < distNext) {
            distNext = dist;
            q.nextInside = enter;
        }
        if (q.inside && q.nextInside) q.inside = false;
        distNext = fminf(distNext, q.dmax);
        if (isinf(distNext)) return false;
        q.segEnd = distNext;
        if (q.inside) {
            if (!q.evaluate) {
                q.T = 0.0f;
                return false;
            }
            svSetup(m, q.org, q.dir, q.rmin, q.s);
            q.w = q.s.init;
            q.t = 1.0f;
            q.sd = q.rmin;
            if (q.sd < q.segEnd) return true;
            q.T *= q.t;      // an empty segment estimates 1
        }
        if (q.segEnd == q.dmax) return false;
        q.rmin = q.segEnd * (1.0f + kRayEpsilon);
        q.inside = q.nextInside;
    }
    return false;
}

__device__ __forceinline__ bool trBegin(const DevMedium &m, TrWalk &q, V3 org, V3 dir, float dmin, float dmax,
                                        float sig, bool evaluate, Rng rng) {
    q.org = org;
    q.dir = dir;
    q.dmax = dmax;
    q.sig = sig;
    q.evaluate = evaluate;
    q.rng = rng;
    q.T = 1.0f;
    q.rmin = dmin;
    q.guard = 0;
    q.inside = mediumContains(m, org + dmin * dir);
    return trAdvance(m, q);
}

// One tentative collision of the current segment (ratioTrackSegment's loop
// body).  Returns true while the walk goes on; q.T is final otherwise.
__device__ __forceinline__ bool trStep(const DevMedium &m, TrWalk &q) {
    float maj;
    const bool tent = svTraverse(m, q.org, q.dir, q.sd, q.segEnd, q.rng.next(), q.sig, q.s, q.w, &q.sd, &maj);
    bool segDone = !(q.sd < q.segEnd);
    if (tent) {
        float ext = q.sig * mediumDensity(m, mediumLocal(m, q.org + q.sd * q.dir));
        float prob = ext / maj;
        if (maj != 0.0f) q.t *= (1.0f - prob);
        if (q.t < 0.1f) {
            if (q.rng.next() < q.t) {
                q.t = 1.0f;
            } else {
                q.t = 0.0f;
                segDone = true;
            }
        }
    }
    if (!segDone) return true;
    q.T *= q.t;
    if (q.T == 0.0f) return false;
    if (q.segEnd == q.dmax) return false;
    q.rmin = q.segEnd * (1.0f + kRayEpsilon);
    q.inside = q.nextInside;
    ++q.guard;
    return trAdvance(m, q);
}

// Hands out work items [0, n) to the lanes of a warp that ask for one, in
// chunks of kTrChunk taken from a global counter (one atomic per chunk).
// All 32 lanes call it together; the chunk range is the same in every lane.
constexpr uint32_t kTrChunk = 64;

__device__ __forceinline__ uint32_t trTake(bool need, uint32_t* take, uint32_t &poolNext, uint32_t &poolEnd) {
    const unsigned mask = __ballot_sync(0xffffffffu, need);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t k = __popc(mask), rank = __popc(mask & ((1u << lane) - 1));
    uint32_t item = poolNext + rank;
    const uint32_t avail = poolEnd - poolNext;
    if (k > avail) {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(take, kTrChunk);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (rank >= avail) item = c + (rank - avail);
        poolNext = c + (k - avail);
        poolEnd = c + kTrChunk;
    } else {
        poolNext += k;
    }
    return item;
}

// Henyey-Greenstein phase function (PhaseFunction/basic_phase_functions.cpp:36-65).
__device__ __forceinline__ float hgValue(float g, float cosTheta) {
    return (1 - g * g) / (4 * kPiF * powf(1 + g * g - 2 * g * cosTheta, 1.5f));
}

__device__ __forceinline__ V3 hgSample(float g, float u0, float u1, float* pdf) {
    float sq = (1 - g * g) / (1 - g + 2 * g * u1);
    float cosTheta = fminf(fmaxf(0.5f / g * (1 + g * g - sq * sq), -1.0f), 1.0f);
    float phi = 2 * kPiF * u0;
    *pdf = hgValue(g, cosTheta);
    float sinTheta = sqrtf(1 - cosTheta * cosTheta);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return V3{cp * sinTheta, sp * sinTheta, cosTheta};
}

// ReferenceFrame(z) with Duff et al.'s orthonormal basis (Vector3D.h:59-66).
__device__ __forceinline__ Frame frameFromZ(V3 z) {
    float sign = z.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sign + z.z);
    const float b = z.x * z.y * a;
    V3 x = V3{1.0f + sign * z.x * z.x * a, sign * b, -sign * z.x};
    V3 y = V3{b, sign + z.y * z.y * a, -z.y};
    return Frame{x, y, z};
}

}  // namespace slrgpu
