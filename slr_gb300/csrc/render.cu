// Wavefront path tracer (PTRenderer semantics) on the GPU.
//
// One wave = S samples of every pixel; each path is one thread slot in SoA
// state arrays.  Per bounce: extend (closest hit) -> shade (emission with
// MIS, Russian roulette, next-event estimation, BSDF sampling) -> shadow (any
// hit) over compacted queues; after the last bounce the wave's paths are
// added to the 16-bin film with compensated summation.  The estimator is the
// reference's PTRenderer::Job::contribution (libSLR/Renderer/PTRenderer.cpp:146-276)
// and Job::kernel (:103-144); only the random numbers differ (counter-based).
#include "render_api.h"
#include "trace_ranges.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "device_bsdf.cuh"
#include "device_medium.cuh"
#include "device_trace.cuh"
#include "device_scene.cuh"

namespace slrgpu {

#define CUDA_TRY(x)                                                                 \
    do {                                                                            \
        cudaError_t e_ = (x);                                                       \
        if (e_ != cudaSuccess) {                                                    \
            setError(std::string(#x) + ": " + cudaGetErrorString(e_));             \
            return SLRGPU_ERR_CUDA;                                                 \
        }                                                                           \
    } while (0)

// ---------------------------------------------------------------------------
// Path state (structure of arrays, N = paths per wave)
// ---------------------------------------------------------------------------
// The scalars of a path in one 32-byte record: one sector per thread,
// wherever the compacted queues have scattered the path.
struct __align__(16) PathScalars {
    uint32_t info;       // bits 0-3 selected lambda, 4 wavelength selected, 5 previous delta, 8-15 depth
    float wlOffset;
    float prevPdf;       // density of the last BSDF sample (MIS of emission hits)
    float initY;         // importance of the initial throughput (Russian roulette)
    float camWeight;     // camera sample weight We0 We1 cos / (areaPDF dirPDF selectWLPDF)
    uint32_t rngCounter;
    uint32_t keyLo, keyHi;   // counter-RNG key of the path (seed, sample index, grid position)
};
static_assert(sizeof(PathScalars) == 32, "one sector per path");

struct WaveState {
    float4* ray;         // [N][2]: origin xyz + tmin, direction xyz + tmax (one sector per path)
    float4* hit;         // t, b1, b2, prim bits
    float* alpha;        // [N][16]: 16 contiguous values per path
    float* L;            // [N][16]
    PathScalars* ps;     // [N]
    float4* shRay;       // [N][2]: shadow ray, as ray
    float* shContrib;    // [N][16]
    uint32_t* queue[2];
    uint32_t* shadowQueue;
    uint32_t* classQueue;  // [kNumClassQueues][N]: paths of one bounce sorted by shading class
    uint32_t* counters;    // [kCtrStride * (maxDepth + 2)], see kCtr*
    unsigned long long* stats;  // 0 extension rays, 1 shadow rays, 2 dropped samples
    uint32_t N;
};

// The reference's renderers sample the sensor in whole 8x8 tiles
// (ImageSensor.cpp:13-14, :42-43; PTRenderer.cpp:104-110), also where a tile
// hangs over the image's right or bottom edge; ImageSensor::add
// (ImageSensor.cpp:125-130) clamps those samples into the last column / row.
// A wave therefore traces every position of the tile-padded sample grid.
constexpr uint32_t kSensorTile = 8;
__host__ __device__ __forceinline__ uint32_t padToTile(uint32_t n) {
    return (n + kSensorTile - 1) / kSensorTile * kSensorTile;
}

// Image sizes every entry point accepts: both sides positive and at most
// 2^20 (so the tile padding cannot wrap a 32-bit side), and at most 2^31 - 1
// positions in the tile-padded grid (path and film indices are 32-bit).
// The product is formed in 64 bits.
int checkImageSize(uint32_t width, uint32_t height) {
    if (width == 0 || height == 0) {
        setError("width and height must be positive");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (width > kMaxImageSide || height > kMaxImageSide) {
        setError("width and height must be at most 2^20");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if ((uint64_t)padToTile(width) * padToTile(height) > 0x7fffffffull) {
        setError("image too large: the tile-padded sample grid exceeds 2^31 - 1 positions");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    return SLRGPU_OK;
}

// One request's share of a wave: `samples` consecutive sample indices from
// `sampleBase`, each over every position of the request's tile-padded grid,
// as the paths [pathBegin, pathBegin + samples * gridPositions).  A path's
// random numbers depend only on (seed, sample index, grid position), so a
// request renders the same alone or in a wave shared with others.
struct WaveSegment {
    uint32_t pathBegin;
    uint32_t width, height;   // image
    uint32_t gridW, gridH;    // tile-padded sample grid
    uint32_t gridPositions;   // gridW * gridH
    uint32_t sampleBase, samples;
    uint32_t seed;
    uint32_t scene;           // index in the wave's scene table (waves of several scenes)
    uint32_t filmBegin;       // first pixel of the request in the wave's film enumeration
    float* filmSum;           // [16][width * height], Kahan sum and compensation
    float* filmComp;
    unsigned long long* dropped;   // non-finite samples of the request
};
constexpr int kMaxWaveSegments = 32;
struct WaveParams {
    uint32_t numSegments;
    uint32_t numPaths;        // sum of samples * gridPositions
    uint32_t filmPixels;      // sum of width * height
    uint32_t pad;
    WaveSegment seg[kMaxWaveSegments];
};

// Per-bounce counter block: [0, kNumClassQueues - 1) paths per shading
// class, kCtrExt paths in the extension queue of the bounce, kCtrShadow
// shadow rays, kCtrMedShadow shadow rays waiting for their transmittance,
// kCtrMedTake the transmittance kernel's work counter, kCtrExtTake and
// kCtrShadowTake the work counters of the surface tracer's extension and
// shadow kernels.  The first kQueueCountColumns are the diagnostics rows.
constexpr int kNumShadeClasses = 6;   // the five material kinds + environment / miss
constexpr int kClassMiss = 5;
constexpr int kClassMedium = 6;       // volumetric: a scattering point in the medium
constexpr int kQueueMedShadow = 7;    // volumetric: unoccluded shadow rays waiting for their transmittance
constexpr int kNumClassQueues = 8;
constexpr int kCtrStride = 13;
constexpr int kCtrExt = 7;
constexpr int kCtrShadow = 8;
constexpr int kCtrMedShadow = 9;
constexpr int kCtrMedTake = 10;
constexpr int kCtrExtTake = 11;
constexpr int kCtrShadowTake = 12;
// hit.w of a path whose ray stopped at a collision in the medium (hit.x = its
// distance, hit.y = 1 inside the density grid's unit cube)
constexpr uint32_t kMediumHit = 0xfffffffeu;

constexpr uint32_t kInfoSelMask = 0xfu;
constexpr uint32_t kInfoWlSelected = 1u << 4;
constexpr uint32_t kInfoPrevDelta = 1u << 5;
constexpr int kInfoSceneShift = 8;    // bits 8-15: the path's scene in a wave of several scenes
constexpr uint32_t kInfoSceneMask = 0xffu << kInfoSceneShift;
constexpr int kInfoDepthShift = 16;

// A wave of several scenes (the serving loop's shared queues): the kernels
// find each path's scene in a table in device memory by the scene index in
// its info word; single-scene waves take the scene by value (MULTI false).
constexpr int kMaxWaveScenes = 8;
template <bool MULTI>
__device__ __forceinline__ const DevScene &pathScene(const DevScene &scArg, const DevScene* __restrict__ scenes,
                                                     uint32_t info) {
    if (MULTI) return scenes[(info & kInfoSceneMask) >> kInfoSceneShift];
    return scArg;
}

__device__ __forceinline__ uint64_t loadKey(const WaveState &ws, uint32_t p) {
    return ((uint64_t)ws.ps[p].keyHi << 32) | ws.ps[p].keyLo;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// wpDev: the wave's parameters in device memory (graph-captured waves, whose
// launch parameters are fixed at capture), or null to use wpArg.
template <bool MULTI>
__global__ void kRaygen(DevScene scArg, WaveState ws, const __grid_constant__ WaveParams wpArg,
                        const WaveParams* __restrict__ wpDev, const DevScene* __restrict__ scenes,
                        bool initAlpha) {
    const WaveParams &wp = wpDev ? *wpDev : wpArg;
    if (blockIdx.x == 0 && threadIdx.x == 0) ws.counters[kCtrExt] = wp.numPaths;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < wp.numPaths; p += gridDim.x * blockDim.x) {
        uint32_t k = 0;
        while (k + 1 < wp.numSegments && p >= wp.seg[k + 1].pathBegin) ++k;
        const WaveSegment &sg = wp.seg[k];
        const DevScene &sc = MULTI ? scenes[sg.scene] : scArg;
        const uint32_t q = p - sg.pathBegin;
        uint32_t s = q / sg.gridPositions;
        uint32_t pixel = q - s * sg.gridPositions;
        uint32_t ix = pixel % sg.gridW, iy = pixel / sg.gridW;
        // replay: the path's tape slot is its grid position (one sample)
        const uint64_t key = sc.rngTape ? (uint64_t)pixel * kRngTapeStride
                                        : pathKey(sg.seed, (uint64_t)(sg.sampleBase + s) * sg.gridPositions + pixel);
        Rng rng{key, 0, sc.rngTape};
        // Draw order of Job::kernel: time, pixel (2), wavelength offset,
        // wavelength selection, lens (2) (PTRenderer.cpp:108-116).
        (void)rng.next();
        float pxf = ix + rng.next();
        float pyf = iy + rng.next();
        float wlOff = rng.next();
        float uSel = rng.next();
        float lu0 = rng.next(), lu1 = rng.next();
        uint32_t sel = min((uint32_t)(kNumLambda * uSel), (uint32_t)(kNumLambda - 1));
        const float selectWLPDF = kNumLambda / (kWavelengthHigh - kWavelengthLow);
        V3 org, dir;
        float w;
        cameraRay(sc.camera, lu0, lu1, pxf / sg.width, pyf / sg.height, &org, &dir, &w);
        ws.ray[2 * (size_t)p] = make_float4(org.x, org.y, org.z, 0.0f);
        ws.ray[2 * (size_t)p + 1] = make_float4(dir.x, dir.y, dir.z, __int_as_float(0x7f800000));
        PathScalars ps;
        ps.info = sel | (MULTI ? sg.scene << kInfoSceneShift : 0u);
        ps.wlOffset = wlOff;
        ps.prevPdf = 0.0f;
        ps.initY = importance(specConst(1.0f), (int)sel);
        ps.camWeight = w / selectWLPDF;
        ps.rngCounter = rng.counter;
        ps.keyLo = (uint32_t)key;
        ps.keyHi = (uint32_t)(key >> 32);
        ws.ps[p] = ps;
        // the surface path tracer's kernels take the throughput of a
        // depth-0 path as 1 without reading it
        if (initAlpha) storeSpec(ws.alpha, p, specConst(1.0f));
        storeSpec(ws.L, p, specConst(0.0f));
        ws.queue[0][p] = p;
    }
}

// Resident blocks per SM the traversal kernels are compiled for; a
// compile-time tuning constant.
#ifndef SLRGPU_TRACE_MIN_BLOCKS
#define SLRGPU_TRACE_MIN_BLOCKS 4
#endif
// Dynamic ray fetch in the wave's traversal kernels (Aila and Laine,
// "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009): each
// warp takes rays from the bounce's queue through a work counter, and
// once SLRGPU_TRACE_REFILL_LANES of its lanes have finished their walks
// they take new rays while the others go on walking; walks advance
// SLRGPU_TRACE_REFILL_VISITS node visits between two looks.  0 turns it off
// (one ray per lane and grid-stride loop).
#ifndef SLRGPU_TRACE_REFILL
#define SLRGPU_TRACE_REFILL 1
#endif
#ifndef SLRGPU_TRACE_REFILL_LANES
#define SLRGPU_TRACE_REFILL_LANES 8
#endif
#ifndef SLRGPU_TRACE_REFILL_VISITS
#define SLRGPU_TRACE_REFILL_VISITS 16
#endif
static_assert(SLRGPU_TRACE_REFILL_LANES >= 1 && SLRGPU_TRACE_REFILL_LANES <= 32, "a warp has 32 lanes");
// The same threshold for the ray-query kernel (slrgpu_trace_rays).
#ifndef SLRGPU_QUERY_REFILL_LANES
#define SLRGPU_QUERY_REFILL_LANES SLRGPU_TRACE_REFILL_LANES
#endif
static_assert(SLRGPU_QUERY_REFILL_LANES >= 1 && SLRGPU_QUERY_REFILL_LANES <= 32, "a warp has 32 lanes");

// The refill step of a warp: when at least SLRGPU_TRACE_REFILL_LANES lanes
// are idle and the queue is not drained, the idle lanes take the next queue
// entries (*slot = entry index, or n when there is none left).  Returns
// whether this lane got one.  Called by all 32 lanes.
__device__ __forceinline__ bool refillLanes(bool live, uint32_t* cursor, uint32_t n, bool &drained, uint32_t* slot) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t idle = __ballot_sync(0xffffffffu, !live);
    if (drained || (uint32_t)__popc(idle) < SLRGPU_TRACE_REFILL_LANES) return false;
    const int leader = __ffs(idle) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(cursor, (uint32_t)__popc(idle));
    base = __shfl_sync(0xffffffffu, base, leader);
    drained = base + (uint32_t)__popc(idle) >= n;
    if (live) return false;
    *slot = base + (uint32_t)__popc(idle & ((1u << lane) - 1));
    return *slot < n;
}

// Shadow rays (PTRenderer.cpp:196-217): an unoccluded ray adds its stored
// contribution to the path's radiance.
// VOL: an unoccluded ray of a scene with a medium goes to the transmittance
// queue (medQueue) instead.
template <bool MULTI, bool WT, bool VOL = false>
__device__ __forceinline__ void shadowRefill(const DevScene &scArg, const WaveState &ws,
                                             const uint32_t* __restrict__ queue, uint32_t n, uint32_t* cursor,
                                             const DevScene* __restrict__ scenes, uint32_t* medQueue = nullptr,
                                             uint32_t* medCount = nullptr) {
    uint32_t stack[kTraceStack];
    AnyWalk<WT> walk;
    uint32_t p = 0, info = 0;
    bool live = false, drained = false;
    for (;;) {
        uint32_t slot;
        bool fin = false;
        if (refillLanes(live, cursor, n, drained, &slot)) {
            p = queue[slot];
            info = MULTI ? ws.ps[p].info : 0u;
            const float4 o = ws.shRay[2 * (size_t)p], d = ws.shRay[2 * (size_t)p + 1];
            fin = walk.begin(pathScene<MULTI>(scArg, scenes, info), V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w);
            live = true;
        }
        if (live && !fin) fin = walk.advance(pathScene<MULTI>(scArg, scenes, info), stack, SLRGPU_TRACE_REFILL_VISITS);
        bool pushMedium = false;
        if (live && fin) {
            if (!walk.occluded) {
                if (VOL && scArg.medium.present) {
                    pushMedium = true;
                } else {
                    Spec c;
                    loadSpec(ws.shContrib, p, c);
                    addSpec(ws.L, p, c);
                }
            }
            live = false;
        }
        if (VOL && __any_sync(0xffffffffu, pushMedium)) queuePush(medQueue, medCount, p, pushMedium);
        if (drained && !__any_sync(0xffffffffu, live)) return;
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256, SLRGPU_TRACE_MIN_BLOCKS) kShadow(DevScene scArg, WaveState ws,
                                                                      const uint32_t* __restrict__ queue,
                                                                      const uint32_t* __restrict__ count,
                                                                      uint32_t* cursor,
                                                                      const DevScene* __restrict__ scenes) {
    const uint32_t n = *count;
#if SLRGPU_TRACE_REFILL
    if (scArg.watertight) shadowRefill<MULTI, true>(scArg, ws, queue, n, cursor, scenes);
    else shadowRefill<MULTI, false>(scArg, ws, queue, n, cursor, scenes);
#else
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t p = queue[i];
        const DevScene &sc = pathScene<MULTI>(scArg, scenes, MULTI ? ws.ps[p].info : 0u);
        float4 o = ws.shRay[2 * (size_t)p], d = ws.shRay[2 * (size_t)p + 1];
        if (!traceAny(sc, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w)) {
            Spec c;
            loadSpec(ws.shContrib, p, c);
            addSpec(ws.L, p, c);
        }
    }
#endif
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ws.stats[1], (unsigned long long)n);
}

// ---------------------------------------------------------------------------
// Material-sorted surface shading.  The extension kernel sorts every path of
// a bounce into one queue per shading class (material kind, or environment
// for rays that hit nothing); one kernel per class then shades its queue with
// that material's BSDF compiled in alone, which keeps each kernel's code
// small (instruction-cache resident) and its warps free of material
// divergence.  Emission with MIS, Russian roulette, next-event estimation and
// BSDF sampling follow PTRenderer::Job::contribution (PTRenderer.cpp:145-277).
// ---------------------------------------------------------------------------
// Russian roulette at the hit (PTRenderer.cpp:266-272) for materials that do
// not emit.  A vertex adds its emission before the roulette; with none to add,
// the roulette is the vertex's first draw from the path's random numbers, so
// the extension kernel can draw it as soon as the hit is known and a path that
// ends there never reaches a shading kernel (at depth > 0 about half of them
// end, and in a shading warp their lanes would idle through next-event
// estimation and BSDF sampling).  The shading kernel of a surviving path
// recomputes the same continuation probability from the same inputs and
// skips the draw.  Returns false when the path ends here (roulette, or the
// maximum depth reached).
#ifndef SLRGPU_EARLY_ROULETTE
#define SLRGPU_EARLY_ROULETTE 1
#endif
__device__ __forceinline__ bool rouletteAtHit(const DevScene &sc, const WaveState &ws, uint32_t p, uint32_t maxDepth) {
    const uint32_t info = ws.ps[p].info;
    const uint32_t depth = info >> kInfoDepthShift;
    if (depth + 1 > maxDepth) return false;
    if (depth == 0) return true;
    Spec alpha;
    loadSpec(ws.alpha, p, alpha);
    const float cp = fminf(importance(alpha, (int)(info & kInfoSelMask)) / ws.ps[p].initY, 1.0f);
    Rng rng{loadKey(ws, p), ws.ps[p].rngCounter, sc.rngTape};
    if (!(rng.next() < cp)) return false;
    ws.ps[p].rngCounter = rng.counter;
    return true;
}

// The shading class of a finished extension ray, or -1 when the path ends at
// the hit's roulette.
__device__ __forceinline__ int hitClass(const DevScene &sc, const WaveState &ws, uint32_t p, uint32_t prim,
                                        uint32_t maxDepth) {
    if (prim == kNoHit) return kClassMiss;
    const DevMaterial &m = sc.materials[sc.prims[prim].material];
    const int cls = (int)m.kind;
    if (SLRGPU_EARLY_ROULETTE && m.emit < 0 && !rouletteAtHit(sc, ws, p, maxDepth)) return -1;
    return cls;
}

// Closest hits of the bounce's extension rays, each path pushed to the
// queue of its shading class (material kind, or miss).
template <bool MULTI>
__device__ __forceinline__ void pushByClass(const WaveState &ws, uint32_t* classCounts, uint32_t p, int cls) {
#pragma unroll
    for (int c = 0; c < kNumShadeClasses; ++c)
        queuePush(ws.classQueue + (size_t)c * ws.N, classCounts + c, p, cls == c);
}

// SORT: push each path to the queue of its shading class.
template <bool MULTI, bool WT, bool SORT = true>
__device__ __forceinline__ void extendRefill(const DevScene &scArg, const WaveState &ws,
                                             const uint32_t* __restrict__ queue, uint32_t n, uint32_t* cursor,
                                             uint32_t* classCounts, const DevScene* __restrict__ scenes,
                                             uint32_t maxDepth = 0) {
    StackEntry stack[kTraceStack];
    ClosestWalk<WT> walk;
    uint32_t p = 0, info = 0;
    bool live = false, drained = false;
    for (;;) {
        uint32_t slot;
        bool fin = false;
        if (refillLanes(live, cursor, n, drained, &slot)) {
            p = queue[slot];
            info = MULTI ? ws.ps[p].info : 0u;
            const float4 o = ws.ray[2 * (size_t)p], d = ws.ray[2 * (size_t)p + 1];
            fin = walk.begin(pathScene<MULTI>(scArg, scenes, info), V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w);
            live = true;
        }
        if (live && !fin) fin = walk.advance(pathScene<MULTI>(scArg, scenes, info), stack, SLRGPU_TRACE_REFILL_VISITS);
        int cls = -1;
        if (live && fin) {
            const DevScene &sc = pathScene<MULTI>(scArg, scenes, info);
            const Hit &h = walk.hit;
            ws.hit[p] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.prim));
            if (SORT) cls = hitClass(sc, ws, p, h.prim, maxDepth);
            live = false;
        }
        if (SORT && __any_sync(0xffffffffu, cls >= 0)) pushByClass<MULTI>(ws, classCounts, p, cls);
        if (drained && !__any_sync(0xffffffffu, live)) return;
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256, SLRGPU_TRACE_MIN_BLOCKS) kExtendSort(DevScene scArg, WaveState ws,
                                                                          const uint32_t* __restrict__ queue,
                            const uint32_t* __restrict__ count, uint32_t* classCounts, uint32_t* cursor,
                            uint32_t maxDepth, const DevScene* __restrict__ scenes) {
    const uint32_t n = *count;
#if SLRGPU_TRACE_REFILL
    if (scArg.watertight) extendRefill<MULTI, true>(scArg, ws, queue, n, cursor, classCounts, scenes, maxDepth);
    else extendRefill<MULTI, false>(scArg, ws, queue, n, cursor, classCounts, scenes, maxDepth);
#else
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        int cls = -1;
        uint32_t p = 0;
        if (active) {
            p = queue[i];
            const DevScene &sc = pathScene<MULTI>(scArg, scenes, MULTI ? ws.ps[p].info : 0u);
            float4 o = ws.ray[2 * (size_t)p], d = ws.ray[2 * (size_t)p + 1];
            Hit h;
            traceClosest(sc, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w, &h);
            ws.hit[p] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.prim));
            cls = hitClass(sc, ws, p, h.prim, maxDepth);
        }
        pushByClass<MULTI>(ws, classCounts, p, cls);
    }
#endif
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ws.stats[0], (unsigned long long)n);
}

// Closest hits of the volumetric path tracer's extension rays (the medium
// interaction comes after, in kVolInteract).
__global__ void __launch_bounds__(256, SLRGPU_TRACE_MIN_BLOCKS) kExtend(DevScene sc, WaveState ws,
                                                                      const uint32_t* __restrict__ queue,
                                                                      const uint32_t* __restrict__ count,
                                                                      uint32_t* cursor) {
    const uint32_t n = *count;
#if SLRGPU_TRACE_REFILL
    if (sc.watertight) extendRefill<false, true, false>(sc, ws, queue, n, cursor, nullptr, nullptr);
    else extendRefill<false, false, false>(sc, ws, queue, n, cursor, nullptr, nullptr);
#else
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t p = queue[i];
        float4 o = ws.ray[2 * (size_t)p], d = ws.ray[2 * (size_t)p + 1];
        Hit h;
        traceClosest(sc, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w, &h);
        ws.hit[p] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.prim));
    }
#endif
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ws.stats[0], (unsigned long long)n);
}

// Paths whose ray left the scene: environment emission (with MIS after a
// non-delta bounce), then the path ends (PTRenderer.cpp:150-152, :234-263).
template <bool MULTI>
__global__ void kShadeMiss(DevScene scArg, WaveState ws, const uint32_t* __restrict__ queue,
                           const uint32_t* __restrict__ count, const DevScene* __restrict__ scenes) {
    const uint32_t n = *count;
    if (!MULTI && !scArg.envPresent) return;
    const float twoPi = 6.28318530717958647692f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = queue[i];
        const uint32_t info = ws.ps[p].info;
        const DevScene &sc = pathScene<MULTI>(scArg, scenes, info);
        if (MULTI && !sc.envPresent) continue;     // no environment: the path just ends
        const uint32_t depth = info >> kInfoDepthShift;
        const bool prevDelta = (info & kInfoPrevDelta) != 0;
        const float wlOff = ws.ps[p].wlOffset;
        const OffsetLambdas lambdas{wlOff};
        float4 rd = ws.ray[2 * (size_t)p + 1];
        V3 dir = V3{rd.x, rd.y, rd.z};
        float theta, phi;
        toPolarYUp(dir, &theta, &phi);
        Spec Le;
        envRadiance(sc, phi / twoPi, theta / kPiF, lambdas, Le);
        float mis = 1.0f;
        if (depth > 0 && !prevDelta) {
            float lightProb = sc.envImportance / (sc.surfImportance + sc.envImportance);
            float lightPdf = lightProb * envAreaPdf(sc, phi, theta) * 1.0f / absDot(dir, -dir);
            float bp = ws.ps[p].prevPdf;
            mis = (bp * bp) / (lightPdf * lightPdf + bp * bp);
        }
        Spec a;
        if (depth == 0) a = specConst(1.0f);
        else loadSpec(ws.alpha, p, a);
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) a.v[k] = a.v[k] * Le.v[k] * mis;
        addSpec(ws.L, p, a);
    }
}

// Resident blocks per SM the shading kernels are compiled for (register cap
// 65536 / (256 x this)); compile-time tuning constants, the GGX dielectric's
// (the largest body: per-wavelength refraction) on its own.
#ifndef SLRGPU_SHADE_SMEM_ALPHA
#define SLRGPU_SHADE_SMEM_ALPHA 1
#endif
#ifndef SLRGPU_SHADE_SMEM_SP
#define SLRGPU_SHADE_SMEM_SP 1
#endif
// A surface point in shared memory, [component][thread] (blocks of 256).
__device__ __forceinline__ void storeSurfShared(float* s, const SurfPoint &sp) {
    const float v[15] = {sp.p.x, sp.p.y, sp.p.z, sp.frame.x.x, sp.frame.x.y, sp.frame.x.z, sp.frame.y.x,
                         sp.frame.y.y, sp.frame.y.z, sp.frame.z.x, sp.frame.z.y, sp.frame.z.z, sp.gn.x, sp.gn.y,
                         sp.gn.z};
#pragma unroll
    for (int k = 0; k < 15; ++k) s[k * 256 + threadIdx.x] = v[k];
}
__device__ __forceinline__ SurfPoint loadSurfShared(const float* s) {
    float v[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) v[k] = s[k * 256 + threadIdx.x];
    SurfPoint sp;
    sp.p = V3{v[0], v[1], v[2]};
    sp.frame = Frame{V3{v[3], v[4], v[5]}, V3{v[6], v[7], v[8]}, V3{v[9], v[10], v[11]}};
    sp.gn = V3{v[12], v[13], v[14]};
    return sp;
}
#ifndef SLRGPU_SHADE_MIN_BLOCKS
#define SLRGPU_SHADE_MIN_BLOCKS 3   // 85 registers: +9 % on the 1M-triangle benchmark over 2 (128)
#endif
#ifndef SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS
#define SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS SLRGPU_SHADE_MIN_BLOCKS
#endif
template <int K, bool MULTI>
__global__ void __launch_bounds__(256, K == kMatGGXScattering ? SLRGPU_SHADE_DIELECTRIC_MIN_BLOCKS
                                                               : SLRGPU_SHADE_MIN_BLOCKS) kShadeSurf(DevScene scArg, WaveState ws, uint32_t maxDepth,
                                                  const uint32_t* __restrict__ inQueue,
                                                  const uint32_t* __restrict__ inCount, uint32_t* outQueue,
                                                  uint32_t* outCount, uint32_t* shQueue, uint32_t* shCount,
                                                  const DevScene* __restrict__ scenes) {
    const uint32_t n = *inCount;
    const uint32_t N = ws.N;
    const float inf = __int_as_float(0x7f800000);
    const float twoPi = 6.28318530717958647692f;
#if SLRGPU_SHADE_SMEM_ALPHA
    // the path's throughput in shared memory ([wavelength][thread]), not in
    // registers, through light and BSDF sampling
    __shared__ float sAlpha[kNumLambda * 256];
#define SLRGPU_ALPHA(k) sAlpha[(k) * 256 + threadIdx.x]
#endif
#if SLRGPU_SHADE_SMEM_SP
    // the surface point likewise, from the BSDF query to the new ray
    __shared__ float sSurf[15 * 256];
#endif
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool active = i < n;
        bool extend = false, shadow = false;
        uint32_t p = active ? inQueue[i] : 0;
        if (active) {
            uint32_t info = ws.ps[p].info;
            const DevScene &sc = pathScene<MULTI>(scArg, scenes, info);
            const uint32_t sceneBits = info & kInfoSceneMask;
            const int sel = (int)(info & kInfoSelMask);
            bool wlSelected = (info & kInfoWlSelected) != 0;
            const bool prevDelta = (info & kInfoPrevDelta) != 0;
            uint32_t depth = info >> kInfoDepthShift;
            const float wlOff = ws.ps[p].wlOffset;
            const OffsetLambdas lambdas{wlOff};
            Rng rng{loadKey(ws, p), ws.ps[p].rngCounter, sc.rngTape};
            float4 ro = ws.ray[2 * (size_t)p], rd = ws.ray[2 * (size_t)p + 1];
            V3 org = V3{ro.x, ro.y, ro.z}, dir = V3{rd.x, rd.y, rd.z};
            float4 hv = ws.hit[p];
            const DevPrim pr = sc.prims[__float_as_uint(hv.w)];
#if SLRGPU_SHADE_SMEM_ALPHA
            {
                Spec a0;
                if (depth == 0) a0 = specConst(1.0f);
                else loadSpec(ws.alpha, p, a0);
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) SLRGPU_ALPHA(k) = a0.v[k];
            }
#else
            Spec alpha;
            if (depth == 0) alpha = specConst(1.0f);
            else loadSpec(ws.alpha, p, alpha);
#define SLRGPU_ALPHA(k) alpha.v[k]
#endif
            bool alive = true;
            SurfPoint sp;
            surfacePoint(sc, pr, org, dir, hv.x, hv.y, hv.z, sp);
            const DevMaterial mat = sc.materials[pr.material];
            V3 dirOut = sp.frame.toLocal(-dir);
            // Emission on hit (PTRenderer.cpp:162-166, :240-263).
            if (mat.emit >= 0) {
                Spec M;
                evalSpectrum(sc, mat.emit, lambdas, M);
                float edf = dirOut.z > 0.0f ? kInvPiF : 0.0f;
                float mis = 1.0f;
                if (depth > 0 && !prevDelta) {
                    float lightProb = (sc.surfImportance / (sc.surfImportance + sc.envImportance)) * sc.lightPMF[0];
                    float dist2 = sqLength(sp.p - org);
                    float lightPdf = lightProb * pr.invArea * dist2 / absDot(dir, sp.gn);
                    float bp = ws.ps[p].prevPdf;
                    mis = (bp * bp) / (lightPdf * lightPdf + bp * bp);
                }
                Spec add;
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) add.v[k] = SLRGPU_ALPHA(k) * (M.v[k] * edf) * mis;
                addSpec(ws.L, p, add);
            }
            // Russian roulette (PTRenderer.cpp:266-272); a material that does
            // not emit had its draw at the hit (rouletteAtHit), and the path
            // is here because it continued.
            if (depth > 0) {
                Spec a1;
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) a1.v[k] = SLRGPU_ALPHA(k);
                float cp = fminf(importance(a1, sel) / ws.ps[p].initY, 1.0f);
                if ((SLRGPU_EARLY_ROULETTE && mat.emit < 0) || rng.next() < cp) {
                    float r = 1.0f / cp;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) SLRGPU_ALPHA(k) *= r;
                } else {
                    alive = false;
                }
            }
            if (alive) {
                ++depth;
                if (depth > maxDepth) alive = false;
            }
            if (alive) {
                Bsdf B;
                makeBsdfK<K>(sc, mat, lambdas, wlSelected, B);
                BsdfQuery q{dirOut, sp.frame.toLocal(sp.gn), sel};
#if SLRGPU_SHADE_SMEM_SP
                storeSurfShared(sSurf, sp);
#define SLRGPU_SP() loadSurfShared(sSurf)
#else
#define SLRGPU_SP() sp
#endif
                // Next-event estimation (PTRenderer.cpp:179-218).
                if (bsdfHasNonDelta(K) && (sc.numLights > 0 || sc.envPresent)) {
                    const SurfPoint spN = SLRGPU_SP();
                    float lightProb;
                    int li = selectLight(sc, rng.next(), &lightProb);
                    float lu0 = rng.next(), lu1 = rng.next();
                    V3 lp, lgn;
                    Spec M;
                    float areaPdf, edfVal, dist2;
                    bool atInf = false;
                    V3 shadowDir;
                    if (li >= 0) {
                        const DevPrim lpr = sc.prims[sc.lightPrims[li]];
                        float su = sqrtf(lu0);
                        float b0 = 1.0f - su, b1 = lu1 * su, b2 = 1.0f - b0 - b1;
                        float4 p0 = sc.vpos[lpr.v0], p1 = sc.vpos[lpr.v1], p2 = sc.vpos[lpr.v2];
                        lp = rn_bary(b0, V3{p0.x, p0.y, p0.z}, b1, V3{p1.x, p1.y, p1.z}, b2, V3{p2.x, p2.y, p2.z});
                        float4 n0 = sc.vnrm[lpr.v0], n1 = sc.vnrm[lpr.v1], n2 = sc.vnrm[lpr.v2];
                        V3 lz = normalize(b0 * V3{n0.x, n0.y, n0.z} + b1 * V3{n1.x, n1.y, n1.z} + b2 * V3{n2.x, n2.y, n2.z});
                        lgn = V3{lpr.ngx, lpr.ngy, lpr.ngz};
                        areaPdf = lpr.invArea;
                        evalSpectrum(sc, sc.materials[lpr.material].emit, lambdas, M);
                        V3 diff = lp - spN.p;
                        dist2 = sqLength(diff);
                        shadowDir = diff * (1.0f / sqrtf(dist2));
                        edfVal = dot(lz, -shadowDir) > 0.0f ? kInvPiF : 0.0f;
                    } else {
                        float uvPdf, topPdf;
                        uint32_t row, col;
                        float d1 = sampleAlias(sc.envTopAlias, sc.envTopPDF, sc.envMapH, lu1, &topPdf, &row);
                        float d0 = sampleAlias(sc.envRowAlias + (size_t)row * sc.envMapW,
                                               sc.envRowPDF + (size_t)row * sc.envMapW, sc.envMapW, lu0, &uvPdf, &col);
                        uvPdf *= topPdf;
                        float phi = d0 * twoPi, theta = d1 * kPiF;
                        float sph, cph, sth, cth;
                        sincosf(phi, &sph, &cph);
                        sincosf(theta, &sth, &cth);
                        lp = V3{-sph * sth, cth, cph * sth};
                        lgn = -lp;
                        atInf = true;
                        areaPdf = uvPdf / (2.0f * kPiF * kPiF * sth);
                        envRadiance(sc, phi / twoPi, theta / kPiF, lambdas, M);
                        edfVal = 1.0f;
                        shadowDir = normalize(lp);
                        dist2 = 1.0f;
                    }
                    float cosShading = absDot(shadowDir, spN.gn);
                    float cosLight = absDot(shadowDir, lgn);
                    if (cosShading * cosLight > 0) {
                        float lightPdf = lightProb * areaPdf;
                        V3 sdl = spN.frame.toLocal(shadowDir);
                        Spec fs;
                        bsdfEval<K>(B, q, sdl, fs);
                        float bsdfPdfV = bsdfPdf<K>(B, q, sdl) * cosLight / dist2;
                        float mis = 1.0f;
                        if (!isinf(areaPdf))
                            mis = (lightPdf * lightPdf) / (lightPdf * lightPdf + bsdfPdfV * bsdfPdfV);
                        float G = cosShading * cosLight / dist2;
                        float scale = G * mis / lightPdf;
                        Spec c;
                        bool nz = false;
#pragma unroll
                        for (int k = 0; k < kNumLambda; ++k) {
                            c.v[k] = ((SLRGPU_ALPHA(k) * (M.v[k] * edfVal)) * fs.v[k]) * scale;
                            nz |= c.v[k] != 0.0f;
                        }
                        if (nz) {
                            storeSpec(ws.shContrib, p, c);
                            float tmax;
                            V3 sdir;
                            if (atInf) {
                                sdir = shadowDir;
                                tmax = 3.402823466e+38f;
                            } else {
                                V3 dd = lp - spN.p;
                                float dist = length(dd);
                                sdir = dd * (1.0f / dist);
                                tmax = dist * (1 - kRayEpsilon);
                            }
                            ws.shRay[2 * (size_t)p] = make_float4(spN.p.x, spN.p.y, spN.p.z, kRayEpsilon);
                            ws.shRay[2 * (size_t)p + 1] = make_float4(sdir.x, sdir.y, sdir.z, tmax);
                            shadow = true;
                        }
                    }
                }
                // BSDF sampling (PTRenderer.cpp:220-236).
                float uc = rng.next(), u0 = rng.next(), u1 = rng.next();
                BsdfSample bs;
                Spec fs;
                bsdfSample<K>(B, q, uc, u0, u1, &bs, fs);
                if (bs.pdf == 0.0f || specIsZero(fs)) {
                    alive = false;
                } else {
                    if ((bs.type & kDirDispersive) && !wlSelected) {
                        bs.pdf /= kNumLambda;
                        wlSelected = true;
                    }
                    float cg = absDot(bs.dir, q.gn);
                    float r = 1.0f / bs.pdf;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) SLRGPU_ALPHA(k) *= (fs.v[k] * cg) * r;
                    const SurfPoint spS = SLRGPU_SP();
                    V3 nd = spS.frame.fromLocal(bs.dir);
                    ws.ray[2 * (size_t)p] = make_float4(spS.p.x, spS.p.y, spS.p.z, kRayEpsilon);
                    ws.ray[2 * (size_t)p + 1] = make_float4(nd.x, nd.y, nd.z, inf);
                    ws.ps[p].prevPdf = bs.pdf;
                    info = (uint32_t)sel | (wlSelected ? kInfoWlSelected : 0u) |
                           (dirIsDelta(bs.type) ? kInfoPrevDelta : 0u) | (depth << kInfoDepthShift) | sceneBits;
                    ws.ps[p].info = info;
                    {
                        Spec a2;
#pragma unroll
                        for (int k = 0; k < kNumLambda; ++k) a2.v[k] = SLRGPU_ALPHA(k);
                        storeSpec(ws.alpha, p, a2);
                    }
                    extend = true;
                }
            }
            ws.ps[p].rngCounter = rng.counter;
        }
        queuePush(shQueue, shCount, p, active && shadow);
        queuePush(outQueue, outCount, p, active && extend);
    }
}

// ---------------------------------------------------------------------------
#undef SLRGPU_ALPHA
#undef SLRGPU_SP
// Volumetric path tracing (VolumetricPTRenderer::Job::contribution,
// libSLR/Renderer/VolumetricPTRenderer.cpp:146-296)
// ---------------------------------------------------------------------------
#ifndef SLRGPU_SHADEVOL_MIN_BLOCKS
#define SLRGPU_SHADEVOL_MIN_BLOCKS 3   // resident blocks per SM of the volumetric shading kernels
#endif
#ifndef SLRGPU_VOLINTERACT_MIN_BLOCKS
#define SLRGPU_VOLINTERACT_MIN_BLOCKS SLRGPU_SHADEVOL_MIN_BLOCKS   // of the free-flight kernel
#endif
// Scene::interact for the volumetric integrator (Scene.cpp:66-94): the
// closest surface hit is known; a collision in the medium before it may stop
// the ray (delta tracking at the selected wavelength, ratio-tracking
// throughput for the others).  The throughput (and a collision's extinction
// coefficient) goes into alpha, the path into the queue of its class: the
// medium, a surface material kind, or the environment.  Splitting the
// interaction from the shading keeps each shading kernel's code to one
// vertex kind.
__global__ void __launch_bounds__(256, SLRGPU_VOLINTERACT_MIN_BLOCKS) kVolInteract(DevScene sc, WaveState ws,
                                                                              const uint32_t* __restrict__ queue,
                                                                              const uint32_t* __restrict__ count,
                                                                              uint32_t* classCounts) {
    const uint32_t n = *count;
    const float inf = __int_as_float(0x7f800000);
    const DevMedium &med = sc.medium;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        int cls = -1;
        uint32_t p = 0;
        if (i < n) {
            p = queue[i];
            float4 hv = ws.hit[p];
            const uint32_t prim = __float_as_uint(hv.w);
            bool medHit = false;
            if (med.present) {
                const uint32_t info = ws.ps[p].info;
                const int sel = (int)(info & kInfoSelMask);
                const bool wlSelected = (info & kInfoWlSelected) != 0;
                const float wlOff = ws.ps[p].wlOffset;
                const OffsetLambdas lambdas{wlOff};
                Rng rng{loadKey(ws, p), ws.ps[p].rngCounter};
                const float4 ro = ws.ray[2 * (size_t)p], rd = ws.ray[2 * (size_t)p + 1];
                const V3 org = V3{ro.x, ro.y, ro.z}, dir = V3{rd.x, rd.y, rd.z};
                Spec sigmaE, thr, alpha;
                evalSpectrum(sc, med.sigmaE, lambdas, sigmaE);
                float tMed = 0.0f;
                V3 mparam = V3{0, 0, 0};
                medHit = mediumInteract(med, org, dir, ro.w, prim == kNoHit ? inf : hv.x, sigmaE, sel, wlSelected,
                                        rng, &tMed, &mparam, thr);
                loadSpec(ws.alpha, p, alpha);
#pragma unroll
                for (int k = 0; k < kNumLambda; ++k) alpha.v[k] *= thr.v[k];
                if (medHit) {
                    const float dens = mediumDensity(med, mparam);
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) alpha.v[k] *= dens * sigmaE.v[k];
                    ws.hit[p] = make_float4(tMed, outsideUnit(mparam) ? 0.0f : 1.0f, 0.0f, __uint_as_float(kMediumHit));
                }
                storeSpec(ws.alpha, p, alpha);
                ws.ps[p].rngCounter = rng.counter;
            }
            if (medHit) cls = kClassMedium;
            else if (prim != kNoHit) cls = (int)sc.materials[sc.prims[prim].material].kind;
            else if (sc.envPresent) cls = kClassMiss;
        }
#pragma unroll
        for (int c = 0; c < kNumClassQueues - 1; ++c)
            queuePush(ws.classQueue + (size_t)c * ws.N, classCounts + c, p, cls == c);
    }
}

template <int K>
__global__ void __launch_bounds__(256, SLRGPU_SHADEVOL_MIN_BLOCKS) kShadeVol(DevScene sc, WaveState ws, uint32_t maxDepth,
                                                 const uint32_t* __restrict__ inQueue,
                                                 const uint32_t* __restrict__ inCount, uint32_t* outQueue,
                                                 uint32_t* outCount, uint32_t* shQueue, uint32_t* shCount) {
    const uint32_t n = *inCount;
    const uint32_t N = ws.N;
    const float inf = __int_as_float(0x7f800000);
    const float twoPi = 6.28318530717958647692f;
    const DevMedium &med = sc.medium;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool active = i < n;
        bool extend = false, shadow = false;
        uint32_t p = active ? inQueue[i] : 0;
        if (active) {
            uint32_t info = ws.ps[p].info;
            const int sel = (int)(info & kInfoSelMask);
            bool wlSelected = (info & kInfoWlSelected) != 0;
            const bool prevDelta = (info & kInfoPrevDelta) != 0;
            uint32_t depth = info >> kInfoDepthShift;
            const float wlOff = ws.ps[p].wlOffset;
            const OffsetLambdas lambdas{wlOff};
            Rng rng{loadKey(ws, p), ws.ps[p].rngCounter};
            float4 ro = ws.ray[2 * (size_t)p], rd = ws.ray[2 * (size_t)p + 1];
            V3 org = V3{ro.x, ro.y, ro.z}, dir = V3{rd.x, rd.y, rd.z};
            float4 hv = ws.hit[p];
            uint32_t prim = __float_as_uint(hv.w);
            Spec alpha;
            loadSpec(ws.alpha, p, alpha);
            bool alive = true;

            // The interaction (kVolInteract): K is its class; the medium
            // throughput and a collision's extinction are in alpha already.
            constexpr bool isMedium = K == kClassMedium;
            constexpr bool atInf = K == kClassMiss;
            constexpr int KB = K < kClassMiss ? K : (int)kMatMatte;   // the material kind of surface classes
            V3 P = V3{0, 0, 0};
            Frame frame = Frame{V3{1, 0, 0}, V3{0, 1, 0}, V3{0, 0, 1}};
            V3 gn = V3{0, 0, 1};
            DevMaterial mat;
            mat.kind = kMatNull;
            mat.emit = -1;
            float hitInvArea = 0.0f;
            Spec sigmaE;
            bool inMedium = false;
            if (isMedium) {
                P = rn_ray_point(org, dir, hv.x);
                frame = frameFromZ(normalize(dir));
                evalSpectrum(sc, med.sigmaE, lambdas, sigmaE);
                inMedium = hv.y != 0.0f;
            } else if (!atInf) {
                const DevPrim pr = sc.prims[prim];
                SurfPoint sp;
                surfacePoint(sc, pr, org, dir, hv.x, hv.y, hv.z, sp);
                P = sp.p;
                frame = sp.frame;
                gn = sp.gn;
                mat = sc.materials[pr.material];
                hitInvArea = pr.invArea;
            }
            if (alive) {
                // Emission (VolumetricPTRenderer.cpp:175-180, :262-278).  The
                // light probability of a surface or environment hit is the one
                // the surface query set (Scene::interact stores the share of
                // surfaces / environment on the medium interaction instead).
                Spec Le;
                bool emitting = false;
                float lightPdf = 0.0f;
                if (atInf) {
                    float theta, phi;
                    toPolarYUp(dir, &theta, &phi);
                    envRadiance(sc, phi / twoPi, theta / kPiF, lambdas, Le);
                    emitting = true;
                    if (depth > 0) lightPdf = 1.0f * envAreaPdf(sc, phi, theta) * 1.0f / absDot(dir, -dir);
                } else if (!isMedium && mat.emit >= 0) {
                    Spec M;
                    evalSpectrum(sc, mat.emit, lambdas, M);
                    V3 dirOut = frame.toLocal(-dir);
                    float edf = dirOut.z > 0.0f ? kInvPiF : 0.0f;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) Le.v[k] = M.v[k] * edf;
                    emitting = true;
                    if (depth > 0) {
                        float dist2 = sqLength(P - org);
                        lightPdf = sc.lightPMF[0] * hitInvArea * dist2 / absDot(dir, gn);
                    }
                }
                if (emitting) {
                    float mis = 1.0f;
                    if (depth > 0 && !prevDelta) {
                        float bp = ws.ps[p].prevPdf;
                        mis = (bp * bp) / (lightPdf * lightPdf + bp * bp);
                    }
                    Spec add;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) add.v[k] = alpha.v[k] * Le.v[k] * mis;
                    addSpec(ws.L, p, add);
                }
                if (atInf) alive = false;
            }
            if (alive && depth > 0) {
                float cp = fminf(importance(alpha, sel) / ws.ps[p].initY, 1.0f);
                if (rng.next() < cp) {
                    float r = 1.0f / cp;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) alpha.v[k] *= r;
                } else {
                    alive = false;
                }
            }
            if (alive) {
                ++depth;
                if (depth > maxDepth) alive = false;
            }
            if (alive) {
                V3 dirOut = frame.toLocal(-dir);
                Bsdf B;
                Spec albedo;
                if (isMedium) {
                    B.kind = kMatNull;
                    const bool in = inMedium;
                    Spec sigmaS;
                    evalSpectrum(sc, med.sigmaS, lambdas, sigmaS);
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k)
                        albedo.v[k] = (in && sigmaE.v[k] > 0) ? sigmaS.v[k] / sigmaE.v[k] : 0.0f;
                } else {
                    makeBsdfK<KB>(sc, mat, lambdas, wlSelected, B);
                }
                BsdfQuery q{dirOut, frame.toLocal(gn), sel};
                const bool nonDelta = isMedium || bsdfHasNonDelta(KB);
                if (nonDelta && (sc.numLights > 0 || sc.envPresent)) {
                    int li;
                    float lightProb;
                    int kind = selectLight3(sc, rng.next(), &li, &lightProb);
                    float lu0 = rng.next(), lu1 = rng.next();
                    V3 lp, lgn;
                    Spec M;
                    float areaPdf, edfVal, dist2;
                    bool lAtInf = false;
                    V3 shadowDir;
                    if (kind == 0) {
                        const DevPrim lpr = sc.prims[sc.lightPrims[li]];
                        float su = sqrtf(lu0);
                        float b0 = 1.0f - su, b1 = lu1 * su, b2 = 1.0f - b0 - b1;
                        float4 p0 = sc.vpos[lpr.v0], p1 = sc.vpos[lpr.v1], p2 = sc.vpos[lpr.v2];
                        lp = rn_bary(b0, V3{p0.x, p0.y, p0.z}, b1, V3{p1.x, p1.y, p1.z}, b2, V3{p2.x, p2.y, p2.z});
                        float4 n0 = sc.vnrm[lpr.v0], n1 = sc.vnrm[lpr.v1], n2 = sc.vnrm[lpr.v2];
                        V3 lz = normalize(b0 * V3{n0.x, n0.y, n0.z} + b1 * V3{n1.x, n1.y, n1.z} + b2 * V3{n2.x, n2.y, n2.z});
                        lgn = V3{lpr.ngx, lpr.ngy, lpr.ngz};
                        areaPdf = lpr.invArea;
                        evalSpectrum(sc, sc.materials[lpr.material].emit, lambdas, M);
                        V3 diff = lp - P;
                        dist2 = sqLength(diff);
                        shadowDir = diff * (1.0f / sqrtf(dist2));
                        edfVal = dot(lz, -shadowDir) > 0.0f ? kInvPiF : 0.0f;
                    } else {
                        float uvPdf, topPdf;
                        uint32_t row, col;
                        float d1 = sampleAlias(sc.envTopAlias, sc.envTopPDF, sc.envMapH, lu1, &topPdf, &row);
                        float d0 = sampleAlias(sc.envRowAlias + (size_t)row * sc.envMapW,
                                               sc.envRowPDF + (size_t)row * sc.envMapW, sc.envMapW, lu0, &uvPdf, &col);
                        uvPdf *= topPdf;
                        float phi = d0 * twoPi, theta = d1 * kPiF;
                        float sph, cph, sth, cth;
                        sincosf(phi, &sph, &cph);
                        sincosf(theta, &sth, &cth);
                        lp = V3{-sph * sth, cth, cph * sth};
                        lgn = -lp;
                        lAtInf = true;
                        areaPdf = uvPdf / (2.0f * kPiF * kPiF * sth);
                        envRadiance(sc, phi / twoPi, theta / kPiF, lambdas, M);
                        edfVal = 1.0f;
                        shadowDir = normalize(lp);
                        dist2 = 1.0f;
                    }
                    float cosLight = absDot(-shadowDir, lgn);
                    float cosInter = isMedium ? 1.0f : absDot(shadowDir, gn);
                    float lightPdf = lightProb * areaPdf;
                    V3 sdl = frame.toLocal(shadowDir);
                    Spec fv;
                    float apdf;
                    if (isMedium) {
                        float ph = hgValue(med.g, sdl.z);
#pragma unroll
                        for (int k = 0; k < kNumLambda; ++k) fv.v[k] = albedo.v[k] * ph;
                        apdf = ph;
                    } else {
                        bsdfEval<KB>(B, q, sdl, fv);
                        apdf = bsdfPdf<KB>(B, q, sdl);
                    }
                    float abdfPdf = apdf * cosLight / dist2;
                    float mis = 1.0f;
                    if (!isinf(areaPdf)) mis = (lightPdf * lightPdf) / (lightPdf * lightPdf + abdfPdf * abdfPdf);
                    float G = cosInter * cosLight / dist2;
                    float scale = G * mis / lightPdf;
                    Spec c;
                    bool nz = false;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) {
                        c.v[k] = ((alpha.v[k] * (M.v[k] * edfVal)) * fv.v[k]) * scale;
                        nz |= c.v[k] != 0.0f;
                    }
                    if (nz) {
                        storeSpec(ws.shContrib, p, c);
                        float tmax;
                        V3 sdir;
                        if (lAtInf) {
                            sdir = shadowDir;
                            tmax = 3.402823466e+38f;
                        } else {
                            V3 dd = lp - P;
                            float dist = length(dd);
                            sdir = dd * (1.0f / dist);
                            tmax = dist * (1 - kRayEpsilon);
                        }
                        ws.shRay[2 * (size_t)p] = make_float4(P.x, P.y, P.z, kRayEpsilon);
                        ws.shRay[2 * (size_t)p + 1] = make_float4(sdir.x, sdir.y, sdir.z, tmax);
                        shadow = true;
                    }
                }
                // Sample the next direction (VolumetricBSDF::sample or BSDF::sample).
                BsdfSample bs;
                Spec fs;
                if (isMedium) {
                    float u0 = rng.next(), u1 = rng.next();
                    float pdf;
                    bs.dir = hgSample(med.g, u0, u1, &pdf);
                    bs.pdf = pdf;
                    bs.type = kDirLowFreq | kDirReflection | kDirTransmission;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) fs.v[k] = albedo.v[k] * pdf;
                } else {
                    float uc = rng.next(), u0 = rng.next(), u1 = rng.next();
                    bsdfSample<KB>(B, q, uc, u0, u1, &bs, fs);
                }
                if (bs.pdf == 0.0f || specIsZero(fs)) {
                    alive = false;
                } else {
                    if ((bs.type & kDirDispersive) && !wlSelected) {
                        bs.pdf /= kNumLambda;
                        wlSelected = true;
                    }
                    V3 nd = frame.fromLocal(bs.dir);
                    float cg = isMedium ? 1.0f : absDot(nd, gn);
                    float r = 1.0f / bs.pdf;
#pragma unroll
                    for (int k = 0; k < kNumLambda; ++k) alpha.v[k] *= (fs.v[k] * cg) * r;
                    ws.ray[2 * (size_t)p] = make_float4(P.x, P.y, P.z, kRayEpsilon);
                    ws.ray[2 * (size_t)p + 1] = make_float4(nd.x, nd.y, nd.z, inf);
                    ws.ps[p].prevPdf = bs.pdf;
                    info = (uint32_t)sel | (wlSelected ? kInfoWlSelected : 0u) |
                           (dirIsDelta(bs.type) ? kInfoPrevDelta : 0u) | (depth << kInfoDepthShift);
                    ws.ps[p].info = info;
                    storeSpec(ws.alpha, p, alpha);
                    extend = true;
                }
            }
            if (!extend) {
                // keep the wavelength-selection flag for the shadow kernel
                ws.ps[p].info = (uint32_t)sel | (wlSelected ? kInfoWlSelected : 0u) | (depth << kInfoDepthShift);
            }
            ws.ps[p].rngCounter = rng.counter;
        }
        queuePush(shQueue, shCount, p, active && shadow);
        queuePush(outQueue, outCount, p, active && extend);
    }
}

// Shadow rays of the volumetric integrator (Scene::testVisibility,
// Scene.cpp:114-135): occlusion by surfaces here; unoccluded rays that may
// cross the medium go to a second queue for their spectral transmittance.
__global__ void __launch_bounds__(256, SLRGPU_TRACE_MIN_BLOCKS) kShadowVol(DevScene sc, WaveState ws,
                                                                         const uint32_t* __restrict__ queue,
                                                                         const uint32_t* __restrict__ count,
                                                                         uint32_t* cursor, uint32_t* medQueue,
                                                                         uint32_t* medCount) {
    const uint32_t n = *count;
#if SLRGPU_TRACE_REFILL
    if (sc.watertight) shadowRefill<false, true, true>(sc, ws, queue, n, cursor, nullptr, medQueue, medCount);
    else shadowRefill<false, false, true>(sc, ws, queue, n, cursor, nullptr, medQueue, medCount);
#else
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool pushMedium = false;
        uint32_t p = 0;
        if (i < n) {
            p = queue[i];
            float4 o = ws.shRay[2 * (size_t)p], d = ws.shRay[2 * (size_t)p + 1];
            if (!traceAny(sc, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w)) {
                if (sc.medium.present) {
                    pushMedium = true;
                } else {
                    Spec c;
                    loadSpec(ws.shContrib, p, c);
                    addSpec(ws.L, p, c);
                }
            }
        }
        queuePush(medQueue, medCount, p, pushMedium);
    }
#endif
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ws.stats[1], (unsigned long long)n);
}

// Medium transmittance of the unoccluded shadow rays: one ratio-tracking walk
// per (ray, wavelength).  The walks of a warp take different numbers of
// steps, so each lane runs its walk one tentative collision at a time and
// takes the next (ray, wavelength) as soon as its own walk ends; the warp
// stays full until the queue runs dry.  Each wavelength draws from its own
// counter range of the ray's per-bounce random stream.
#ifndef SLRGPU_MEDIUM_MIN_BLOCKS
#define SLRGPU_MEDIUM_MIN_BLOCKS 4     // 64 registers; measured best of 2, 3, 4
#endif
__global__ void __launch_bounds__(256, SLRGPU_MEDIUM_MIN_BLOCKS) kShadowVolMedium(DevScene sc, WaveState ws,
                                                                                  const uint32_t* __restrict__ queue,
                                 const uint32_t* __restrict__ count, uint32_t* take, uint32_t bounce) {
    const uint32_t n = *count * kNumLambda;
    uint32_t poolNext = 0, poolEnd = 0;
    TrWalk q;
    uint32_t item = 0;
    bool walking = false, exhausted = false;
    for (;;) {
        // lanes without a walk take items until theirs needs steps
        for (;;) {
            const bool need = !walking && !exhausted;
            if (!__any_sync(0xffffffffu, need)) break;
            const uint32_t it = trTake(need, take, poolNext, poolEnd);
            if (!need) continue;
            if (it >= n) {
                exhausted = true;
                continue;
            }
            item = it;
            const uint32_t p = queue[item / kNumLambda];
            const int wl = (int)(item % kNumLambda);
            const float4 o = ws.shRay[2 * (size_t)p], d = ws.shRay[2 * (size_t)p + 1];
            const uint32_t info = ws.ps[p].info;
            const int sel = (int)(info & kInfoSelMask);
            const bool wlSelected = (info & kInfoWlSelected) != 0;
            // this thread's wavelength only, with the shading kernel's arithmetic
            const float sig = evalSpectrumAt(sc, sc.medium.sigmaE, lambdaAt(wl, ws.ps[p].wlOffset));
            const Rng rng{mix64(loadKey(ws, p) ^ (0x9e3779b97f4a7c15ull * (bounce + 1))), (uint32_t)wl << 24};
            walking = trBegin(sc.medium, q, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, o.w, d.w, sig,
                              !wlSelected || wl == sel, rng);
            if (!walking && q.T != 0.0f) {
                const size_t k = (size_t)p * kNumLambda + wl;
                ws.L[k] += q.T * ws.shContrib[k];
            }
        }
        if (!__any_sync(0xffffffffu, walking)) break;
        if (walking) {
            walking = trStep(sc.medium, q);
            if (!walking && q.T != 0.0f) {
                const size_t k = (size_t)queue[item / kNumLambda] * kNumLambda + item % kNumLambda;
                ws.L[k] += q.T * ws.shContrib[k];
            }
        }
    }
}

// Adds the wave's paths to the film: C = L * weight, dropped when not finite
// (PTRenderer.cpp:129-138); binning and compensated sum of
// SpectrumStorage::add (spectrum_types.h:716-739, CompensatedSum.h:16-33).
__global__ void kAccumulate(WaveState ws, const __grid_constant__ WaveParams wpArg,
                            const WaveParams* __restrict__ wpDev) {
    const WaveParams &wp = wpDev ? *wpDev : wpArg;
    const float recBinWidth = kNumLambda / (kWavelengthHigh - kWavelengthLow);
    for (uint32_t fp = blockIdx.x * blockDim.x + threadIdx.x; fp < wp.filmPixels; fp += gridDim.x * blockDim.x) {
        uint32_t k = 0;
        while (k + 1 < wp.numSegments && fp >= wp.seg[k + 1].filmBegin) ++k;
        const WaveSegment &sg = wp.seg[k];
        const uint32_t P = sg.width * sg.height;
        const uint32_t pix = fp - sg.filmBegin;
        float sum[kNumLambda], comp[kNumLambda];
#pragma unroll
        for (int b = 0; b < kNumLambda; ++b) {
            sum[b] = sg.filmSum[(size_t)b * P + pix];
            comp[b] = sg.filmComp[(size_t)b * P + pix];
        }
        unsigned long long dropped = 0;
        // Grid positions clamped into this pixel: itself, plus the overhang
        // of the last column / row.
        const uint32_t x = pix % sg.width, y = pix / sg.width;
        const uint32_t xEnd = x + 1 == sg.width ? sg.gridW : x + 1;
        const uint32_t yEnd = y + 1 == sg.height ? sg.gridH : y + 1;
        for (uint32_t s = 0; s < sg.samples; ++s)
        for (uint32_t gy = y; gy < yEnd; ++gy)
        for (uint32_t gx = x; gx < xEnd; ++gx) {
            const uint32_t p = sg.pathBegin + s * sg.gridPositions + gy * sg.gridW + gx;
            float w = ws.ps[p].camWeight;
            Spec Lp;
            loadSpec(ws.L, p, Lp);
            float c[kNumLambda];
            bool finite = true;
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) {
                c[i] = Lp.v[i] * w;
                finite &= isfinite(c[i]);
            }
            if (!finite) { ++dropped; continue; }
            float wlOff = ws.ps[p].wlOffset;
            float addend[kNumLambda];
            // Wavelength i of a path falls in film bin i unless rounding moves
            // it across a bin edge; then every bin sums its wavelengths in
            // order.  0 + x keeps the sign of zero the summing loop gives.
            bool own = true;
            uint32_t bins[kNumLambda];
#pragma unroll
            for (int i = 0; i < kNumLambda; ++i) {
                float lam = lambdaAt(i, wlOff);
                float f = __fmul_rn(divRange(__fsub_rn(lam, kWavelengthLow)), (float)kNumLambda);
                bins[i] = min((uint32_t)f, (uint32_t)(kNumLambda - 1));
                own &= bins[i] == (uint32_t)i;
            }
            if (own) {
#pragma unroll
                for (int b = 0; b < kNumLambda; ++b) addend[b] = __fadd_rn(0.0f, c[b] * recBinWidth);
            } else {
#pragma unroll
                for (int b = 0; b < kNumLambda; ++b) addend[b] = 0.0f;
#pragma unroll
                for (int i = 0; i < kNumLambda; ++i) {
#pragma unroll
                    for (int b = 0; b < kNumLambda; ++b)
                        if (b == (int)bins[i]) addend[b] += c[i] * recBinWidth;
                }
            }
#pragma unroll
            for (int b = 0; b < kNumLambda; ++b) {
                float cin = __fsub_rn(addend[b], comp[b]);
                float st = __fadd_rn(sum[b], cin);
                comp[b] = __fsub_rn(__fsub_rn(st, sum[b]), cin);
                sum[b] = st;
            }
        }
#pragma unroll
        for (int b = 0; b < kNumLambda; ++b) {
            sg.filmSum[(size_t)b * P + pix] = sum[b];
            sg.filmComp[(size_t)b * P + pix] = comp[b];
        }
        if (dropped) {
            atomicAdd(&ws.stats[2], dropped);
            if (sg.dropped) atomicAdd(sg.dropped, dropped);
        }
    }
}

// Film layout conversion [16][P] -> [P][16].
__global__ void kFilmToPixelMajor(const float* __restrict__ src, float* __restrict__ dst, uint32_t P) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P * kNumLambda; i += gridDim.x * blockDim.x) {
        uint32_t pix = i / kNumLambda, b = i % kNumLambda;
        dst[i] = src[(size_t)b * P + pix];
    }
}

// Ray queries (slrgpu_trace_rays): each warp takes the rays of its own
// contiguous range, and lanes whose walk has ended take the range's next rays
// while the others go on walking (the refill of the wave kernels, with the
// warp's cursor in registers instead of a counter in memory).
template <bool WT, bool ANY>
__device__ __forceinline__ void traceQueries(const DevScene &sc, const float4* __restrict__ rays, uint32_t n,
                                             uint32_t* prim, float* t, float* b1, float* b2) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t chunk = ((uint64_t)n + warps - 1) / warps;
    const uint64_t first = (uint64_t)warp * chunk;
    uint32_t cursor = first < n ? (uint32_t)first : n;
    const uint32_t end = first + chunk < n ? (uint32_t)(first + chunk) : n;
    StackEntry cstack[ANY ? 1 : kTraceStack];
    uint32_t astack[ANY ? kTraceStack : 1];
    ClosestWalk<WT> cw;
    AnyWalk<WT> aw;
    uint32_t i = 0;
    bool live = false;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !live);
        bool fin = false;
        if (cursor < end && (uint32_t)__popc(idle) >= SLRGPU_QUERY_REFILL_LANES) {
            if (!live) {
                const uint32_t k = cursor + (uint32_t)__popc(idle & ((1u << lane) - 1));
                if (k < end) {
                    i = k;
                    const float4 o = rays[2 * (size_t)i], d = rays[2 * (size_t)i + 1];
                    const V3 org = V3{o.x, o.y, o.z}, dir = V3{d.x, d.y, d.z};
                    fin = ANY ? aw.begin(sc, org, dir, o.w, d.w) : cw.begin(sc, org, dir, o.w, d.w);
                    live = true;
                }
            }
            cursor = end - cursor > (uint32_t)__popc(idle) ? cursor + (uint32_t)__popc(idle) : end;
        }
        if (live && !fin)
            fin = ANY ? aw.advance(sc, astack, SLRGPU_TRACE_REFILL_VISITS)
                      : cw.advance(sc, cstack, SLRGPU_TRACE_REFILL_VISITS);
        if (live && fin) {
            if (ANY) {
                prim[i] = aw.occluded ? 1u : 0u;
            } else {
                prim[i] = cw.hit.prim;
                if (t) t[i] = cw.hit.t;
                if (b1) b1[i] = cw.hit.b1;
                if (b2) b2[i] = cw.hit.b2;
            }
            live = false;
        }
        if (cursor >= end && !__any_sync(0xffffffffu, live)) return;
    }
}

__global__ void __launch_bounds__(256, SLRGPU_TRACE_MIN_BLOCKS) kTrace(DevScene sc, const float* __restrict__ rays,
                                                                     uint32_t n, int anyHit, uint32_t* prim, float* t,
                                                                     float* b1, float* b2) {
    const float4* r = reinterpret_cast<const float4*>(rays);
    if (anyHit) {
        if (sc.watertight) traceQueries<true, true>(sc, r, n, prim, t, b1, b2);
        else traceQueries<false, true>(sc, r, n, prim, t, b1, b2);
    } else {
        if (sc.watertight) traceQueries<true, false>(sc, r, n, prim, t, b1, b2);
        else traceQueries<false, false>(sc, r, n, prim, t, b1, b2);
    }
}

// BSDF queries at fixed inputs (16 floats in, 40 out per query; the layout of
// slrgpu_bsdf_query in include/slrgpu.h).
// Replays a given stream of 32-bit values as uniforms (then 0x80000000), with
// the reference's 23-bit conversion, so that medium queries draw exactly the
// uniforms a test hands them.
struct ReplayRng {
    const uint32_t* vals;
    uint32_t n;
    uint32_t counter;
    __device__ float next() {
        uint32_t v = counter < n ? vals[counter] : 0x80000000u;
        ++counter;
        return __uint_as_float((v >> 9) | 0x3f800000u) - 1.0f;
    }
};

// One medium query per thread: on a segment inside the medium, mode 0
// free-path sampling (DensityGridMediumDistribution::interact), 1
// transmittance (::evaluateTransmittance), 2 extinction coefficient at a
// normalised position (::evaluateExtinctionCoefficient); on any segment, 3
// and 4 the same through the boundary walk of MediumObjectAggregate.
// Layouts as slrgpu_medium_query.
__global__ void kMediumQuery(DevScene sc, int mode, uint32_t n, const float* __restrict__ rays,
                             const float* __restrict__ lambdasIn, const int* __restrict__ selIn,
                             const uint32_t* __restrict__ vals, uint32_t nvals, float* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* r = rays + 8 * (size_t)i;
        float* o = out + 24 * (size_t)i;
        float lambdas[kNumLambda];
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) lambdas[k] = lambdasIn[16 * (size_t)i + k];
        const int sel = selIn[i] & 0xff;
        const bool wlSelected = (selIn[i] & 0x100) != 0;
        Spec sigmaE;
        evalSpectrum(sc, sc.medium.sigmaE, lambdas, sigmaE);
        ReplayRng rng{vals + (size_t)nvals * i, nvals, 0};
        V3 org = V3{r[0], r[1], r[2]}, dir = V3{r[4], r[5], r[6]};
        Spec v = specConst(0.0f);
        float hit = 0.0f, dist = 0.0f;
        V3 param = V3{0.0f, 0.0f, 0.0f};
        if (mode == 0) {
            float t;
            V3 pr;
            if (mediumInteractSegment(sc.medium, org, dir, r[3], r[7], sigmaE, sel, wlSelected, rng, &t, &pr, v)) {
                hit = 1.0f;
                dist = t;
                param = pr;
            }
        } else if (mode == 1) {
            mediumTransmittanceSegment(sc.medium, org, dir, r[3], r[7], sigmaE, sel, wlSelected, rng, v);
        } else if (mode == 3) {
            float t;
            V3 pr;
            if (mediumInteract(sc.medium, org, dir, r[3], r[7], sigmaE, sel, wlSelected, rng, &t, &pr, v)) {
                hit = 1.0f;
                dist = t;
                param = pr;
            }
        } else if (mode == 4) {
            mediumTransmittance(sc.medium, org, dir, r[3], r[7], sigmaE, sel, wlSelected, rng, v);
        } else {
            float d = mediumDensity(sc.medium, org);
#pragma unroll
            for (int k = 0; k < kNumLambda; ++k) v.v[k] = d * sigmaE.v[k];
        }
        o[0] = hit;
        o[1] = dist;
        o[2] = param.x;
        o[3] = param.y;
        o[4] = param.z;
        o[5] = (float)rng.counter;
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) o[6 + k] = v.v[k];
        o[22] = 0.0f;
        o[23] = 0.0f;
    }
}

__global__ void kBsdfQuery(Bsdf B, const float* __restrict__ q, uint32_t n, float* __restrict__ o) {
    prepareIorPairs(B);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* qi = q + 16 * (size_t)i;
        float* oi = o + 40 * (size_t)i;
        BsdfQuery bq{V3{qi[0], qi[1], qi[2]}, V3{qi[3], qi[4], qi[5]}, (int)qi[6]};
        BsdfSample bs;
        Spec fs;
        bsdfSample(B, bq, qi[8], qi[9], qi[10], &bs, fs);
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) oi[k] = bs.pdf == 0.0f ? 0.0f : fs.v[k];
        oi[16] = bs.dir.x; oi[17] = bs.dir.y; oi[18] = bs.dir.z;
        oi[19] = bs.pdf;
        oi[20] = (float)bs.type;
        V3 ed = V3{qi[11], qi[12], qi[13]};
        Spec fe;
        bsdfEval(B, bq, ed, fe);
#pragma unroll
        for (int k = 0; k < kNumLambda; ++k) oi[21 + k] = fe.v[k];
        oi[37] = bsdfPdf(B, bq, ed);
        oi[38] = 0.0f;
        oi[39] = 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {
// Each scene array gets a device allocation and a pinned host mirror; the
// mirror is what slrgpu_scene_reupload copies from.
template <typename T>
int upload(DeviceBuffers &db, const std::vector<T> &v, const T** out) {
    *out = nullptr;
    if (v.empty()) return SLRGPU_OK;
    const size_t bytes = v.size() * sizeof(T);
    void* p = nullptr;
    void* h = nullptr;
    CUDA_TRY(cudaMalloc(&p, bytes));
    db.allocs.push_back(p);
    CUDA_TRY(cudaMallocHost(&h, bytes));
    db.pinned.push_back(h);
    db.sizes.push_back(bytes);
    std::memcpy(h, v.data(), bytes);
    CUDA_TRY(cudaMemcpy(p, h, bytes, cudaMemcpyHostToDevice));
    *out = (const T*)p;
    return SLRGPU_OK;
}

template <typename T>
T* allocDev(std::vector<void*> &allocs, size_t n, cudaError_t* err) {
    void* p = nullptr;
    *err = cudaMalloc(&p, n * sizeof(T) + 16);
    if (*err != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (T*)p;
}
}  // namespace

void DeviceBuffers::release() {
    for (void* p : allocs) cudaFree(p);
    for (void* p : pinned) cudaFreeHost(p);
    allocs.clear();
    pinned.clear();
    sizes.clear();
}

int reuploadScene(DeviceScene* ds, uint64_t* bytes, cudaStream_t stream) {
    uint64_t total = 0;
    for (size_t i = 0; i < ds->buffers.allocs.size(); ++i) {
        CUDA_TRY(cudaMemcpyAsync(ds->buffers.allocs[i], ds->buffers.pinned[i], ds->buffers.sizes[i],
                                 cudaMemcpyHostToDevice, stream));
        total += ds->buffers.sizes[i];
    }
    if (bytes) *bytes = total;
    return SLRGPU_OK;
}

int uploadScene(const HostScene &hs, const BuiltScene &bs, DeviceScene* ds) {
    ds->buffers.release();
    DevScene &sc = ds->sc;
    std::memset(&sc, 0, sizeof(sc));
    DeviceBuffers &db = ds->buffers;
    int rc;
#define UP(vec, field) if ((rc = upload(db, vec, &sc.field)) != SLRGPU_OK) return rc
    UP(bs.wide.nodes, nodes);
    UP(bs.wide.frags, frags);
    {
        // Vertices of every fragment as given, for the watertight test.
        std::vector<float4> wv(3 * bs.wide.frags.size());
        for (size_t i = 0; i < bs.wide.frags.size(); ++i) {
            const uint32_t prim = bs.wide.frags[i].prim;
            const DevPrim &pr = bs.prims[prim];
            const float4 a = bs.vpos[pr.v0], b = bs.vpos[pr.v1], c = bs.vpos[pr.v2];
            wv[3 * i] = float4{a.x, a.y, a.z, 0.0f};
            std::memcpy(&wv[3 * i].w, &prim, sizeof(prim));
            wv[3 * i + 1] = float4{b.x, b.y, b.z, 0.0f};
            wv[3 * i + 2] = float4{c.x, c.y, c.z, 0.0f};
        }
        UP(wv, wtVerts);
    }
    UP(bs.prims, prims);
    UP(bs.vpos, vpos);
    UP(bs.vnrm, vnrm);
    UP(bs.vtan, vtan);
    UP(hs.materials, materials);
    static std::atomic<uint64_t> nextUid{1};
    ds->uid = nextUid.fetch_add(1);
    ds->kindMask = 0;
    for (const DevMaterial &m : hs.materials)
        if (m.kind < kMatNull) ds->kindMask |= 1u << m.kind;
    UP(hs.spectra, spectra);
    UP(hs.specValues, specValues);
    std::vector<float> ups(upsSpectra(), upsSpectra() + (size_t)upsNumPoints() * kUpsNumSamples);
    UP(ups, upsSpectra);
    UP(bs.lightPrims, lightPrims);
    UP(bs.lightCDF, lightCDF);
    UP(bs.lightAlias, lightAlias);
    UP(bs.lightPMF, lightPMF);
    if (hs.envPresent) {
        UP(bs.env.texels, envTexels);
        UP(bs.env.rowPDF, envRowPDF);
        UP(bs.env.rowCDF, envRowCDF);
        UP(bs.env.topPDF, envTopPDF);
        UP(bs.env.topCDF, envTopCDF);
        UP(bs.env.rowAlias, envRowAlias);
        UP(bs.env.topAlias, envTopAlias);
    }
    if (hs.medium.present) {
        DevMedium &m = sc.medium;
        UP(hs.medium.density, medium.density);
        UP(bs.superVoxels.corners, medium.superVoxels);
        UP(bs.superVoxels.maxDiff, medium.maxDiff);
        m.present = 1;
        m.nx = hs.medium.nx; m.ny = hs.medium.ny; m.nz = hs.medium.nz;
        m.svx = bs.superVoxels.svx; m.svy = bs.superVoxels.svy; m.svz = bs.superVoxels.svz;
        for (int k = 0; k < 3; ++k) {
            m.bmin[k] = hs.medium.bmin[k];
            m.bmax[k] = hs.medium.bmax[k];
            m.svWidth[k] = bs.superVoxels.width[k];
            m.invSvWidth[k] = 1.0f / m.svWidth[k];
            m.invExtent[k] = 1.0f / (m.bmax[k] - m.bmin[k]);
        }
        m.sigmaS = hs.medium.sigmaS;
        m.sigmaE = hs.medium.sigmaE;
        m.g = hs.medium.g;
        m.importance = 0.0f;   // density media do not emit
    }
#undef UP
    sc.numPrims = (uint32_t)bs.prims.size();
    sc.numNodes = (uint32_t)bs.wide.nodes.size();
    sc.numLights = (uint32_t)bs.lightPrims.size();
    sc.surfImportance = (float)bs.lightPrims.size();
    sc.envPresent = hs.envPresent ? 1u : 0u;
    sc.envImportance = hs.envPresent ? 1.0f : 0.0f;
    sc.envWidth = bs.env.width;
    sc.envHeight = bs.env.height;
    sc.envScale = bs.env.scale;
    sc.envMapW = bs.env.mapW;
    sc.envMapH = bs.env.mapH;
    sc.worldRadius = bs.worldRadius;
    sc.worldDiscArea = bs.worldDiscArea;
    for (int k = 0; k < 3; ++k) sc.worldCenter[k] = bs.worldCenter[k];
    sc.camera = bs.camera;
    return SLRGPU_OK;
}

int RenderEngine::ensure(uint32_t N, uint32_t maxDepth) {
    if (N <= capacity && maxDepth <= depthCapacity && ws) return SLRGPU_OK;
    release();
    cudaError_t e;
    WaveState* w = new WaveState();
    std::memset(w, 0, sizeof(*w));
    w->N = N;
    w->ray = allocDev<float4>(allocs, 2ull * N, &e); if (!w->ray) goto fail;
    w->hit = allocDev<float4>(allocs, N, &e); if (!w->hit) goto fail;
    w->alpha = allocDev<float>(allocs, (size_t)N * kNumLambda, &e); if (!w->alpha) goto fail;
    w->L = allocDev<float>(allocs, (size_t)N * kNumLambda, &e); if (!w->L) goto fail;
    w->ps = allocDev<PathScalars>(allocs, N, &e); if (!w->ps) goto fail;
    w->shRay = allocDev<float4>(allocs, 2ull * N, &e); if (!w->shRay) goto fail;
    w->shContrib = allocDev<float>(allocs, (size_t)N * kNumLambda, &e); if (!w->shContrib) goto fail;
    w->queue[0] = allocDev<uint32_t>(allocs, N, &e); if (!w->queue[0]) goto fail;
    w->queue[1] = allocDev<uint32_t>(allocs, N, &e); if (!w->queue[1]) goto fail;
    w->shadowQueue = allocDev<uint32_t>(allocs, N, &e); if (!w->shadowQueue) goto fail;
    w->classQueue = allocDev<uint32_t>(allocs, (size_t)N * kNumClassQueues, &e); if (!w->classQueue) goto fail;
    w->counters = allocDev<uint32_t>(allocs, (size_t)kCtrStride * (maxDepth + 2), &e); if (!w->counters) goto fail;
    w->stats = allocDev<unsigned long long>(allocs, 4, &e); if (!w->stats) goto fail;
    ws = w;
    capacity = N;
    depthCapacity = maxDepth;
    stateBytes = (uint64_t)N * (2 * 16 + 16 + 2 * 4 * kNumLambda + sizeof(PathScalars) + 2 * 16 + 4 * kNumLambda +
                                3 * 4 + 4 * kNumClassQueues) +
                 4ull * kCtrStride * (maxDepth + 2) + 4 * sizeof(unsigned long long);
    return SLRGPU_OK;
fail:
    delete w;
    release();
    setError(std::string("path state allocation failed: ") + cudaGetErrorString(e));
    return SLRGPU_ERR_OUT_OF_MEMORY;
}

RenderEngine::~RenderEngine() {
    release();
    if (bpt) bptEngineDestroy(bpt);
}

static_assert(kCtrStride >= (int)kQueueCountColumns, "queue-count rows are the first columns of the counter blocks");
int RenderEngine::queueCounts(uint32_t* out, uint32_t capacity, uint32_t* rows) {
    if (!ws) {
        *rows = 0;
        return SLRGPU_OK;
    }
    *rows = depthCapacity + 2;
    const size_t n = (size_t)kQueueCountColumns * (depthCapacity + 2);
    if (capacity < n) {
        setError("capacity below rows x 11 counters");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    CUDA_TRY(cudaMemcpy2D(out, kQueueCountColumns * sizeof(uint32_t), ws->counters, kCtrStride * sizeof(uint32_t),
                          kQueueCountColumns * sizeof(uint32_t), depthCapacity + 2, cudaMemcpyDeviceToHost));
    return SLRGPU_OK;
}

int RenderEngine::ensureFilm(uint32_t P) {
    if (filmPixels >= P) return SLRGPU_OK;
    if (filmSum) cudaFree(filmSum);
    if (filmComp) cudaFree(filmComp);
    if (filmOut) cudaFree(filmOut);
    filmSum = filmComp = filmOut = nullptr;
    filmPixels = 0;
    CUDA_TRY(cudaMalloc(&filmSum, (size_t)P * kNumLambda * sizeof(float)));
    CUDA_TRY(cudaMalloc(&filmComp, (size_t)P * kNumLambda * sizeof(float)));
    CUDA_TRY(cudaMalloc(&filmOut, (size_t)P * kNumLambda * sizeof(float)));
    filmPixels = P;
    return SLRGPU_OK;
}

void RenderEngine::release() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    delete ws;
    ws = nullptr;
    capacity = 0;
    depthCapacity = 0;
    stateBytes = 0;
    if (filmSum) { cudaFree(filmSum); filmSum = nullptr; }
    if (filmComp) { cudaFree(filmComp); filmComp = nullptr; }
    if (filmOut) { cudaFree(filmOut); filmOut = nullptr; }
    filmPixels = 0;
}

static int gridFor(const void* kernel, int block) {
    int dev = 0, sms = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, block, 0);
    return std::max(1, sms * std::max(1, perSM));
}

// Persistent grid sizes (resident blocks per SM x SMs) of the wave kernels,
// computed once per process.
struct WaveGrids {
    int raygen, extend, shadow, accumulate, volInteract, shadowVol, shadowVolMedium, extendSort, shadeMiss;
    int shadeSurf[kNumShadeClasses - 1];
    // the multi-scene instances
    int raygenM, shadowM, extendSortM, shadeMissM;
    int shadeSurfM[kNumShadeClasses - 1];
    int shadeVol[kNumClassQueues - 1];
};
static const WaveGrids &waveGrids(int block) {
    static WaveGrids g;
    static std::once_flag once;
    std::call_once(once, [&]() {
        g.raygen = gridFor((const void*)kRaygen<false>, block);
        g.extend = gridFor((const void*)kExtend, block);
        g.shadow = gridFor((const void*)kShadow<false>, block);
        g.accumulate = gridFor((const void*)kAccumulate, block);
        g.volInteract = gridFor((const void*)kVolInteract, block);
        g.shadeVol[0] = gridFor((const void*)kShadeVol<0>, block);
        g.shadeVol[1] = gridFor((const void*)kShadeVol<1>, block);
        g.shadeVol[2] = gridFor((const void*)kShadeVol<2>, block);
        g.shadeVol[3] = gridFor((const void*)kShadeVol<3>, block);
        g.shadeVol[4] = gridFor((const void*)kShadeVol<4>, block);
        g.shadeVol[5] = gridFor((const void*)kShadeVol<5>, block);
        g.shadeVol[6] = gridFor((const void*)kShadeVol<6>, block);
        g.shadowVol = gridFor((const void*)kShadowVol, block);
        g.shadowVolMedium = gridFor((const void*)kShadowVolMedium, block);
        g.extendSort = gridFor((const void*)kExtendSort<false>, block);
        g.shadeMiss = gridFor((const void*)kShadeMiss<false>, block);
        g.shadeSurf[kMatMatte] = gridFor((const void*)kShadeSurf<kMatMatte, false>, block);
        g.shadeSurf[kMatSpecularReflection] = gridFor((const void*)kShadeSurf<kMatSpecularReflection, false>, block);
        g.shadeSurf[kMatSpecularScattering] = gridFor((const void*)kShadeSurf<kMatSpecularScattering, false>, block);
        g.shadeSurf[kMatGGXReflection] = gridFor((const void*)kShadeSurf<kMatGGXReflection, false>, block);
        g.shadeSurf[kMatGGXScattering] = gridFor((const void*)kShadeSurf<kMatGGXScattering, false>, block);
        g.raygenM = gridFor((const void*)kRaygen<true>, block);
        g.shadowM = gridFor((const void*)kShadow<true>, block);
        g.extendSortM = gridFor((const void*)kExtendSort<true>, block);
        g.shadeMissM = gridFor((const void*)kShadeMiss<true>, block);
        g.shadeSurfM[kMatMatte] = gridFor((const void*)kShadeSurf<kMatMatte, true>, block);
        g.shadeSurfM[kMatSpecularReflection] = gridFor((const void*)kShadeSurf<kMatSpecularReflection, true>, block);
        g.shadeSurfM[kMatSpecularScattering] = gridFor((const void*)kShadeSurf<kMatSpecularScattering, true>, block);
        g.shadeSurfM[kMatGGXReflection] = gridFor((const void*)kShadeSurf<kMatGGXReflection, true>, block);
        g.shadeSurfM[kMatGGXScattering] = gridFor((const void*)kShadeSurf<kMatGGXScattering, true>, block);
    });
    return g;
}

// Optional per-launch timing of the wave kernels by kernel class.  Timing
// stops (and the incomplete mark is dropped) if an event cannot be created or
// recorded; the render itself goes on.
struct LaunchMarks {
    std::vector<cudaEvent_t>* pool = nullptr;   // null: no timing
    cudaStream_t stream = 0;
    struct Mark { int cls; size_t ev; };
    std::vector<Mark> marks;
    size_t used = 0;
    bool pending = false;                       // the last mark still needs its end event
    bool record() {
        if (used == pool->size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return false;
            pool->push_back(e);
        }
        return cudaEventRecord((*pool)[used++], stream) == cudaSuccess;
    }
    void stop() {
        if (pending) marks.pop_back();
        pending = false;
        pool = nullptr;
    }
    void begin(int cls) {
        if (!pool) return;
        marks.push_back(Mark{cls, used});
        pending = true;
        if (!record()) stop();
    }
    void end() {
        if (!pool) return;
        if (!record()) {
            stop();
            return;
        }
        pending = false;
    }
};

// Sample grid and wave size of a render: every position of the tile-padded
// grid is one path per sample index; a wave holds S sample indices.
// Paths in flight per wave when samples_per_wave is 0 (a tuned constant).
#ifndef SLRGPU_WAVE_PATHS
#define SLRGPU_WAVE_PATHS (4u << 20)
#endif

struct WavePlan {
    uint32_t gridW, gridH, gridPositions, filmPixels, S;
};
static WavePlan planWaves(const slrgpu_settings &s, uint32_t autoPaths) {
    WavePlan pl;
    pl.gridW = padToTile(s.width);
    pl.gridH = padToTile(s.height);
    pl.gridPositions = pl.gridW * pl.gridH;
    pl.filmPixels = s.width * s.height;
    uint32_t S = s.samples_per_wave;
    if (S == 0) S = std::max(1u, autoPaths / pl.gridPositions);
    pl.S = std::min(S, s.spp);
    return pl;
}

// One wave: camera rays for every path of the wave's segments, then per
// bounce the extension, shading and shadow kernels over the device-side
// queues, then the film update of every segment.  Stream-ordered; counters,
// queues and path state live in w.  Adds the number of kernel launches to
// *launchCount; returns SLRGPU_OK, or SLRGPU_ERR_CUDA (error text set) when
// the counter reset or a launch was rejected.
// The scenes of a wave of several scenes (surface path tracer only): their
// table in device memory, the union of their material kinds, whether any
// has an environment.
struct WaveSceneTable {
    const DevScene* dev;
    uint32_t kindMask;
    bool env;
};

// One bounce of the surface path tracer: closest hits sorted by shading
// class, the shading kernels of the classes present, the shadow rays.
template <bool MULTI>
static void surfaceBounce(const DevScene &sc, const DevScene* scenes, uint32_t kindMask, bool env, const WaveState &w,
                          uint32_t D, uint32_t* ctr, uint32_t* next, const uint32_t* inQueue, uint32_t* outQueue,
                          cudaStream_t stream, LaunchMarks &lm, uint64_t &launches) {
    const int block = 256;
    const WaveGrids &g = waveGrids(block);
    lm.begin(SLRGPU_KERNEL_EXTEND);
    kExtendSort<MULTI><<<MULTI ? g.extendSortM : g.extendSort, block, 0, stream>>>(sc, w, inQueue, ctr + kCtrExt, ctr,
                                                                                  ctr + kCtrExtTake, D, scenes);
    lm.end();
    ++launches;
    if (env) {
        lm.begin(SLRGPU_KERNEL_SHADE);
        kShadeMiss<MULTI><<<MULTI ? g.shadeMissM : g.shadeMiss, block, 0, stream>>>(
            sc, w, w.classQueue + (size_t)kClassMiss * w.N, ctr + kClassMiss, scenes);
        lm.end();
        ++launches;
    }
    // One kernel per material kind present.
    for (int k = 0; k < kNumShadeClasses - 1; ++k) {
        if (!(kindMask & (1u << k))) continue;
        const uint32_t* cq = w.classQueue + (size_t)k * w.N;
        const int grid = MULTI ? g.shadeSurfM[k] : g.shadeSurf[k];
        lm.begin(SLRGPU_KERNEL_SHADE);
#define SLRGPU_SHADESURF(KK)                                                                                   \
    kShadeSurf<KK, MULTI><<<grid, block, 0, stream>>>(sc, w, D, cq, ctr + k, outQueue, next + kCtrExt, w.shadowQueue, \
                                                      ctr + kCtrShadow, scenes)
        switch (k) {
        case kMatMatte: SLRGPU_SHADESURF(kMatMatte); break;
        case kMatSpecularReflection: SLRGPU_SHADESURF(kMatSpecularReflection); break;
        case kMatSpecularScattering: SLRGPU_SHADESURF(kMatSpecularScattering); break;
        case kMatGGXReflection: SLRGPU_SHADESURF(kMatGGXReflection); break;
        default: SLRGPU_SHADESURF(kMatGGXScattering); break;
        }
#undef SLRGPU_SHADESURF
        lm.end();
        ++launches;
    }
    lm.begin(SLRGPU_KERNEL_SHADOW);
    kShadow<MULTI><<<MULTI ? g.shadowM : g.shadow, block, 0, stream>>>(sc, w, w.shadowQueue, ctr + kCtrShadow,
                                                                       ctr + kCtrShadowTake, scenes);
    lm.end();
    ++launches;
}

static int runWave(const DeviceScene &ds0, const WaveState &w, const WaveParams &wp, uint32_t D, bool volumetric,
                   bool watertight, cudaStream_t stream, LaunchMarks &lm, uint64_t* launchCount,
                   const WaveParams* wpDev = nullptr, const float* rngTape = nullptr,
                   const WaveSceneTable* multi = nullptr) {
    // the scene as the kernels see it, with the triangle test chosen
    struct { DevScene sc; uint32_t kindMask; } ds{ds0.sc, ds0.kindMask};
    ds.sc.watertight = watertight ? 1u : 0u;
    ds.sc.rngTape = rngTape;
    const int block = 256;
    const WaveGrids &g = waveGrids(block);
    uint64_t launches = 0;
    CUDA_TRY(cudaMemsetAsync(w.counters, 0, (size_t)kCtrStride * (D + 2) * sizeof(uint32_t), stream));
    if (multi && volumetric) {
        setError("waves of several scenes are for the surface path tracer");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    lm.begin(SLRGPU_KERNEL_RAYGEN);
    if (multi)
        kRaygen<true><<<g.raygenM, block, 0, stream>>>(ds.sc, w, wp, wpDev, multi->dev, volumetric);
    else
        kRaygen<false><<<g.raygen, block, 0, stream>>>(ds.sc, w, wp, wpDev, nullptr, volumetric);
    lm.end();
    ++launches;
    for (uint32_t b = 0; b <= D; ++b) {
        TraceRange range("bounce %u", b);
        uint32_t* ctr = w.counters + (size_t)kCtrStride * b;
        uint32_t* next = ctr + kCtrStride;
        uint32_t* inQueue = w.queue[b & 1];
        uint32_t* outQueue = w.queue[(b + 1) & 1];
        if (volumetric) {
            lm.begin(SLRGPU_KERNEL_EXTEND);
            kExtend<<<g.extend, block, 0, stream>>>(ds.sc, w, inQueue, ctr + kCtrExt, ctr + kCtrExtTake);
            lm.end();
            // the medium collision (or not), then one shading kernel per
            // vertex class present
            lm.begin(SLRGPU_KERNEL_SHADE);
            kVolInteract<<<g.volInteract, block, 0, stream>>>(ds.sc, w, inQueue, ctr + kCtrExt, ctr);
            lm.end();
            launches += 2;
            for (int k = 0; k < kNumClassQueues - 1; ++k) {
                const bool present = k < kClassMiss ? (ds.kindMask & (1u << k)) != 0
                                                    : (k == kClassMiss ? ds.sc.envPresent != 0 : ds.sc.medium.present != 0);
                if (!present) continue;
                const uint32_t* cq = w.classQueue + (size_t)k * w.N;
                lm.begin(SLRGPU_KERNEL_SHADE);
#define SLRGPU_SHADEVOL(KK)                                                                              \
    kShadeVol<KK><<<g.shadeVol[KK], block, 0, stream>>>(ds.sc, w, D, cq, ctr + k, outQueue, next + kCtrExt, \
                                                        w.shadowQueue, ctr + kCtrShadow)
                switch (k) {
                case 0: SLRGPU_SHADEVOL(0); break;
                case 1: SLRGPU_SHADEVOL(1); break;
                case 2: SLRGPU_SHADEVOL(2); break;
                case 3: SLRGPU_SHADEVOL(3); break;
                case 4: SLRGPU_SHADEVOL(4); break;
                case 5: SLRGPU_SHADEVOL(5); break;
                default: SLRGPU_SHADEVOL(6); break;
                }
#undef SLRGPU_SHADEVOL
                lm.end();
                ++launches;
            }
            // unoccluded shadow rays that cross the medium wait in their own queue
            uint32_t* medQueue = w.classQueue + (size_t)kQueueMedShadow * w.N;
            lm.begin(SLRGPU_KERNEL_SHADOW);
            kShadowVol<<<g.shadowVol, block, 0, stream>>>(ds.sc, w, w.shadowQueue, ctr + kCtrShadow,
                                                          ctr + kCtrShadowTake, medQueue, ctr + kCtrMedShadow);
            lm.end();
            lm.begin(SLRGPU_KERNEL_SHADOW);
            kShadowVolMedium<<<g.shadowVolMedium, block, 0, stream>>>(ds.sc, w, medQueue, ctr + kCtrMedShadow,
                                                                      ctr + kCtrMedTake, b);
            lm.end();
            launches += 2;
            continue;
        }
        if (multi)
            surfaceBounce<true>(ds.sc, multi->dev, multi->kindMask, multi->env, w, D, ctr, next, inQueue, outQueue,
                                stream, lm, launches);
        else
            surfaceBounce<false>(ds.sc, nullptr, ds.kindMask, ds.sc.envPresent != 0, w, D, ctr, next, inQueue,
                                 outQueue, stream, lm, launches);
    }
    lm.begin(SLRGPU_KERNEL_ACCUMULATE);
    kAccumulate<<<g.accumulate, block, 0, stream>>>(w, wp, wpDev);
    lm.end();
    ++launches;
    *launchCount += launches;
    CUDA_TRY(cudaGetLastError());
    return SLRGPU_OK;
}

// The wave loop of one render (slrgpu_render, slrgpu_render_noalloc): waves
// of pl.S sample indices over the whole sample grid, one segment each.
static int runWaves(const DeviceScene &ds, const slrgpu_settings &s, const WavePlan &pl, const WaveState &w,
                    float* filmSum, float* filmComp, cudaStream_t stream, LaunchMarks &lm, uint64_t* launches,
                    const float* rngTape = nullptr) {
    for (uint32_t base = 0; base < s.spp; base += pl.S) {
        TraceRange range("wave: samples %u..%u", s.sample_base + base, s.sample_base + std::min(s.spp, base + pl.S));
        WaveParams wp;
        std::memset(&wp, 0, sizeof(wp));
        WaveSegment &sg = wp.seg[0];
        sg.pathBegin = 0;
        sg.width = s.width;
        sg.height = s.height;
        sg.gridW = pl.gridW;
        sg.gridH = pl.gridH;
        sg.gridPositions = pl.gridPositions;
        sg.sampleBase = s.sample_base + base;
        sg.samples = std::min(pl.S, s.spp - base);
        sg.seed = s.seed;
        sg.filmBegin = 0;
        sg.filmSum = filmSum;
        sg.filmComp = filmComp;
        sg.dropped = nullptr;
        wp.numSegments = 1;
        wp.numPaths = sg.samples * pl.gridPositions;
        wp.filmPixels = s.width * s.height;
        int rc = runWave(ds, w, wp, s.max_depth, s.volumetric != 0, (s.flags & SLRGPU_FLAG_WATERTIGHT) != 0,
                         stream, lm, launches, nullptr, rngTape);
        if (rc != SLRGPU_OK) return rc;
    }
    return SLRGPU_OK;
}

int RenderEngine::render(const DeviceScene &ds, const slrgpu_settings &s, float* film, bool filmOnDevice,
                         slrgpu_render_stats* stats, cudaStream_t stream, float* filmState, const float* rngTape) {
    auto t0 = std::chrono::steady_clock::now();
    TraceRange range("render %ux%u, %u spp, depth %u", s.width, s.height, s.spp, s.max_depth);
    if (s.spp == 0) {
        setError("width, height and spp must be positive");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (int rc = checkImageSize(s.width, s.height)) return rc;
    if (s.max_depth > 1000) {
        setError("max_depth must be <= 1000");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const bool bidir = (s.flags & SLRGPU_FLAG_BPT) != 0;
    const WavePlan pl = planWaves(s, SLRGPU_WAVE_PATHS);
    const uint32_t P = pl.filmPixels;
    if (!bidir) {
        const uint64_t Nwant = (uint64_t)pl.S * pl.gridPositions;
        if (Nwant > 0x7fffffffull) {
            setError("paths per wave exceed 2^31");
            return SLRGPU_ERR_INVALID_ARGUMENT;
        }
        int rc = ensure((uint32_t)Nwant, s.max_depth);
        if (rc != SLRGPU_OK) return rc;
    } else if (!bpt) {
        bpt = bptEngineCreate();
    }
    if (filmState && bidir) {
        setError("continuing a film is supported for the path tracers only");
        return SLRGPU_ERR_UNSUPPORTED;
    }
    int rc = ensureFilm(P);
    if (rc != SLRGPU_OK) return rc;
    const size_t planeBytes = (size_t)P * kNumLambda * sizeof(float);
    if (filmState) {
        // continue the compensated sums of earlier sample ranges: a film
        // rendered in consecutive ranges equals the one-call film bit for bit
        CUDA_TRY(cudaMemcpyAsync(filmSum, filmState, planeBytes, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(filmComp, filmState + (size_t)P * kNumLambda, planeBytes, cudaMemcpyHostToDevice,
                                 stream));
    } else {
        CUDA_TRY(cudaMemsetAsync(filmSum, 0, planeBytes, stream));
        CUDA_TRY(cudaMemsetAsync(filmComp, 0, planeBytes, stream));
    }
    if (!bidir) CUDA_TRY(cudaMemsetAsync(ws->stats, 0, 4 * sizeof(unsigned long long), stream));
    // the render's start and end events, destroyed on every return path
    struct EventPair {
        cudaEvent_t e[2] = {nullptr, nullptr};
        ~EventPair() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } events;
    CUDA_TRY(cudaEventCreate(&events.e[0]));
    CUDA_TRY(cudaEventCreate(&events.e[1]));
    cudaEvent_t e0 = events.e[0], e1 = events.e[1];
    CUDA_TRY(cudaEventRecord(e0, stream));
    const bool profile = (s.flags & SLRGPU_FLAG_PROFILE_KERNELS) != 0;
    LaunchMarks lm;
    lm.stream = stream;
    if (profile) lm.pool = &eventPool;
    uint64_t launches = 0;
    slrgpu_render_stats bst;
    std::memset(&bst, 0, sizeof(bst));
    if (bidir) {
        rc = renderBpt(*bpt, ds, s, filmSum, filmComp, stream, &launches, profile ? &eventPool : nullptr, &bst);
        if (rc != SLRGPU_OK) return rc;
    } else {
        rc = runWaves(ds, s, pl, *ws, filmSum, filmComp, stream, lm, &launches, rngTape);
        if (rc != SLRGPU_OK) return rc;
    }
    CUDA_TRY(cudaGetLastError());
    float* dst = filmOnDevice && film ? film : filmOut;
    kFilmToPixelMajor<<<waveGrids(256).accumulate, 256, 0, stream>>>(filmSum, dst, P);
    ++launches;
    CUDA_TRY(cudaEventRecord(e1, stream));
    if (!filmOnDevice && film)
        CUDA_TRY(cudaMemcpyAsync(film, filmOut, planeBytes, cudaMemcpyDeviceToHost, stream));
    if (filmState) {
        CUDA_TRY(cudaMemcpyAsync(filmState, filmSum, planeBytes, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaMemcpyAsync(filmState + (size_t)P * kNumLambda, filmComp, planeBytes, cudaMemcpyDeviceToHost,
                                 stream));
    }
    unsigned long long hstats[4] = {0, 0, 0, 0};
    if (!bidir) CUDA_TRY(cudaMemcpyAsync(hstats, ws->stats, sizeof(hstats), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        if (bidir) {
            std::memcpy(stats->kernel_ms, bst.kernel_ms, sizeof(stats->kernel_ms));
            std::memcpy(stats->kernel_count, bst.kernel_count, sizeof(stats->kernel_count));
            hstats[0] = bst.extension_rays;
            hstats[1] = bst.shadow_rays;
            hstats[2] = bst.dropped_samples;
        }
        for (const LaunchMarks::Mark &m : lm.marks) {
            float kms = 0;
            cudaEventElapsedTime(&kms, eventPool[m.ev], eventPool[m.ev + 1]);
            stats->kernel_ms[m.cls] += kms;
            stats->kernel_count[m.cls] += 1;
        }
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->kernel_seconds = ms * 1e-3;
        stats->path_samples = (uint64_t)pl.gridPositions * s.spp;
        stats->extension_rays = hstats[0];
        stats->shadow_rays = hstats[1];
        stats->dropped_samples = hstats[2];
        stats->kernel_launches = launches;
    }
    return SLRGPU_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free render (slrgpu_render_noalloc)
//
// For callers that may not allocate device memory once they are running: a
// real-time loop that owns a fixed memory budget, a host that hands the GPU
// to the renderer only between its own allocations, or an embedding runtime
// whose allocator forbids cudaMalloc after start-up.  The path state, queues,
// counters and the film sums live in one file-scope device array of a fixed
// size, which every GPU that loads this library keeps until the process
// exits.  Limits: the tile-padded sample grid (width and height rounded up to
// multiples of 8) times the samples per wave <= kNoAllocMaxPaths, and
// max_depth <= kNoAllocMaxDepth.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoAllocMaxPaths = 65536;
constexpr uint32_t kNoAllocMaxDepth = 64;

constexpr size_t naAlign(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kNaRay = 0;
constexpr size_t kNaHit = naAlign(kNaRay + 32ull * kNoAllocMaxPaths);
constexpr size_t kNaAlpha = naAlign(kNaHit + 16ull * kNoAllocMaxPaths);
constexpr size_t kNaL = naAlign(kNaAlpha + 4ull * kNumLambda * kNoAllocMaxPaths);
constexpr size_t kNaScalars = naAlign(kNaL + 4ull * kNumLambda * kNoAllocMaxPaths);
constexpr size_t kNaShRay = naAlign(kNaScalars + sizeof(PathScalars) * kNoAllocMaxPaths);
constexpr size_t kNaShContrib = naAlign(kNaShRay + 32ull * kNoAllocMaxPaths);
constexpr size_t kNaQueue0 = naAlign(kNaShContrib + 4ull * kNumLambda * kNoAllocMaxPaths);
constexpr size_t kNaQueue1 = naAlign(kNaQueue0 + 4ull * kNoAllocMaxPaths);
constexpr size_t kNaShQueue = naAlign(kNaQueue1 + 4ull * kNoAllocMaxPaths);
constexpr size_t kNaClassQueue = naAlign(kNaShQueue + 4ull * kNoAllocMaxPaths);
constexpr size_t kNaCounters = naAlign(kNaClassQueue + 4ull * kNumClassQueues * kNoAllocMaxPaths);
constexpr size_t kNaStats = naAlign(kNaCounters + 4ull * kCtrStride * (kNoAllocMaxDepth + 2));
constexpr size_t kNaFilmSum = naAlign(kNaStats + 8ull * 4);
constexpr size_t kNaFilmComp = naAlign(kNaFilmSum + 4ull * kNumLambda * kNoAllocMaxPaths);
constexpr size_t kNoAllocScratchBytes = naAlign(kNaFilmComp + 4ull * kNumLambda * kNoAllocMaxPaths);

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noallocMu;
void* g_noallocAddr[64] = {};   // device address of g_noallocScratch, per device
}  // namespace

size_t noAllocScratchBytes() { return kNoAllocScratchBytes; }

int renderNoAlloc(const DeviceScene &ds, const slrgpu_settings &s, float* film, cudaStream_t stream) {
    if (!film) {
        setError("film must be a device pointer");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (s.spp == 0) {
        setError("width, height and spp must be positive");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (int rc = checkImageSize(s.width, s.height)) return rc;
    if ((uint64_t)padToTile(s.width) * padToTile(s.height) > kNoAllocMaxPaths) {
        setError("slrgpu_render_noalloc: the sample grid (width and height rounded up to multiples of 8) exceeds "
                 "the fixed scratch limit of " + std::to_string(kNoAllocMaxPaths) + " positions");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (s.max_depth > kNoAllocMaxDepth) {
        setError("slrgpu_render_noalloc: max_depth exceeds the fixed scratch limit of " +
                 std::to_string(kNoAllocMaxDepth));
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const WavePlan pl = planWaves(s, kNoAllocMaxPaths);
    if ((uint64_t)pl.S * pl.gridPositions > kNoAllocMaxPaths) {
        setError("slrgpu_render_noalloc: sample grid * samples_per_wave exceeds the fixed scratch limit of " +
                 std::to_string(kNoAllocMaxPaths) + " paths");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const uint32_t P = pl.filmPixels;
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        setError("device index out of range for the scratch table");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    unsigned char* base = nullptr;
    {
        // First call on this device (with it current): resolve the device
        // address of the scratch array.  The host-side symbol is only a
        // stand-in and must never be handed to a kernel.
        std::lock_guard<std::mutex> lock(g_noallocMu);
        if (!g_noallocAddr[dev]) {
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noallocScratch);
            if (e != cudaSuccess || !ptr) {
                setError(std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
                return SLRGPU_ERR_CUDA;
            }
            g_noallocAddr[dev] = ptr;
        }
        base = (unsigned char*)g_noallocAddr[dev];
    }
    WaveState w;
    std::memset(&w, 0, sizeof(w));
    w.N = pl.S * pl.gridPositions;
    w.ray = (float4*)(base + kNaRay);
    w.hit = (float4*)(base + kNaHit);
    w.alpha = (float*)(base + kNaAlpha);
    w.L = (float*)(base + kNaL);
    w.ps = (PathScalars*)(base + kNaScalars);
    w.shRay = (float4*)(base + kNaShRay);
    w.shContrib = (float*)(base + kNaShContrib);
    w.queue[0] = (uint32_t*)(base + kNaQueue0);
    w.queue[1] = (uint32_t*)(base + kNaQueue1);
    w.shadowQueue = (uint32_t*)(base + kNaShQueue);
    w.classQueue = (uint32_t*)(base + kNaClassQueue);
    w.counters = (uint32_t*)(base + kNaCounters);
    w.stats = (unsigned long long*)(base + kNaStats);
    float* filmSum = (float*)(base + kNaFilmSum);
    float* filmComp = (float*)(base + kNaFilmComp);
    // The array keeps the previous call's contents: clear the accumulators
    // (the wave loop clears the queue counters of every wave itself).
    CUDA_TRY(cudaMemsetAsync(filmSum, 0, (size_t)P * kNumLambda * sizeof(float), stream));
    CUDA_TRY(cudaMemsetAsync(filmComp, 0, (size_t)P * kNumLambda * sizeof(float), stream));
    CUDA_TRY(cudaMemsetAsync(w.stats, 0, 4 * sizeof(unsigned long long), stream));
    LaunchMarks lm;
    uint64_t launches = 0;
    if (int rc = runWaves(ds, s, pl, w, filmSum, filmComp, stream, lm, &launches)) return rc;
    kFilmToPixelMajor<<<waveGrids(256).accumulate, 256, 0, stream>>>(filmSum, film, P);
    CUDA_TRY(cudaGetLastError());
    return SLRGPU_OK;
}

// ---------------------------------------------------------------------------
// Film output (ImageSensor::saveImage, Core/ImageSensor.cpp:139-195): the 16
// bins times scale x sensitivity -> XYZ with the discretised colour matching
// functions -> sRGB (double-precision matrix, spectrum_base.h:68-72) ->
// clamp at 0 -> 1 - exp(-x) -> sRGB gamma (spectrum_base.cpp:16-21) ->
// min(255, 256 x value), written as bottom-up BGR rows padded to 4 bytes.
// The arithmetic is rounded as the reference's host build rounds it (no
// contraction; the double expressions stay double).
// ---------------------------------------------------------------------------
struct FilmColor {
    float xbar[16], ybar[16], zbar[16];
    float integral;
};

__device__ __forceinline__ float srgbGamma(float v) {
    if ((double)v <= 0.0031308) return (float)__dmul_rn(12.92, (double)v);
    return (float)__dsub_rn(__dmul_rn(1.055, pow((double)v, 1.0 / 2.4)), 0.055);
}

__global__ void kFilmToBmp(const float* __restrict__ film, uint32_t w, uint32_t h, float scale, FilmColor fc,
                           uint8_t* __restrict__ out, uint32_t rowBytes) {
    const uint32_t P = w * h;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < P; pix += gridDim.x * blockDim.x) {
        const uint32_t i = pix / w, j = pix - i * w;
        float X = 0.0f, Y = 0.0f, Z = 0.0f;
#pragma unroll
        for (int b = 0; b < kNumLambda; ++b) {
            const float v = __fmul_rn(film[(size_t)pix * kNumLambda + b], scale);
            X = __fadd_rn(X, __fmul_rn(fc.xbar[b], v));
            Y = __fadd_rn(Y, __fmul_rn(fc.ybar[b], v));
            Z = __fadd_rn(Z, __fmul_rn(fc.zbar[b], v));
        }
        X = __fdiv_rn(X, fc.integral);
        Y = __fdiv_rn(Y, fc.integral);
        Z = __fdiv_rn(Z, fc.integral);
        const double x = X, y = Y, z = Z;
        float rgb[3];
        rgb[0] = (float)__dsub_rn(__dsub_rn(__dmul_rn(3.2404542, x), __dmul_rn(1.5371385, y)), __dmul_rn(0.4985314, z));
        rgb[1] = (float)__dadd_rn(__dadd_rn(__dmul_rn(-0.9692660, x), __dmul_rn(1.8760108, y)), __dmul_rn(0.0415560, z));
        rgb[2] = (float)__dadd_rn(__dsub_rn(__dmul_rn(0.0556434, x), __dmul_rn(0.2040259, y)), __dmul_rn(1.0572252, z));
        uint8_t bytes[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float v = rgb[c] < 0.0f ? 0.0f : rgb[c];
            v = __fsub_rn(1.0f, expf(-v));
            const float g = __fmul_rn(256.0f, srgbGamma(v));
            bytes[c] = (uint8_t)min(255u, (uint32_t)g);
        }
        uint8_t* dst = out + (size_t)(h - i - 1) * rowBytes + 3 * j;
        dst[0] = bytes[2];
        dst[1] = bytes[1];
        dst[2] = bytes[0];
    }
}

int filmToBmp(const float* film, uint32_t width, uint32_t height, bool filmOnDevice, float scale, float sensitivity,
              uint8_t* pixels) {
    if (width == 0 || height == 0) {
        setError("width and height must be positive");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    FilmColor fc;
    discretizedCmf(fc.xbar, fc.ybar, fc.zbar, &fc.integral);
    if (std::isinf(sensitivity)) sensitivity = 1.0f;
    scale *= sensitivity;
    const uint32_t rowBytes = 3 * width + width % 4;
    const size_t filmBytes = (size_t)width * height * kNumLambda * sizeof(float);
    const size_t outBytes = (size_t)rowBytes * height;
    float* dfilm = nullptr;
    uint8_t* dout = nullptr;
    cudaError_t e = cudaSuccess;
    if (!filmOnDevice) {
        e = cudaMalloc(&dfilm, filmBytes);
        if (e == cudaSuccess) e = cudaMemcpy(dfilm, film, filmBytes, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&dout, outBytes);
    if (e == cudaSuccess) e = cudaMemset(dout, 0, outBytes);
    if (e == cudaSuccess) {
        kFilmToBmp<<<std::min<uint32_t>((width * height + 255) / 256, 4096), 256>>>(
            filmOnDevice ? film : dfilm, width, height, scale, fc, dout, rowBytes);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(pixels, dout, outBytes, cudaMemcpyDeviceToHost);
    if (dfilm) cudaFree(dfilm);
    if (dout) cudaFree(dout);
    if (e != cudaSuccess) {
        setError(cudaGetErrorString(e));
        return SLRGPU_ERR_CUDA;
    }
    return SLRGPU_OK;
}

// ---------------------------------------------------------------------------
// Wave slots for the serving loop: path state for up to `paths` paths and
// waves whose segments come from several requests of one scene.
// ---------------------------------------------------------------------------
// A slot captures the launch sequence of a wave (counter reset, ray
// generation, every bounce's kernels, film update) once per (scene, max
// depth, integrator) as a CUDA graph and replays it for every later wave of
// that kind; the wave's segments travel in device memory (copied from pinned
// staging memory before each replay), so the captured launches never change.
static_assert(kMaxWaveScenesApi == kMaxWaveScenes, "one scene-table size");
struct WaveSlot {
    RenderEngine engine;   // path state only; films belong to the requests
    WaveParams* dParams = nullptr;
    WaveParams* hParams = nullptr;   // pinned
    DevScene* dScenes = nullptr;     // [kMaxWaveScenes]: the scene table of waves of several scenes
    DevScene* hScenes = nullptr;     // pinned
    struct Graph {
        uint64_t sceneUid;           // 0: a wave of several scenes
        uint32_t depth;
        bool volumetric;
        bool watertight;
        uint32_t kindMask;           // waves of several scenes: the kinds and the environment
        bool env;
        cudaGraphExec_t exec;
        uint64_t launches;
    };
    std::vector<Graph> graphs;
    ~WaveSlot() {
        for (Graph &g : graphs) cudaGraphExecDestroy(g.exec);
        if (dParams) cudaFree(dParams);
        if (hParams) cudaFreeHost(hParams);
        if (dScenes) cudaFree(dScenes);
        if (hScenes) cudaFreeHost(hScenes);
    }
};

WaveSlot* waveSlotCreate(uint32_t paths, uint32_t maxDepth, std::string* err) {
    WaveSlot* slot = new WaveSlot();
    if (slot->engine.ensure(paths, maxDepth) != SLRGPU_OK ||
        cudaMalloc(&slot->dParams, sizeof(WaveParams)) != cudaSuccess ||
        cudaMallocHost(&slot->hParams, sizeof(WaveParams)) != cudaSuccess ||
        cudaMalloc(&slot->dScenes, kMaxWaveScenes * sizeof(DevScene)) != cudaSuccess ||
        cudaMallocHost(&slot->hScenes, kMaxWaveScenes * sizeof(DevScene)) != cudaSuccess) {
        if (err) *err = "wave slot allocation failed";
        delete slot;
        return nullptr;
    }
    return slot;
}

void waveSlotDestroy(WaveSlot* slot) { delete slot; }

uint32_t waveSlotCapacity(const WaveSlot* slot) { return slot->engine.capacity; }

uint64_t waveSlotBytes(const WaveSlot* slot) {
    return slot->engine.stateBytes + sizeof(WaveParams) + kMaxWaveScenes * sizeof(DevScene);
}

uint32_t sampleGridPositions(uint32_t width, uint32_t height) { return padToTile(width) * padToTile(height); }

int launchWave(const DeviceScene* const* scenes, int numScenes, WaveSlot* slot, const SegmentDesc* segs, int numSegs,
               uint32_t maxDepth, bool volumetric, bool watertight, cudaStream_t stream, uint64_t* launches,
               bool useGraph) {
    if (numSegs <= 0 || numSegs > kMaxWaveSegments) {
        setError("a wave holds 1 to 32 segments");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (numScenes <= 0 || numScenes > kMaxWaveScenes || (numScenes > 1 && volumetric)) {
        setError("a wave holds 1 to 8 scenes (one for the volumetric path tracer)");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const DeviceScene &ds = *scenes[0];
    // waves of several scenes: the scene table, as the kernels see it
    WaveSceneTable table{slot->dScenes, 0u, false};
    const bool multi = numScenes > 1;
    if (multi) {
        for (int i = 0; i < numScenes; ++i) {
            DevScene sc = scenes[i]->sc;
            sc.watertight = watertight ? 1u : 0u;
            sc.rngTape = nullptr;
            slot->hScenes[i] = sc;
            table.kindMask |= scenes[i]->kindMask;
            table.env = table.env || sc.envPresent != 0;
        }
    }
    for (int i = 0; i < numSegs; ++i)
        if ((int)segs[i].scene >= numScenes) {
            setError("segment scene index out of range");
            return SLRGPU_ERR_INVALID_ARGUMENT;
        }
    if (maxDepth > slot->engine.depthCapacity) {
        setError("max_depth exceeds the wave slot's counter capacity");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    WaveParams wp;
    std::memset(&wp, 0, sizeof(wp));
    uint64_t paths = 0, pixels = 0;
    for (int i = 0; i < numSegs; ++i) {
        const SegmentDesc &d = segs[i];
        WaveSegment &sg = wp.seg[i];
        sg.pathBegin = (uint32_t)paths;
        sg.width = d.width;
        sg.height = d.height;
        sg.gridW = padToTile(d.width);
        sg.gridH = padToTile(d.height);
        sg.gridPositions = sg.gridW * sg.gridH;
        sg.sampleBase = d.sampleBase;
        sg.samples = d.samples;
        sg.seed = d.seed;
        sg.scene = d.scene;
        sg.filmBegin = (uint32_t)pixels;
        sg.filmSum = d.filmSum;
        sg.filmComp = d.filmComp;
        sg.dropped = d.dropped;
        paths += (uint64_t)sg.samples * sg.gridPositions;
        pixels += (uint64_t)d.width * d.height;
    }
    if (paths > slot->engine.capacity || pixels > 0x7fffffffull) {
        setError("wave larger than the slot");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    wp.numSegments = (uint32_t)numSegs;
    wp.numPaths = (uint32_t)paths;
    wp.filmPixels = (uint32_t)pixels;
    // The previous wave on this slot has completed (the caller waits for it),
    // so the staging copies are free to overwrite.
    if (multi)
        CUDA_TRY(cudaMemcpyAsync(slot->dScenes, slot->hScenes, numScenes * sizeof(DevScene), cudaMemcpyHostToDevice,
                                 stream));
    if (!useGraph) {
        LaunchMarks lm;
        uint64_t n = 0;
        int rc = runWave(ds, *slot->engine.ws, wp, maxDepth, volumetric, watertight, stream, lm, &n, nullptr, nullptr,
                         multi ? &table : nullptr);
        if (launches) *launches += n;
        return rc;
    }
    const uint64_t uid = multi ? 0 : ds.uid;
    WaveSlot::Graph* graph = nullptr;
    for (WaveSlot::Graph &g : slot->graphs)
        if (g.sceneUid == uid && g.depth == maxDepth && g.volumetric == volumetric && g.watertight == watertight &&
            (!multi || (g.kindMask == table.kindMask && g.env == table.env)))
            graph = &g;
    if (!graph) {
        waveGrids(256);   // occupancy queries stay outside the capture
        // Capture on this stream: the launches read their segments from
        // slot->dParams, so the by-value parameters are left empty.
        WaveParams empty;
        std::memset(&empty, 0, sizeof(empty));
        LaunchMarks lm;
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        uint64_t n = 0;
        int rc = runWave(ds, *slot->engine.ws, empty, maxDepth, volumetric, watertight, stream, lm, &n,
                         slot->dParams, nullptr, multi ? &table : nullptr);
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (rc != SLRGPU_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) {
            setError(std::string("wave capture failed: ") + cudaGetErrorString(e));
            return SLRGPU_ERR_CUDA;
        }
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            setError(std::string("wave graph instantiation failed: ") + cudaGetErrorString(e));
            return SLRGPU_ERR_CUDA;
        }
        slot->graphs.push_back(
            WaveSlot::Graph{uid, maxDepth, volumetric, watertight, table.kindMask, table.env, exec, n});
        graph = &slot->graphs.back();
    }
    std::memcpy(slot->hParams, &wp, sizeof(wp));
    CUDA_TRY(cudaMemcpyAsync(slot->dParams, slot->hParams, sizeof(wp), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaGraphLaunch(graph->exec, stream));
    if (launches) *launches += graph->launches;
    return SLRGPU_OK;
}

int launchFilmToPixelMajor(const float* filmSum, float* out, uint32_t pixels, cudaStream_t stream) {
    kFilmToPixelMajor<<<waveGrids(256).accumulate, 256, 0, stream>>>(filmSum, out, pixels);
    CUDA_TRY(cudaGetLastError());
    return SLRGPU_OK;
}

int bsdfQuery(int kind, const float* s0, const float* s1, const float* s2, float ax, float ay, const float* queries,
              uint32_t n, float* out) {
    Bsdf B;
    std::memset(&B, 0, sizeof(B));
    static const uint32_t kinds[5] = {kMatMatte, kMatSpecularReflection, kMatSpecularScattering, kMatGGXReflection,
                                      kMatGGXScattering};
    if (kind < 0 || kind > 4) {
        setError("unknown BSDF kind");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    B.kind = kinds[kind];
    for (int i = 0; i < kNumLambda; ++i) {
        B.a.v[i] = s0[i];
        B.b.v[i] = s1 ? s1[i] : s0[i];
        B.c.v[i] = s2 ? s2[i] : s0[i];
    }
    B.ax = ax;
    B.ay = ay;
    B.dispersive = true;
    if (n == 0) return SLRGPU_OK;
    float *dq = nullptr, *dout = nullptr;
    CUDA_TRY(cudaMalloc(&dq, (size_t)n * 16 * sizeof(float)));
    cudaError_t e = cudaMalloc(&dout, (size_t)n * 40 * sizeof(float));
    if (e != cudaSuccess) { cudaFree(dq); setError(cudaGetErrorString(e)); return SLRGPU_ERR_CUDA; }
    e = cudaMemcpy(dq, queries, (size_t)n * 16 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        kBsdfQuery<<<std::min<uint32_t>((n + 255) / 256, 4096), 256>>>(B, dq, n, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 40 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dq);
    cudaFree(dout);
    if (e != cudaSuccess) { setError(cudaGetErrorString(e)); return SLRGPU_ERR_CUDA; }
    return SLRGPU_OK;
}

int mediumQuery(const DeviceScene &ds, int mode, uint32_t n, const float* rays, const float* lambdas, const int* sel,
                const uint32_t* vals, uint32_t nvals, float* out) {
    if (!ds.sc.medium.present) {
        setError("the scene has no medium");
        return SLRGPU_ERR_STATE;
    }
    if (mode < 0 || mode > 4) {
        setError("medium query mode must be 0 to 4");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return SLRGPU_OK;
    const size_t bRays = (size_t)n * 8 * sizeof(float), bLam = (size_t)n * 16 * sizeof(float);
    const size_t bSel = (size_t)n * sizeof(int), bVals = (size_t)n * nvals * sizeof(uint32_t);
    const size_t bOut = (size_t)n * 24 * sizeof(float);
    unsigned char* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, bRays + bLam + bSel + bVals + bOut + 64));
    float* dRays = (float*)d;
    float* dLam = (float*)(d + bRays);
    int* dSel = (int*)(d + bRays + bLam);
    uint32_t* dVals = (uint32_t*)(d + bRays + bLam + bSel);
    float* dOut = (float*)(d + bRays + bLam + bSel + bVals);
    cudaError_t e = cudaMemcpy(dRays, rays, bRays, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dLam, lambdas, bLam, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dSel, sel, bSel, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bVals) e = cudaMemcpy(dVals, vals, bVals, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        kMediumQuery<<<std::min<uint32_t>((n + 127) / 128, 4096), 128>>>(ds.sc, mode, n, dRays, dLam, dSel, dVals,
                                                                         nvals, dOut);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dOut, bOut, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        setError(cudaGetErrorString(e));
        return SLRGPU_ERR_CUDA;
    }
    return SLRGPU_OK;
}

int traceRays(const DeviceScene &ds, const float* rays, uint32_t n, int anyHit, uint32_t* prim, float* t, float* b1,
              float* b2, cudaStream_t stream) {
    if (n == 0) return SLRGPU_OK;
    static int grid = 0;
    if (!grid) grid = gridFor((const void*)kTrace, 256);
    DevScene sc = ds.sc;
    sc.watertight = (anyHit & 2) ? 1u : 0u;
    kTrace<<<grid, 256, 0, stream>>>(sc, rays, n, anyHit & 1, prim, t, b1, b2);
    CUDA_TRY(cudaGetLastError());
    return SLRGPU_OK;
}

}  // namespace slrgpu
