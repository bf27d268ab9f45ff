// Internal interface between the C ABI (capi.cpp) and the CUDA side (render.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/slrgpu.h"
#include "scene_host.h"
#include "slrgpu_types.h"

namespace slrgpu {

void setError(const std::string &msg);

struct DeviceBuffers {
    std::vector<void*> allocs;   // device arrays
    std::vector<void*> pinned;   // pinned host mirrors of the same arrays
    std::vector<size_t> sizes;
    void release();
    ~DeviceBuffers() { release(); }
};

struct DeviceScene {
    DevScene sc;
    DeviceBuffers buffers;
    uint32_t kindMask = 0;   // bit k: some material of kind k (MaterialKind) exists
    uint64_t uid = 0;        // unique per upload (keys captured wave graphs)
};

// Device bytes a committed scene holds (BVH, triangles, vertices, materials,
// spectra, environment and medium tables).
inline uint64_t deviceSceneBytes(const DeviceScene &ds) {
    uint64_t b = 0;
    for (size_t n : ds.buffers.sizes) b += n;
    return b;
}

struct WaveState;
struct BptEngine;   // bidirectional path state (bpt.cu)

// Per-context path state and film buffers, grown on demand.
struct RenderEngine {
    WaveState* ws = nullptr;
    BptEngine* bpt = nullptr;
    std::vector<void*> allocs;
    uint32_t capacity = 0;
    uint32_t depthCapacity = 0;
    uint64_t stateBytes = 0;     // device bytes of the path state (ws)
    float* filmSum = nullptr;
    float* filmComp = nullptr;
    float* filmOut = nullptr;
    uint32_t filmPixels = 0;
    std::vector<cudaEvent_t> eventPool;

    int ensure(uint32_t paths, uint32_t maxDepth);
    int ensureFilm(uint32_t pixels);
    // the last wave's per-bounce queue counters (rows of kQueueCountColumns)
    int queueCounts(uint32_t* out, uint32_t capacity, uint32_t* rows);
    void release();
    // filmState (host, optional): the compensated film sums to continue
    // from (2 x 16 x width x height floats: sum planes, then compensation
    // planes), updated in place; film may then be null.
    int render(const DeviceScene &ds, const slrgpu_settings &s, float* film, bool filmOnDevice,
               slrgpu_render_stats* stats, cudaStream_t stream, float* filmState = nullptr,
               const float* rngTape = nullptr);   // device tape of slrgpu_render_replay
    ~RenderEngine();
};

// Bidirectional path tracing (BPTRenderer) into a compensated 16-bin film
// ([16][width * height] sum and compensation planes on the device, added
// to).  eventPool non-null: per-kernel timing into stats->kernel_ms.
BptEngine* bptEngineCreate();
void bptEngineDestroy(BptEngine* e);
int renderBpt(BptEngine &eng, const DeviceScene &ds, const slrgpu_settings &s, float* filmSum, float* filmComp,
              cudaStream_t stream, uint64_t* launches, std::vector<cudaEvent_t>* eventPool,
              slrgpu_render_stats* stats);

// Wave slots (serving): path state for up to `paths` paths in flight.
struct WaveSlot;
// One request's share of a wave: samples [sampleBase, sampleBase + samples)
// over its whole tile-padded sample grid, accumulated into its film
// (16-bin planes of width * height floats, sum and compensation).
struct SegmentDesc {
    uint32_t width, height, sampleBase, samples, seed;
    uint32_t scene;                // index in launchWave's scene list
    float* filmSum;
    float* filmComp;
    unsigned long long* dropped;   // device counter, or null
};
WaveSlot* waveSlotCreate(uint32_t paths, uint32_t maxDepth, std::string* err);
void waveSlotDestroy(WaveSlot* slot);
uint32_t waveSlotCapacity(const WaveSlot* slot);
uint64_t waveSlotBytes(const WaveSlot* slot);   // device bytes the slot holds
uint32_t sampleGridPositions(uint32_t width, uint32_t height);
// Largest image side any entry point accepts; checkImageSize() also bounds
// the tile-padded grid to 2^31 - 1 positions (sets the error text).
constexpr uint32_t kMaxImageSide = 1u << 20;
// columns of slrgpu_context_queue_counts' rows
constexpr uint32_t kQueueCountColumns = 11;
// uniforms per grid position of slrgpu_render_replay's tapes
constexpr uint32_t kRngTapeFloats = 256;
int checkImageSize(uint32_t width, uint32_t height);
// useGraph: replay the slot's captured graph for this (scene, depth,
// integrator), capturing it on first use.
// A wave of up to kMaxWaveScenesApi scenes: with more than one, the surface
// path tracer's kernels find each path's scene in a table (volumetric waves
// take one scene).
constexpr int kMaxWaveScenesApi = 8;
int launchWave(const DeviceScene* const* scenes, int numScenes, WaveSlot* slot, const SegmentDesc* segs, int numSegs,
               uint32_t maxDepth,
               bool volumetric, bool watertight, cudaStream_t stream, uint64_t* launches, bool useGraph);
int launchFilmToPixelMajor(const float* filmSum, float* out, uint32_t pixels, cudaStream_t stream);

// Film -> 8-bit sRGB BMP pixel rows (bottom-up BGR, rows padded to 4 bytes).
int filmToBmp(const float* film, uint32_t width, uint32_t height, bool filmOnDevice, float scale, float sensitivity,
              uint8_t* pixels);

int uploadScene(const HostScene &hs, const BuiltScene &bs, DeviceScene* ds);
int reuploadScene(DeviceScene* ds, uint64_t* bytes, cudaStream_t stream);
// Render with all scratch in a fixed device array (no allocation).
int renderNoAlloc(const DeviceScene &ds, const slrgpu_settings &s, float* film, cudaStream_t stream);
size_t noAllocScratchBytes();
int bsdfQuery(int kind, const float* s0, const float* s1, const float* s2, float ax, float ay, const float* queries,
              uint32_t n, float* out);
int mediumQuery(const DeviceScene &ds, int mode, uint32_t n, const float* rays, const float* lambdas, const int* sel,
                const uint32_t* vals, uint32_t nvals, float* out);
int traceRays(const DeviceScene &ds, const float* rays, uint32_t n, int anyHit, uint32_t* prim, float* t, float* b1,
              float* b2, cudaStream_t stream);

}  // namespace slrgpu
