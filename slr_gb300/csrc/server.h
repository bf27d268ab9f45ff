// Serving loop: continuous batching of render requests on one GPU.
//
// Requests of any resident scene, resolution and sample count are queued,
// admitted while their films fit the HBM budget, and rendered in waves.  In
// the batched mode a wave packs the next samples of several admitted
// requests (same integrator and max depth; for the surface path tracer of up
// to 8 different scenes, whose paths then share one set of queues) into one
// set of launches, and several waves run concurrently on their own streams
// and path-state slots; requests that arrive while others are on the GPU
// join the next wave.  The plain mode renders one request at a time
// with waves of that request only, as slrgpu_render does.  A request's random
// numbers depend only on (seed, sample, pixel) and its film accumulates its
// samples in order, so its film is bit-identical in either mode and to
// slrgpu_render.
//
// The HBM budget covers everything the server keeps on the device for its
// requests: the path-state slots (charged at creation), each resident scene
// that an admitted request renders (charged once, while any of its admitted
// requests is alive) and the admitted requests' films.  A request can be
// cancelled, or given a deadline after which the server cancels it; either
// stops issuing its samples, and it ends once its waves in flight finish.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <string>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/slrgpu.h"
#include "render_api.h"

namespace slrgpu {

// slrgpu_debug_inject_fault's sites (host side only).
int injectFault(int site, uint32_t count);

class Server {
public:
    Server(int device, const slrgpu_server_config &cfg);
    ~Server();
    int init();   // allocates the wave slots; SLRGPU_OK or an error code
    // `pin` counts the scene's unfinished requests (the scene must not be
    // destroyed while it is nonzero).
    int submit(const DeviceScene* ds, std::atomic<int>* pin, const slrgpu_settings &s, uint64_t* id);
    int poll(uint64_t id, slrgpu_request_info* info);
    int wait(uint64_t id, float* filmHost, slrgpu_request_info* info, double timeoutSeconds);
    int cancel(uint64_t id);
    int setDeadline(uint64_t id, double secondsFromNow);
    void stats(slrgpu_server_stats* st);

private:
    struct Request {
        uint64_t id = 0;
        const DeviceScene* ds = nullptr;
        std::atomic<int>* pin = nullptr;
        slrgpu_settings settings{};
        int status = SLRGPU_REQUEST_QUEUED;
        double tSubmit = 0, tStart = 0, tDone = 0;
        uint32_t samplesIssued = 0, samplesDone = 0;
        uint32_t pixels = 0, gridPositions = 0;
        uint64_t footprint = 0;
        float* filmSum = nullptr;
        float* filmComp = nullptr;
        float* filmOut = nullptr;
        unsigned long long* dropped = nullptr;
        unsigned long long droppedHost = 0;
        bool finishing = false;
        bool admitted = false;    // its footprint counts against the budget
        bool cancelled = false;   // no more samples are issued
        int cancelStatus = 0;     // the status it ends with once its waves finish
        double deadline = -1;     // server time after which it is cancelled (< 0: none)
        cudaEvent_t doneEvent = nullptr;
        std::string error;
    };
    struct Slot {
        WaveSlot* wave = nullptr;
        cudaStream_t stream = nullptr;
        cudaEvent_t event = nullptr;
        bool busy = false;
        // the wave in flight: requests and the sample count each reaches
        std::vector<std::pair<Request*, uint32_t>> segments;
        const DeviceScene* ds = nullptr;
    };

    void worker();
    double now() const;
    void admitLocked();
    bool launchWaves();          // returns true when a wave was launched
    bool reapSlots(bool block);  // returns true when a slot finished
    void reapFinishing();
    void failRequest(Request* r, const std::string &why);
    void retireLocked(Request* r, int status, const std::string &why);
    int cancelLocked(Request* r, int status, const std::string &why);
    bool inFlightLocked(const Request* r) const;
    void retireCancelledLocked();
    void expireDeadlinesLocked();
    void releaseBudgetLocked(Request* r);
    void releaseBuffers(Request* r);

    int device_;
    slrgpu_server_config cfg_;
    std::chrono::steady_clock::time_point t0_;
    std::mutex mu_;
    std::condition_variable cvWork_, cvDone_;
    std::deque<Request*> pending_;
    std::vector<Request*> active_;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> requests_;
    std::vector<Slot> slots_;
    cudaStream_t allocStream_ = nullptr;   // film allocation, clearing and release
    uint64_t nextId_ = 1;
    uint64_t usedBytes_ = 0;      // slots + charged scenes + admitted films
    uint64_t slotBytes_ = 0;
    // resident scenes charged to the budget: admitted requests alive, bytes
    std::unordered_map<const DeviceScene*, std::pair<int, uint64_t>> sceneCharge_;
    bool stop_ = false;
    std::thread thread_;
    // statistics
    uint64_t mixedWaves_ = 0;
    uint64_t wavesLaunched_ = 0, kernelLaunches_ = 0, pathSamplesDone_ = 0, requestsDone_ = 0;
    double firstStart_ = -1, lastDone_ = 0;
};

}  // namespace slrgpu
