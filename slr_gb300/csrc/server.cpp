// Serving loop with continuous batching (see server.h).
#include "server.h"
#include "trace_ranges.h"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace slrgpu {

namespace {
constexpr uint32_t kDefaultSlotPaths = 4u << 20;
constexpr uint32_t kDefaultMaxDepth = 64;
constexpr uint64_t kDefaultBudget = 150ull << 30;
constexpr int kMaxSegmentsPerWave = 32;

uint64_t filmBytes(uint32_t pixels) { return 3ull * pixels * 16 * sizeof(float); }

// Host-side fault injection (slrgpu_debug_inject_fault): the next n film
// allocations or wave launches of any server fail as if the CUDA call had.
std::atomic<uint32_t> g_faultFilmAlloc{0}, g_faultWaveLaunch{0};
bool takeFault(std::atomic<uint32_t> &counter) {
    uint32_t v = counter.load();
    while (v > 0)
        if (counter.compare_exchange_weak(v, v - 1)) return true;
    return false;
}
}  // namespace

int injectFault(int site, uint32_t count) {
    switch (site) {
    case SLRGPU_FAULT_SERVER_FILM_ALLOC: g_faultFilmAlloc.store(count); return SLRGPU_OK;
    case SLRGPU_FAULT_SERVER_WAVE_LAUNCH: g_faultWaveLaunch.store(count); return SLRGPU_OK;
    default:
        setError("unknown fault site");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
}

Server::Server(int device, const slrgpu_server_config &cfg) : device_(device), cfg_(cfg) {
    if (cfg_.mode != SLRGPU_SERVER_PLAIN) cfg_.mode = SLRGPU_SERVER_BATCHED;
    if (cfg_.slots == 0) cfg_.slots = cfg_.mode == SLRGPU_SERVER_PLAIN ? 1 : 4;
    if (cfg_.mode == SLRGPU_SERVER_PLAIN) cfg_.slots = 1;
    if (cfg_.paths_per_slot == 0) cfg_.paths_per_slot = kDefaultSlotPaths;
    if (cfg_.max_depth == 0) cfg_.max_depth = kDefaultMaxDepth;
    if (cfg_.hbm_budget_bytes == 0) cfg_.hbm_budget_bytes = kDefaultBudget;
    t0_ = std::chrono::steady_clock::now();
}

int Server::init() {
    cudaError_t e = cudaSetDevice(device_);
    if (e != cudaSuccess) {
        setError(cudaGetErrorString(e));
        return SLRGPU_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&allocStream_, cudaStreamNonBlocking) != cudaSuccess) {
        setError("server: stream creation failed");
        return SLRGPU_ERR_CUDA;
    }
    slots_.resize(cfg_.slots);
    for (Slot &sl : slots_) {
        std::string err;
        sl.wave = waveSlotCreate(cfg_.paths_per_slot, cfg_.max_depth, &err);
        if (!sl.wave) {
            setError("server: " + err);
            return SLRGPU_ERR_OUT_OF_MEMORY;
        }
        slotBytes_ += waveSlotBytes(sl.wave);
        if (slotBytes_ > cfg_.hbm_budget_bytes) {
            setError("server: the path-state slots alone exceed the HBM budget");
            return SLRGPU_ERR_INVALID_ARGUMENT;
        }
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.event, cudaEventDisableTiming) != cudaSuccess) {
            setError("server: stream or event creation failed");
            return SLRGPU_ERR_CUDA;
        }
    }
    usedBytes_ = slotBytes_;
    thread_ = std::thread(&Server::worker, this);
    return SLRGPU_OK;
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lock(mu_);
        stop_ = true;
    }
    cvWork_.notify_all();
    if (thread_.joinable()) thread_.join();
    cudaSetDevice(device_);
    for (Slot &sl : slots_) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.event) cudaEventDestroy(sl.event);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.wave) waveSlotDestroy(sl.wave);
    }
    for (auto &kv : requests_) {
        Request* r = kv.second.get();
        if (r->pin) r->pin->fetch_sub(1);
        r->pin = nullptr;
        releaseBuffers(r);
    }
    if (allocStream_) {
        cudaStreamSynchronize(allocStream_);
        cudaStreamDestroy(allocStream_);
    }
}

double Server::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

int Server::submit(const DeviceScene* ds, std::atomic<int>* pin, const slrgpu_settings &s, uint64_t* id) {
    if (s.spp == 0) {
        setError("width, height and spp must be positive");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    if (int rc = checkImageSize(s.width, s.height)) return rc;
    if (s.max_depth > cfg_.max_depth) {
        setError("max_depth exceeds the server's max_depth");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const uint64_t grid = sampleGridPositions(s.width, s.height);
    if (grid > cfg_.paths_per_slot) {
        setError("one sample of the image exceeds the server's paths per slot");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    const uint64_t pixels = (uint64_t)s.width * s.height;
    if (slotBytes_ + deviceSceneBytes(*ds) + filmBytes((uint32_t)pixels) > cfg_.hbm_budget_bytes) {
        setError("the request's film and scene, with the path-state slots, exceed the server's HBM budget");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    std::unique_ptr<Request> r(new Request());
    r->ds = ds;
    r->pin = pin;
    r->settings = s;
    r->pixels = (uint32_t)pixels;
    r->gridPositions = (uint32_t)grid;
    r->footprint = filmBytes((uint32_t)pixels);
    {
        std::lock_guard<std::mutex> lock(mu_);
        r->id = nextId_++;
        r->tSubmit = now();
        *id = r->id;
        if (pin) pin->fetch_add(1);
        pending_.push_back(r.get());
        requests_[r->id] = std::move(r);
    }
    cvWork_.notify_all();
    return SLRGPU_OK;
}

static void fillInfo(slrgpu_request_info* info, int status, uint32_t sppDone, double ts, double tb, double td,
                     uint64_t samples, uint64_t dropped) {
    if (!info) return;
    std::memset(info, 0, sizeof(*info));
    info->status = status;
    info->spp_done = sppDone;
    info->submit_seconds = ts;
    info->start_seconds = tb;
    info->done_seconds = td;
    info->path_samples = samples;
    info->dropped_samples = dropped;
}

int Server::poll(uint64_t id, slrgpu_request_info* info) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) {
        setError("unknown request");
        return SLRGPU_ERR_INVALID_HANDLE;
    }
    Request* r = it->second.get();
    fillInfo(info, r->status, r->samplesDone, r->tSubmit, r->tStart, r->tDone,
             (uint64_t)r->samplesDone * r->gridPositions, r->droppedHost);
    return SLRGPU_OK;
}

int Server::wait(uint64_t id, float* filmHost, slrgpu_request_info* info, double timeoutSeconds) {
    std::unique_ptr<Request> owned;
    {
        std::unique_lock<std::mutex> lock(mu_);
        auto it = requests_.find(id);
        if (it == requests_.end()) {
            setError("unknown request");
            return SLRGPU_ERR_INVALID_HANDLE;
        }
        Request* r = it->second.get();
        auto finished = [&]() { return r->status == SLRGPU_REQUEST_DONE || r->status < 0; };
        if (timeoutSeconds < 0) {
            cvDone_.wait(lock, finished);
        } else if (!cvDone_.wait_for(lock, std::chrono::duration<double>(timeoutSeconds), finished)) {
            setError("timeout");
            fillInfo(info, r->status, r->samplesDone, r->tSubmit, r->tStart, r->tDone,
                     (uint64_t)r->samplesDone * r->gridPositions, r->droppedHost);
            return SLRGPU_ERR_TIMEOUT;
        }
        owned = std::move(it->second);
        requests_.erase(it);
        releaseBudgetLocked(owned.get());
    }
    cvWork_.notify_all();   // budget freed
    Request* r = owned.get();
    fillInfo(info, r->status, r->samplesDone, r->tSubmit, r->tStart, r->tDone,
             (uint64_t)r->samplesDone * r->gridPositions, r->droppedHost);
    int rc = SLRGPU_OK;
    if (r->status < 0) {
        setError(r->error);
        rc = r->status;
    } else if (filmHost) {
        cudaSetDevice(device_);
        cudaError_t e = cudaMemcpy(filmHost, r->filmOut, (size_t)r->pixels * 16 * sizeof(float),
                                   cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            setError(cudaGetErrorString(e));
            rc = SLRGPU_ERR_CUDA;
        }
    }
    releaseBuffers(r);
    return rc;
}

// Gives back the request's film bytes and, with its scene's last admitted
// request, the scene's bytes.  Holds mu_.
void Server::releaseBudgetLocked(Request* r) {
    if (!r->admitted) return;
    r->admitted = false;
    usedBytes_ -= r->footprint;
    auto it = sceneCharge_.find(r->ds);
    if (it != sceneCharge_.end() && --it->second.first == 0) {
        usedBytes_ -= it->second.second;
        sceneCharge_.erase(it);
    }
}

// True while a wave holding samples of the request is on the GPU.  Holds mu_.
bool Server::inFlightLocked(const Request* r) const {
    for (const Slot &sl : slots_)
        if (sl.busy)
            for (const auto &pr : sl.segments)
                if (pr.first == r) return true;
    return false;
}

// Ends a request with a final status.  Holds mu_.
void Server::retireLocked(Request* r, int status, const std::string &why) {
    r->status = status;
    r->error = why;
    r->tDone = now();
    if (r->pin) r->pin->fetch_sub(1);
    r->pin = nullptr;
    active_.erase(std::remove(active_.begin(), active_.end(), r), active_.end());
    cvDone_.notify_all();
}

// Cancels a queued or running request: a queued one ends now, a running one
// stops getting samples and ends when its waves in flight finish.  A request
// whose film is already being converted is left to finish.  Holds mu_.
int Server::cancelLocked(Request* r, int status, const std::string &why) {
    if (r->status == SLRGPU_REQUEST_DONE || r->status < 0 || r->finishing || r->cancelled) {
        setError("the request has already finished or is finishing");
        return SLRGPU_ERR_STATE;
    }
    auto q = std::find(pending_.begin(), pending_.end(), r);
    if (q != pending_.end()) {
        pending_.erase(q);
        retireLocked(r, status, why);
        return SLRGPU_OK;
    }
    r->cancelled = true;
    r->cancelStatus = status;
    r->error = why;
    if (!inFlightLocked(r)) retireLocked(r, status, why);
    return SLRGPU_OK;
}

void Server::retireCancelledLocked() {
    for (size_t i = 0; i < active_.size();) {
        Request* r = active_[i];
        if (r->cancelled && !inFlightLocked(r)) {
            retireLocked(r, r->cancelStatus, r->error);   // removes it from active_
            continue;
        }
        ++i;
    }
}

void Server::expireDeadlinesLocked() {
    const double t = now();
    std::vector<Request*> late;
    for (Request* r : pending_)
        if (r->deadline >= 0 && t > r->deadline) late.push_back(r);
    for (Request* r : active_)
        if (r->deadline >= 0 && t > r->deadline && !r->finishing && !r->cancelled) late.push_back(r);
    for (Request* r : late) cancelLocked(r, SLRGPU_ERR_TIMEOUT, "deadline exceeded");
}

int Server::cancel(uint64_t id) {
    int rc;
    {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = requests_.find(id);
        if (it == requests_.end()) {
            setError("unknown request");
            return SLRGPU_ERR_INVALID_HANDLE;
        }
        rc = cancelLocked(it->second.get(), SLRGPU_ERR_CANCELLED, "cancelled");
    }
    cvWork_.notify_all();
    return rc;
}

int Server::setDeadline(uint64_t id, double secondsFromNow) {
    if (!(secondsFromNow >= 0)) {
        setError("the deadline must be a non-negative number of seconds");
        return SLRGPU_ERR_INVALID_ARGUMENT;
    }
    {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = requests_.find(id);
        if (it == requests_.end()) {
            setError("unknown request");
            return SLRGPU_ERR_INVALID_HANDLE;
        }
        Request* r = it->second.get();
        if (r->status == SLRGPU_REQUEST_DONE || r->status < 0) {
            setError("the request has already finished");
            return SLRGPU_ERR_STATE;
        }
        r->deadline = now() + secondsFromNow;
    }
    cvWork_.notify_all();
    return SLRGPU_OK;
}

void Server::stats(slrgpu_server_stats* st) {
    std::lock_guard<std::mutex> lock(mu_);
    std::memset(st, 0, sizeof(*st));
    st->requests_done = requestsDone_;
    st->path_samples_done = pathSamplesDone_;
    st->waves = wavesLaunched_;
    st->kernel_launches = kernelLaunches_;
    st->bytes_in_use = usedBytes_;
    st->queued = (uint32_t)pending_.size();
    st->active = (uint32_t)active_.size();
    st->mixed_scene_waves = mixedWaves_;
    st->first_start_seconds = firstStart_;
    st->last_done_seconds = lastDone_;
}

void Server::releaseBuffers(Request* r) {
    // Only called once the request's work has finished on the GPU.
    cudaSetDevice(device_);
    if (r->doneEvent) cudaEventDestroy(r->doneEvent);
    if (r->filmSum) cudaFreeAsync(r->filmSum, allocStream_);
    if (r->filmComp) cudaFreeAsync(r->filmComp, allocStream_);
    if (r->filmOut) cudaFreeAsync(r->filmOut, allocStream_);
    if (r->dropped) cudaFreeAsync(r->dropped, allocStream_);
    r->doneEvent = nullptr;
    r->filmSum = r->filmComp = r->filmOut = nullptr;
    r->dropped = nullptr;
}

void Server::failRequest(Request* r, const std::string &why) {
    if (r->status == SLRGPU_REQUEST_DONE || r->status < 0) return;
    retireLocked(r, SLRGPU_ERR_CUDA, why);
}

// Moves queued requests into the active set, oldest first, while their films
// fit the budget (plain mode: one active request at a time).  Holds mu_.
void Server::admitLocked() {
    while (!pending_.empty()) {
        if (cfg_.mode == SLRGPU_SERVER_PLAIN && !active_.empty()) return;
        Request* r = pending_.front();
        auto charged = sceneCharge_.find(r->ds);
        const uint64_t sceneBytes = charged == sceneCharge_.end() ? deviceSceneBytes(*r->ds) : 0;
        if (usedBytes_ + r->footprint + sceneBytes > cfg_.hbm_budget_bytes) return;
        size_t freeB = 0, totalB = 0;
        if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess && freeB < r->footprint + (256ull << 20)) return;
        pending_.pop_front();
        TraceRange range("admit request %llu", (unsigned long long)r->id);
        // Stream-ordered allocation: no device-wide synchronisation while
        // other requests' waves run.
        const size_t planes = (size_t)r->pixels * 16 * sizeof(float);
        cudaStream_t st = allocStream_;
        bool ok = !takeFault(g_faultFilmAlloc) &&
                  cudaMallocAsync((void**)&r->filmSum, planes, st) == cudaSuccess &&
                  cudaMallocAsync((void**)&r->filmComp, planes, st) == cudaSuccess &&
                  cudaMallocAsync((void**)&r->filmOut, planes, st) == cudaSuccess &&
                  cudaMallocAsync((void**)&r->dropped, sizeof(unsigned long long), st) == cudaSuccess &&
                  cudaEventCreateWithFlags(&r->doneEvent, cudaEventDisableTiming) == cudaSuccess &&
                  cudaMemsetAsync(r->filmSum, 0, planes, st) == cudaSuccess &&
                  cudaMemsetAsync(r->filmComp, 0, planes, st) == cudaSuccess &&
                  cudaMemsetAsync(r->dropped, 0, sizeof(unsigned long long), st) == cudaSuccess &&
                  cudaStreamSynchronize(st) == cudaSuccess;
        usedBytes_ += r->footprint + sceneBytes;
        if (charged == sceneCharge_.end()) sceneCharge_[r->ds] = {1, sceneBytes};
        else ++charged->second.first;
        r->admitted = true;
        if (!ok) {
            r->status = SLRGPU_ERR_OUT_OF_MEMORY;
            r->error = "film allocation failed";
            r->tDone = now();
            if (r->pin) r->pin->fetch_sub(1);
            r->pin = nullptr;
            cvDone_.notify_all();
            continue;
        }
        r->status = SLRGPU_REQUEST_RUNNING;
        r->tStart = now();
        if (firstStart_ < 0) firstStart_ = r->tStart;
        active_.push_back(r);
    }
}

// Fills every idle slot with a wave: the next samples of admitted requests,
// oldest first, that share an integrator, max depth and triangle test.  In
// the batched mode a surface path-tracer wave takes requests of up to
// kMaxWaveScenesApi scenes into one set of queues; a volumetric wave takes
// one scene.  A request is in at most one wave at a time (its film adds its
// samples in order).  Holds mu_.
bool Server::launchWaves() {
    bool launched = false;
    for (Slot &sl : slots_) {
        if (sl.busy) continue;
        // the oldest active request that still has samples to issue and no
        // wave in flight picks the wave's integrator and depth
        Request* lead = nullptr;
        for (Request* r : active_)
            if (r->samplesIssued < r->settings.spp && !r->cancelled && !inFlightLocked(r)) {
                lead = r;
                break;
            }
        if (!lead) break;
        const bool mixScenes = cfg_.mode == SLRGPU_SERVER_BATCHED && !lead->settings.volumetric;
        const uint32_t cap = waveSlotCapacity(sl.wave);
        std::vector<SegmentDesc> segs;
        std::vector<const DeviceScene*> scenes{lead->ds};
        sl.segments.clear();
        uint64_t paths = 0;
        for (Request* r : active_) {
            if ((int)segs.size() == kMaxSegmentsPerWave) break;
            if (r->samplesIssued >= r->settings.spp || r->cancelled || inFlightLocked(r)) continue;
            if (r->settings.volumetric != lead->settings.volumetric ||
                r->settings.max_depth != lead->settings.max_depth ||
                (r->settings.flags & SLRGPU_FLAG_WATERTIGHT) != (lead->settings.flags & SLRGPU_FLAG_WATERTIGHT))
                continue;
            if (cfg_.mode == SLRGPU_SERVER_PLAIN && r != lead) continue;
            uint32_t sceneIdx = 0;
            while (sceneIdx < scenes.size() && scenes[sceneIdx] != r->ds) ++sceneIdx;
            if (sceneIdx == scenes.size()) {
                if (!mixScenes || (int)scenes.size() == kMaxWaveScenesApi) continue;
                scenes.push_back(r->ds);
            }
            uint64_t room = (cap - paths) / r->gridPositions;
            if (room == 0) {
                if (sceneIdx + 1 == scenes.size() && sceneIdx > 0 && scenes.back() == r->ds) {
                    // nothing of this scene made it in
                    bool used = false;
                    for (const SegmentDesc &d : segs) used = used || d.scene == sceneIdx;
                    if (!used) scenes.pop_back();
                }
                break;
            }
            uint32_t take = (uint32_t)std::min<uint64_t>(room, r->settings.spp - r->samplesIssued);
            if (r->settings.samples_per_wave) take = std::min(take, r->settings.samples_per_wave);
            SegmentDesc d;
            d.width = r->settings.width;
            d.height = r->settings.height;
            d.sampleBase = r->settings.sample_base + r->samplesIssued;
            d.samples = take;
            d.seed = r->settings.seed;
            d.scene = sceneIdx;
            d.filmSum = r->filmSum;
            d.filmComp = r->filmComp;
            d.dropped = r->dropped;
            segs.push_back(d);
            r->samplesIssued += take;
            sl.segments.emplace_back(r, r->samplesIssued);
            paths += (uint64_t)take * r->gridPositions;
        }
        if (segs.empty()) break;
        TraceRange range("server wave %llu: %d requests", (unsigned long long)wavesLaunched_, (int)segs.size());
        uint64_t n = 0;
        int rc = SLRGPU_ERR_CUDA;
        if (takeFault(g_faultWaveLaunch))
            setError("injected wave launch failure");
        else
            rc = launchWave(scenes.data(), (int)scenes.size(), sl.wave, segs.data(), (int)segs.size(),
                            lead->settings.max_depth, lead->settings.volumetric != 0,
                            (lead->settings.flags & SLRGPU_FLAG_WATERTIGHT) != 0, sl.stream, &n,
                            cfg_.mode == SLRGPU_SERVER_BATCHED);
        if (rc != SLRGPU_OK) {
            for (auto &pr : sl.segments) failRequest(pr.first, "wave launch failed");
            sl.segments.clear();
            cvDone_.notify_all();
            continue;
        }
        cudaEventRecord(sl.event, sl.stream);
        sl.busy = true;
        sl.ds = lead->ds;
        ++wavesLaunched_;
        if (scenes.size() > 1) ++mixedWaves_;
        kernelLaunches_ += n;
        launched = true;
    }
    return launched;
}

// Completes the waves of finished slots; a request whose last sample is done
// gets its film converted on that slot's stream.  Holds mu_ (released while
// blocking on an event).
bool Server::reapSlots(bool block) {
    bool any = false;
    for (Slot &sl : slots_) {
        if (!sl.busy) continue;
        cudaError_t q = cudaEventQuery(sl.event);
        if (q == cudaErrorNotReady) continue;
        sl.busy = false;
        sl.ds = nullptr;
        any = true;
        if (q != cudaSuccess) {
            for (auto &pr : sl.segments) failRequest(pr.first, cudaGetErrorString(q));
            sl.segments.clear();
            cvDone_.notify_all();
            continue;
        }
        for (auto &pr : sl.segments) {
            Request* r = pr.first;
            r->samplesDone = std::max(r->samplesDone, pr.second);
            if (r->samplesDone == r->settings.spp && !r->finishing && !r->cancelled && r->status >= 0) {
                r->finishing = true;
                launchFilmToPixelMajor(r->filmSum, r->filmOut, r->pixels, sl.stream);
                cudaMemcpyAsync(&r->droppedHost, r->dropped, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                sl.stream);
                cudaEventRecord(r->doneEvent, sl.stream);
            }
        }
        sl.segments.clear();
    }
    (void)block;
    return any;
}

void Server::reapFinishing() {
    bool notify = false;
    for (size_t i = 0; i < active_.size();) {
        Request* r = active_[i];
        if (r->finishing && cudaEventQuery(r->doneEvent) == cudaSuccess) {
            r->status = SLRGPU_REQUEST_DONE;
            r->tDone = now();
            lastDone_ = r->tDone;
            ++requestsDone_;
            pathSamplesDone_ += (uint64_t)r->settings.spp * r->gridPositions;
            if (r->pin) r->pin->fetch_sub(1);
            r->pin = nullptr;
            active_.erase(active_.begin() + i);
            notify = true;
        } else {
            ++i;
        }
    }
    if (notify) cvDone_.notify_all();
}

void Server::worker() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lock(mu_);
    while (true) {
        if (stop_) break;
        expireDeadlinesLocked();
        admitLocked();
        bool launched = launchWaves();
        reapSlots(false);
        retireCancelledLocked();
        reapFinishing();
        bool busy = false;
        for (const Slot &sl : slots_) busy |= sl.busy;
        bool finishing = false;
        for (Request* r : active_) finishing |= r->finishing;
        if (!busy && !finishing && !launched) {
            // nothing on the GPU: sleep until a request arrives or budget frees
            cvWork_.wait_for(lock, std::chrono::milliseconds(50));
            continue;
        }
        if (!launched) {
            // wait for the GPU without holding the lock
            lock.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(50));
            lock.lock();
        }
    }
    // drain: finish what is on the GPU; queued requests are cancelled
    for (Slot &sl : slots_)
        if (sl.busy) cudaEventSynchronize(sl.event);
    for (Request* r : pending_) {
        r->status = SLRGPU_ERR_STATE;
        r->error = "server destroyed";
        if (r->pin) r->pin->fetch_sub(1);
        r->pin = nullptr;
    }
    pending_.clear();
    for (Request* r : active_) {
        if (r->finishing) cudaEventSynchronize(r->doneEvent);
        r->status = r->finishing ? SLRGPU_REQUEST_DONE : SLRGPU_ERR_STATE;
        if (!r->finishing) r->error = "server destroyed";
        if (r->pin) r->pin->fetch_sub(1);
        r->pin = nullptr;
    }
    active_.clear();
    cvDone_.notify_all();
}

}  // namespace slrgpu
