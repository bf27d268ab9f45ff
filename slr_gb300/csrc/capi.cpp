// C ABI of the GPU path tracer (declared in include/slrgpu.h).
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/slrgpu.h"
#include "render_api.h"
#include "scene_host.h"
#include "server.h"
#include "trace_ranges.h"

namespace slrgpu {

namespace {
thread_local std::string t_lastError;

struct Context {
    int device = 0;
    RenderEngine engine;
    std::mutex mu;
};

struct Scene {
    Context* ctx = nullptr;
    HostScene host;
    BuiltScene built;
    bool hostBuilt = false;
    DeviceScene dev;
    bool committed = false;
    std::atomic<int> inFlight{0};   // unfinished server requests
    std::mutex mu;
};

struct ServerRec {
    Context* ctx = nullptr;
    std::unique_ptr<Server> server;
};

std::mutex g_registryMu;
std::unordered_map<uint64_t, std::unique_ptr<Context>> g_contexts;
std::unordered_map<uint64_t, std::unique_ptr<Scene>> g_scenes;
std::unordered_map<uint64_t, std::unique_ptr<ServerRec>> g_servers;

ServerRec* findServer(slrgpu_handle h) {
    std::lock_guard<std::mutex> lock(g_registryMu);
    auto it = g_servers.find(h);
    return it == g_servers.end() ? nullptr : it->second.get();
}

Context* findContext(slrgpu_handle h) {
    std::lock_guard<std::mutex> lock(g_registryMu);
    auto it = g_contexts.find(h);
    return it == g_contexts.end() ? nullptr : it->second.get();
}

Scene* findScene(slrgpu_handle h) {
    std::lock_guard<std::mutex> lock(g_registryMu);
    auto it = g_scenes.find(h);
    return it == g_scenes.end() ? nullptr : it->second.get();
}

int fail(int code, const std::string &msg) {
    t_lastError = msg;
    return code;
}

#define GET_SCENE(var, h)                                                         \
    Scene* var = findScene(h);                                                    \
    if (!var) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid scene handle");     \
    std::lock_guard<std::mutex> var##_lock(var->mu);                              \
    if (var->committed || var->hostBuilt) {                                       \
        if (mutating) return fail(SLRGPU_ERR_STATE, "scene already committed");  \
    }

bool validSpectrum(const Scene* s, int id) { return id >= 0 && id < (int)s->host.spectra.size(); }
bool validMaterial(const Scene* s, int id) { return id >= 0 && id < (int)s->host.materials.size(); }

int addMaterial(Scene* s, const DevMaterial &m, int* id) {
    s->host.materials.push_back(m);
    if (id) *id = (int)s->host.materials.size() - 1;
    return SLRGPU_OK;
}

int ensureHostBuilt(Scene* s) {
    if (s->hostBuilt) return SLRGPU_OK;
    TraceRange range("scene build: SBVH, wide BVH, light and environment tables");
    std::string err;
    if (!buildScene(s->host, &s->built, &err)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, err);
    s->hostBuilt = true;
    return SLRGPU_OK;
}

void fillStats(const Scene* s, slrgpu_bvh_stats* st) {
    if (!st) return;
    st->num_triangles = (uint32_t)s->built.prims.size();
    st->num_fragments = s->built.sbvh.numFragments;
    st->depth = s->built.sbvh.depth;
    st->num_binary_nodes = (uint32_t)s->built.sbvh.nodes.size();
    st->num_wide_nodes = (uint32_t)s->built.wide.nodes.size();
    st->width = (uint32_t)kBvhWidth;
    st->sah_cost = s->built.sbvh.cost;
    st->build_seconds = s->built.buildSeconds;
}
}  // namespace

void setError(const std::string &msg) { t_lastError = msg; }

}  // namespace slrgpu

using namespace slrgpu;

extern "C" {

const char* slrgpu_last_error(void) { return t_lastError.c_str(); }

int slrgpu_version(void) { return 1; }

int slrgpu_context_create(int device, slrgpu_handle* ctx) {
    if (!ctx) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "ctx is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(SLRGPU_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= n) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    std::unique_ptr<Context> c(new Context());
    c->device = device;
    uint64_t h = (uint64_t)(uintptr_t)c.get();
    std::lock_guard<std::mutex> lock(g_registryMu);
    g_contexts[h] = std::move(c);
    *ctx = h;
    return SLRGPU_OK;
}

int slrgpu_context_queue_counts(slrgpu_handle ctx, uint32_t* counts, uint32_t capacity, uint32_t* rows) {
    if (!counts || !rows) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "counts and rows must not be NULL");
    Context* c = findContext(ctx);
    if (!c) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lock(c->mu);
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return c->engine.queueCounts(counts, capacity, rows);
}

int slrgpu_context_destroy(slrgpu_handle ctx) {
    std::unique_ptr<Context> c;
    {
        std::lock_guard<std::mutex> lock(g_registryMu);
        auto it = g_contexts.find(ctx);
        if (it == g_contexts.end()) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid context handle");
        for (auto &kv : g_scenes)
            if (kv.second->ctx == it->second.get()) return fail(SLRGPU_ERR_STATE, "context still has scenes");
        for (auto &kv : g_servers)
            if (kv.second->ctx == it->second.get()) return fail(SLRGPU_ERR_STATE, "context still has servers");
        c = std::move(it->second);
        g_contexts.erase(it);
    }
    cudaSetDevice(c->device);
    c->engine.release();
    return SLRGPU_OK;
}

int slrgpu_scene_create(slrgpu_handle ctx, slrgpu_handle* scene) {
    if (!scene) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "scene is NULL");
    Context* c = nullptr;
    if (ctx != 0) {
        c = findContext(ctx);
        if (!c) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid context handle");
    }
    std::unique_ptr<Scene> s(new Scene());
    s->ctx = c;
    uint64_t h = (uint64_t)(uintptr_t)s.get();
    std::lock_guard<std::mutex> lock(g_registryMu);
    g_scenes[h] = std::move(s);
    *scene = h;
    return SLRGPU_OK;
}

int slrgpu_scene_destroy(slrgpu_handle scene) {
    std::unique_ptr<Scene> s;
    {
        std::lock_guard<std::mutex> lock(g_registryMu);
        auto it = g_scenes.find(scene);
        if (it == g_scenes.end()) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid scene handle");
        if (it->second->inFlight.load() > 0) return fail(SLRGPU_ERR_STATE, "scene has unfinished server requests");
        s = std::move(it->second);
        g_scenes.erase(it);
    }
    if (s->ctx) cudaSetDevice(s->ctx->device);
    s->dev.buffers.release();
    return SLRGPU_OK;
}

int slrgpu_spectrum_rgb(slrgpu_handle scene, int spectrum_type, float r, float g, float b, int* id) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (spectrum_type < 0 || spectrum_type > 2) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad spectrum type");
    if (!std::isfinite(r) || !std::isfinite(g) || !std::isfinite(b))
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "non-finite RGB");
    s->host.spectra.push_back(upsampledFromRGB(spectrum_type, r, g, b));
    if (id) *id = (int)s->host.spectra.size() - 1;
    return SLRGPU_OK;
}

int slrgpu_spectrum_regular(slrgpu_handle scene, float min_wl, float max_wl, const float* values, uint32_t n, int* id) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!values || n < 2 || !(max_wl > min_wl)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad regular spectrum");
    DevSpectrum sp{};
    sp.kind = kSpecRegular;
    sp.offset = (uint32_t)s->host.specValues.size();
    sp.count = n;
    sp.p0 = min_wl;
    sp.p1 = max_wl;
    s->host.specValues.insert(s->host.specValues.end(), values, values + n);
    s->host.spectra.push_back(sp);
    if (id) *id = (int)s->host.spectra.size() - 1;
    return SLRGPU_OK;
}

int slrgpu_spectrum_irregular(slrgpu_handle scene, const float* wls, const float* values, uint32_t n, int* id) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!wls || !values || n < 2) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad irregular spectrum");
    for (uint32_t i = 1; i < n; ++i)
        if (!(wls[i] > wls[i - 1])) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "wavelengths must increase");
    DevSpectrum sp{};
    sp.kind = kSpecIrregular;
    sp.offset = (uint32_t)s->host.specValues.size();
    sp.count = n;
    s->host.specValues.insert(s->host.specValues.end(), wls, wls + n);
    s->host.specValues.insert(s->host.specValues.end(), values, values + n);
    s->host.spectra.push_back(sp);
    if (id) *id = (int)s->host.spectra.size() - 1;
    return SLRGPU_OK;
}

static int materialCommon(slrgpu_handle scene, uint32_t kind, int a, int b, int c, float ax, float ay, int nspec,
                          int* id) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    int sp[3] = {a, b, c};
    for (int i = 0; i < nspec; ++i)
        if (!validSpectrum(s, sp[i])) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "invalid spectrum id");
    if ((kind == kMatGGXReflection || kind == kMatGGXScattering) && !(ax > 0.0f && ay > 0.0f))
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "GGX roughness must be positive");
    DevMaterial m{};
    m.kind = kind;
    for (int i = 0; i < 3; ++i) m.spec[i] = i < nspec ? sp[i] : -1;
    m.alphaX = ax;
    m.alphaY = ay;
    m.emit = -1;
    return addMaterial(s, m, id);
}

int slrgpu_material_matte(slrgpu_handle scene, int reflectance, int* id) {
    return materialCommon(scene, kMatMatte, reflectance, -1, -1, 0, 0, 1, id);
}
int slrgpu_material_specular_reflection(slrgpu_handle scene, int coeff, int eta, int k, int* id) {
    return materialCommon(scene, kMatSpecularReflection, coeff, eta, k, 0, 0, 3, id);
}
int slrgpu_material_specular_scattering(slrgpu_handle scene, int coeff, int eta_ext, int eta_int, int* id) {
    return materialCommon(scene, kMatSpecularScattering, coeff, eta_ext, eta_int, 0, 0, 3, id);
}
int slrgpu_material_microfacet_reflection(slrgpu_handle scene, int eta, int k, float ax, float ay, int* id) {
    return materialCommon(scene, kMatGGXReflection, eta, k, -1, ax, ay, 2, id);
}
int slrgpu_material_microfacet_scattering(slrgpu_handle scene, int eta_ext, int eta_int, float ax, float ay, int* id) {
    return materialCommon(scene, kMatGGXScattering, eta_ext, eta_int, -1, ax, ay, 2, id);
}

int slrgpu_material_emitter(slrgpu_handle scene, int base_material, int emittance, int* id) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!validMaterial(s, base_material)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "invalid base material");
    if (!validSpectrum(s, emittance)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "invalid emittance spectrum");
    DevMaterial m = s->host.materials[base_material];
    if (m.emit >= 0) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "base material is already emitting");
    m.emit = emittance;
    return addMaterial(s, m, id);
}

int slrgpu_scene_add_mesh(slrgpu_handle scene, const float* positions, const float* normals, const float* tangents,
                          const float* uvs, uint32_t nv, const uint32_t* indices, uint32_t nt, int material) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!positions || !normals || !tangents || !indices || nv == 0)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "mesh arrays must not be NULL");
    if (!validMaterial(s, material)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "invalid material id");
    for (uint64_t i = 0; i < 3ull * nt; ++i)
        if (indices[i] >= nv) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "vertex index out of range");
    // a corrupted mesh (NaN or infinite positions) would poison the BVH's
    // bounds for every ray of the scene; the reference does not check
    for (uint64_t i = 0; i < 3ull * nv; ++i)
        if (!std::isfinite(positions[i]))
            return fail(SLRGPU_ERR_INVALID_ARGUMENT, "vertex positions must be finite");
    uint64_t total = 0;
    for (const HostMesh &m : s->host.meshes) total += m.idx.size() / 3;
    if (total + nt >= (1ull << 26)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "too many triangles (limit 2^26)");
    HostMesh m;
    m.pos.assign(positions, positions + 3 * (size_t)nv);
    m.nrm.assign(normals, normals + 3 * (size_t)nv);
    m.tan.assign(tangents, tangents + 3 * (size_t)nv);
    if (uvs) m.uv.assign(uvs, uvs + 2 * (size_t)nv);
    else m.uv.assign(2 * (size_t)nv, 0.0f);
    m.idx.assign(indices, indices + 3 * (size_t)nt);
    m.material = material;
    s->host.meshes.push_back(std::move(m));
    return SLRGPU_OK;
}

int slrgpu_environment_ibl(slrgpu_handle scene, const uint16_t* rgba_half, uint32_t w, uint32_t h, float scale) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!rgba_half || w < 4 || h < 4) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "environment must be at least 4x4");
    s->host.envPresent = true;
    s->host.envRGBA.assign(rgba_half, rgba_half + 4 * (size_t)w * h);
    s->host.envW = w;
    s->host.envH = h;
    s->host.envScale = scale;
    return SLRGPU_OK;
}

int slrgpu_medium_density_grid(slrgpu_handle scene, const float* bmin, const float* bmax, int sigma_s, int sigma_e,
                               const float* density, uint32_t nx, uint32_t ny, uint32_t nz, float hg_g) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!bmin || !bmax || !density || nx < 2 || ny < 2 || nz < 2)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad density grid");
    if (!validSpectrum(s, sigma_s) || !validSpectrum(s, sigma_e))
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "invalid coefficient spectrum");
    HostMedium &m = s->host.medium;
    m.present = true;
    for (int k = 0; k < 3; ++k) { m.bmin[k] = bmin[k]; m.bmax[k] = bmax[k]; }
    m.sigmaS = sigma_s;
    m.sigmaE = sigma_e;
    m.nx = nx; m.ny = ny; m.nz = nz;
    m.density.assign(density, density + (size_t)nx * ny * nz);
    m.g = hg_g;
    return SLRGPU_OK;
}

int slrgpu_medium_density_grid_file(slrgpu_handle scene, const char* path, const float* bmin, const float* bmax,
                                    int sigma_s, int sigma_e, float hg_g) {
    if (!path) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "path is NULL");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(SLRGPU_ERR_INVALID_ARGUMENT, std::string("failed to read density grid file: ") + path);
    uint32_t n[3] = {0, 0, 0};
    bool ok = std::fread(n, sizeof(uint32_t), 3, fp) == 3 && n[0] >= 2 && n[1] >= 2 && n[2] >= 2 &&
              (uint64_t)n[0] * n[1] * n[2] <= (1ull << 32);
    std::vector<float> density;
    if (ok) {
        density.resize((size_t)n[0] * n[1] * n[2]);
        ok = std::fread(density.data(), sizeof(float), density.size(), fp) == density.size();
    }
    std::fclose(fp);
    if (!ok) return fail(SLRGPU_ERR_INVALID_ARGUMENT, std::string("malformed density grid file: ") + path);
    return slrgpu_medium_density_grid(scene, bmin, bmax, sigma_s, sigma_e, density.data(), n[0], n[1], n[2], hg_g);
}

int slrgpu_camera_perspective(slrgpu_handle scene, const float* m, float sensitivity, float aspect, float fov_y,
                              float lens_radius, float img_dist, float obj_dist) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!m || !(aspect > 0) || !(fov_y > 0) || !(img_dist > 0) || !(obj_dist > 0) || lens_radius < 0)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad perspective camera");
    s->host.cameraPresent = true;
    s->host.cameraKind = 0;
    std::memcpy(s->host.camMatrix, m, 16 * sizeof(float));
    s->host.camSensitivity = sensitivity;
    s->host.camAspect = aspect;
    s->host.camFovY = fov_y;
    s->host.camLensRadius = lens_radius;
    s->host.camImgDist = img_dist;
    s->host.camObjDist = obj_dist;
    return SLRGPU_OK;
}

int slrgpu_camera_equirect(slrgpu_handle scene, const float* m, float sensitivity, float phi_angle, float theta_angle) {
    const bool mutating = true;
    GET_SCENE(s, scene);
    if (!m || !(phi_angle > 0) || !(theta_angle > 0)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad equirect camera");
    s->host.cameraPresent = true;
    s->host.cameraKind = 1;
    std::memcpy(s->host.camMatrix, m, 16 * sizeof(float));
    s->host.camSensitivity = sensitivity;
    s->host.camPhiAngle = phi_angle;
    s->host.camThetaAngle = theta_angle;
    return SLRGPU_OK;
}

int slrgpu_scene_build_host(slrgpu_handle scene, slrgpu_bvh_stats* stats) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    int rc = ensureHostBuilt(s);
    if (rc != SLRGPU_OK) return rc;
    fillStats(s, stats);
    return SLRGPU_OK;
}

int slrgpu_scene_commit(slrgpu_handle scene, slrgpu_bvh_stats* stats) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!s->ctx) return fail(SLRGPU_ERR_STATE, "scene has no context");
    int rc = ensureHostBuilt(s);
    if (rc != SLRGPU_OK) return rc;
    if (!s->committed) {
        cudaError_t e = cudaSetDevice(s->ctx->device);
        if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
        TraceRange range("scene upload");
        rc = uploadScene(s->host, s->built, &s->dev);
        if (rc != SLRGPU_OK) return rc;
        s->committed = true;
    }
    fillStats(s, stats);
    return SLRGPU_OK;
}

int slrgpu_scene_reupload(slrgpu_handle scene, uint64_t* bytes) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    std::lock_guard<std::mutex> lock(s->ctx->mu);
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return reuploadScene(&s->dev, bytes, 0);
}

int slrgpu_render(slrgpu_handle scene, const slrgpu_settings* settings, float* film, int film_on_device,
                  slrgpu_render_stats* stats) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!settings || !film) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "settings and film must not be NULL");
    if (int rc = checkImageSize(settings->width, settings->height)) return rc;
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (!s->host.cameraPresent) return fail(SLRGPU_ERR_STATE, "scene has no camera");
    if (settings->volumetric && !s->host.medium.present)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "volumetric render of a scene without medium");
    std::lock_guard<std::mutex> lock(s->ctx->mu);
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return s->ctx->engine.render(s->dev, *settings, film, film_on_device != 0, stats, 0);
}

int slrgpu_render_continue(slrgpu_handle scene, const slrgpu_settings* settings, float* film_state, float* film,
                           slrgpu_render_stats* stats) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!settings || !film_state) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "settings and film_state must not be NULL");
    if (int rc = checkImageSize(settings->width, settings->height)) return rc;
    if (settings->flags & SLRGPU_FLAG_BPT)
        return fail(SLRGPU_ERR_UNSUPPORTED, "continuing a film is supported for the path tracers only");
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (!s->host.cameraPresent) return fail(SLRGPU_ERR_STATE, "scene has no camera");
    if (settings->volumetric && !s->host.medium.present)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "volumetric render of a scene without medium");
    std::lock_guard<std::mutex> lock(s->ctx->mu);
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return s->ctx->engine.render(s->dev, *settings, film, false, stats, 0, film_state);
}

int slrgpu_render_replay(slrgpu_handle scene, const slrgpu_settings* settings, const float* tapes, float* film,
                         slrgpu_render_stats* stats) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!settings || !tapes || !film) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "settings, tapes and film must not be NULL");
    if (int rc = checkImageSize(settings->width, settings->height)) return rc;
    if (settings->spp != 1 || settings->sample_base != 0 || settings->volumetric ||
        (settings->flags & (SLRGPU_FLAG_BPT | SLRGPU_FLAG_WATERTIGHT)))
        return fail(SLRGPU_ERR_UNSUPPORTED, "replay renders one sample of the surface path tracer");
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (!s->host.cameraPresent) return fail(SLRGPU_ERR_STATE, "scene has no camera");
    std::lock_guard<std::mutex> lock(s->ctx->mu);
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    const size_t n = (size_t)sampleGridPositions(settings->width, settings->height) * kRngTapeFloats;
    float* dev = nullptr;
    if ((e = cudaMalloc(&dev, n * sizeof(float))) != cudaSuccess) return fail(SLRGPU_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
    int rc = SLRGPU_OK;
    if ((e = cudaMemcpy(dev, tapes, n * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
        rc = fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    else
        rc = s->ctx->engine.render(s->dev, *settings, film, false, stats, 0, nullptr, dev);
    cudaFree(dev);
    return rc;
}

int slrgpu_render_noalloc(slrgpu_handle scene, const slrgpu_settings* settings, float* film_device, void* stream) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!settings || !film_device) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "settings and film must not be NULL");
    if (int rc = checkImageSize(settings->width, settings->height)) return rc;
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (!s->host.cameraPresent) return fail(SLRGPU_ERR_STATE, "scene has no camera");
    if (settings->volumetric && !s->host.medium.present)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "volumetric render of a scene without medium");
    if (settings->flags & SLRGPU_FLAG_BPT)
        return fail(SLRGPU_ERR_UNSUPPORTED, "the allocation-free render has no bidirectional path tracer");
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return renderNoAlloc(s->dev, *settings, film_device, (cudaStream_t)stream);
}

uint64_t slrgpu_render_noalloc_scratch_bytes(void) { return (uint64_t)noAllocScratchBytes(); }

int slrgpu_trace(slrgpu_handle scene, const float* rays, uint32_t n, int any_hit, uint32_t* prim, float* t, float* b1,
                 float* b2, void* stream) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (n > 0 && (!rays || !prim)) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "rays and prim must not be NULL");
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return traceRays(s->dev, rays, n, any_hit, prim, t, b1, b2, (cudaStream_t)stream);
}

int slrgpu_bsdf_query(int kind, const float* spec0, const float* spec1, const float* spec2, float alpha_x,
                      float alpha_y, const float* queries, uint32_t n, float* out) {
    if (!spec0 || (n > 0 && (!queries || !out))) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return bsdfQuery(kind, spec0, spec1, spec2, alpha_x, alpha_y, queries, n, out);
}

int slrgpu_medium_query(slrgpu_handle scene, int mode, uint32_t n, const float* rays, const float* lambdas,
                        const int* sel, const uint32_t* vals, uint32_t num_vals, float* out) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (n > 0 && (!rays || !lambdas || !sel || !out || (num_vals > 0 && !vals)))
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaError_t e = cudaSetDevice(s->ctx->device);
    if (e != cudaSuccess) return fail(SLRGPU_ERR_CUDA, cudaGetErrorString(e));
    return mediumQuery(s->dev, mode, n, rays, lambdas, sel, vals, num_vals, out);
}

// ---- serving -------------------------------------------------------------------
int slrgpu_server_create(slrgpu_handle ctx, const slrgpu_server_config* config, slrgpu_handle* server) {
    if (!server) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "server is NULL");
    Context* c = findContext(ctx);
    if (!c) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid context handle");
    slrgpu_server_config cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    if (config) cfg = *config;
    std::unique_ptr<ServerRec> rec(new ServerRec());
    rec->ctx = c;
    rec->server.reset(new Server(c->device, cfg));
    int rc = rec->server->init();
    if (rc != SLRGPU_OK) return rc;
    uint64_t h = (uint64_t)(uintptr_t)rec.get();
    std::lock_guard<std::mutex> lock(g_registryMu);
    g_servers[h] = std::move(rec);
    *server = h;
    return SLRGPU_OK;
}

int slrgpu_server_destroy(slrgpu_handle server) {
    std::unique_ptr<ServerRec> rec;
    {
        std::lock_guard<std::mutex> lock(g_registryMu);
        auto it = g_servers.find(server);
        if (it == g_servers.end()) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
        rec = std::move(it->second);
        g_servers.erase(it);
    }
    rec->server.reset();
    return SLRGPU_OK;
}

int slrgpu_server_submit(slrgpu_handle server, slrgpu_handle scene, const slrgpu_settings* settings,
                         uint64_t* request) {
    ServerRec* rec = findServer(server);
    if (!rec) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
    if (!settings || !request) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "settings and request must not be NULL");
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!s->committed) return fail(SLRGPU_ERR_NOT_COMMITTED, "scene not committed");
    if (s->ctx != rec->ctx) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "scene belongs to another context");
    if (!s->host.cameraPresent) return fail(SLRGPU_ERR_STATE, "scene has no camera");
    if (settings->volumetric && !s->host.medium.present)
        return fail(SLRGPU_ERR_INVALID_ARGUMENT, "volumetric render of a scene without medium");
    if (settings->flags & SLRGPU_FLAG_BPT)
        return fail(SLRGPU_ERR_UNSUPPORTED, "the server renders with the path tracers only");
    return rec->server->submit(&s->dev, &s->inFlight, *settings, request);
}

int slrgpu_server_poll(slrgpu_handle server, uint64_t request, slrgpu_request_info* info) {
    ServerRec* rec = findServer(server);
    if (!rec) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
    return rec->server->poll(request, info);
}

int slrgpu_server_wait(slrgpu_handle server, uint64_t request, float* film, slrgpu_request_info* info,
                       double timeout_seconds) {
    ServerRec* rec = findServer(server);
    if (!rec) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
    return rec->server->wait(request, film, info, timeout_seconds);
}

int slrgpu_server_get_stats(slrgpu_handle server, slrgpu_server_stats* stats) {
    ServerRec* rec = findServer(server);
    if (!rec) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
    if (!stats) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "stats is NULL");
    rec->server->stats(stats);
    return SLRGPU_OK;
}

int slrgpu_server_cancel(slrgpu_handle server, uint64_t request) {
    ServerRec* rec = findServer(server);
    if (!rec) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
    return rec->server->cancel(request);
}

int slrgpu_server_set_deadline(slrgpu_handle server, uint64_t request, double seconds) {
    ServerRec* rec = findServer(server);
    if (!rec) return fail(SLRGPU_ERR_INVALID_HANDLE, "invalid server handle");
    return rec->server->setDeadline(request, seconds);
}

int slrgpu_debug_inject_fault(int site, uint32_t count) { return injectFault(site, count); }

// ---- film output ---------------------------------------------------------------
int slrgpu_film_to_bmp(const float* film, uint32_t width, uint32_t height, int film_on_device, float scale,
                       float sensitivity, uint8_t* pixels, const char* path) {
    if (!film) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "film is NULL");
    if (width == 0 || height == 0) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "width and height must be positive");
    const uint32_t rowBytes = 3 * width + width % 4;
    std::vector<uint8_t> buf((size_t)rowBytes * height);
    int rc = filmToBmp(film, width, height, film_on_device != 0, scale, sensitivity, buf.data());
    if (rc != SLRGPU_OK) return rc;
    if (pixels) std::memcpy(pixels, buf.data(), buf.size());
    if (path) {
        // 54-byte BITMAPFILEHEADER + BITMAPINFOHEADER, 24 bits, no compression,
        // 1 pixel per metre (Helper/bmp_exporter.cpp:15-53).
        uint8_t header[54];
        std::memset(header, 0, sizeof(header));
        auto put32 = [&](int off, uint32_t v) { for (int k = 0; k < 4; ++k) header[off + k] = (uint8_t)(v >> (8 * k)); };
        auto put16 = [&](int off, uint16_t v) { header[off] = (uint8_t)v; header[off + 1] = (uint8_t)(v >> 8); };
        header[0] = 'B';
        header[1] = 'M';
        put32(2, (uint32_t)buf.size() + 54);
        put32(10, 54);
        put32(14, 40);
        put32(18, width);
        put32(22, height);
        put16(26, 1);
        put16(28, 24);
        put32(30, 0);
        put32(34, (uint32_t)buf.size());
        put32(38, 1);
        put32(42, 1);
        FILE* fp = std::fopen(path, "wb");
        if (!fp) return fail(SLRGPU_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
        bool ok = std::fwrite(header, 1, sizeof(header), fp) == sizeof(header) &&
                  std::fwrite(buf.data(), 1, buf.size(), fp) == buf.size();
        std::fclose(fp);
        if (!ok) return fail(SLRGPU_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    }
    return SLRGPU_OK;
}

int slrgpu_film_cmf(float* bins, float* integral) {
    if (!bins || !integral) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    discretizedCmf(bins, bins + 16, bins + 32, integral);
    return SLRGPU_OK;
}

// ---- host-side diagnostics ----------------------------------------------------
int slrgpu_scene_sbvh_dump(slrgpu_handle scene, float* boxes, uint32_t* words, uint32_t* leaf_prims) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    int rc = ensureHostBuilt(s);
    if (rc != SLRGPU_OK) return rc;
    const SbvhResult &b = s->built.sbvh;
    for (size_t i = 0; i < b.nodes.size(); ++i) {
        const SbvhNode &n = b.nodes[i];
        if (boxes)
            for (int k = 0; k < 3; ++k) { boxes[6 * i + k] = n.bmin[k]; boxes[6 * i + 3 + k] = n.bmax[k]; }
        if (words) {
            words[5 * i + 0] = n.c0; words[5 * i + 1] = n.c1;
            words[5 * i + 2] = n.offset; words[5 * i + 3] = n.count;
            words[5 * i + 4] = n.leaf ? 0xffffffffu : n.axis;
        }
    }
    if (leaf_prims) std::memcpy(leaf_prims, b.leafPrims.data(), b.leafPrims.size() * sizeof(uint32_t));
    return SLRGPU_OK;
}

int slrgpu_spectrum_evaluate(slrgpu_handle scene, int id, const float* lambdas, uint32_t num_sets, float* out) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!validSpectrum(s, id) || !lambdas || !out) return fail(SLRGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    for (uint32_t i = 0; i < num_sets; ++i)
        evaluateSpectrum(s->host.spectra[id], s->host.specValues.data(), lambdas + 16 * (size_t)i, out + 16 * (size_t)i);
    return SLRGPU_OK;
}

int slrgpu_environment_tables(slrgpu_handle scene, uint32_t* map_w, uint32_t* map_h, float* row_pdf, float* row_cdf,
                              float* top_pdf, float* top_cdf, float* texel_params) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    if (!s->host.envPresent) return fail(SLRGPU_ERR_STATE, "scene has no environment");
    int rc = ensureHostBuilt(s);
    if (rc != SLRGPU_OK) return rc;
    const HostEnvironment &e = s->built.env;
    if (map_w) *map_w = e.mapW;
    if (map_h) *map_h = e.mapH;
    if (row_pdf) std::memcpy(row_pdf, e.rowPDF.data(), e.rowPDF.size() * sizeof(float));
    if (row_cdf) std::memcpy(row_cdf, e.rowCDF.data(), e.rowCDF.size() * sizeof(float));
    if (top_pdf) std::memcpy(top_pdf, e.topPDF.data(), e.topPDF.size() * sizeof(float));
    if (top_cdf) std::memcpy(top_cdf, e.topCDF.data(), e.topCDF.size() * sizeof(float));
    if (texel_params) std::memcpy(texel_params, e.texels.data(), e.texels.size() * sizeof(EnvTexel));
    return SLRGPU_OK;
}

int slrgpu_scene_alias_tables(slrgpu_handle scene, uint32_t* num_lights, float* light_prob, uint32_t* light_alias,
                              float* top_prob, uint32_t* top_alias, float* row_prob, uint32_t* row_alias) {
    const bool mutating = false;
    GET_SCENE(s, scene);
    int rc = ensureHostBuilt(s);
    if (rc != SLRGPU_OK) return rc;
    auto split = [](const std::vector<AliasEntry> &t, float* prob, uint32_t* alias) {
        for (size_t i = 0; i < t.size(); ++i) {
            if (prob) prob[i] = t[i].prob;
            if (alias) alias[i] = t[i].alias;
        }
    };
    if (num_lights) *num_lights = (uint32_t)s->built.lightAlias.size();
    split(s->built.lightAlias, light_prob, light_alias);
    split(s->built.env.topAlias, top_prob, top_alias);
    split(s->built.env.rowAlias, row_prob, row_alias);
    return SLRGPU_OK;
}

}  // extern "C"
