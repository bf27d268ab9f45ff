// A test application of the C++ shim (include/slrgpu_renderer.hpp): it builds
// each scene twice with the same calls, once through the reference's node API
// (the oracle driver's ora_* functions, oracle/ref_driver.cpp) and once
// through SLRGPU::SceneBuilder, and renders the reference's SLR::Scene
// through an SLR::Renderer reference bound to the GPU renderers.  TEST
// INFRASTRUCTURE ONLY (tests/test_gpu_shim.py).  The app_* functions take the
// ora_* functions' arguments, so oracle.RefScene can drive them.
#include <cstdint>
#include <cstring>
#include <memory>

#include "slrgpu_renderer.hpp"

extern "C" {
void* ora_scene_new();
void ora_scene_free(void* p);
int ora_spectrum_rgb(void* p, int spType, float r, float g, float b);
int ora_spectrum_regular(void* p, float minWL, float maxWL, const float* vals, int n);
int ora_spectrum_irregular(void* p, const float* wls, const float* vals, int n);
int ora_material_matte(void* p, int refl);
int ora_material_specular_reflection(void* p, int coeff, int eta, int k);
int ora_material_specular_scattering(void* p, int coeff, int etaExt, int etaInt);
int ora_material_microfacet_reflection(void* p, int eta, int k, float ax, float ay);
int ora_material_microfacet_scattering(void* p, int etaExt, int etaInt, float ax, float ay);
int ora_material_emitter(void* p, int baseMat, int emittance);
int ora_mesh(void* p, const float* pos, const float* nrm, const float* tan, const float* uv, int nv,
             const uint32_t* idx, int ntri, int material);
int ora_env_ibl(void* p, const uint16_t* rgbaHalf, int w, int h, float scale);
int ora_medium_density_grid(void* p, const float* bmin, const float* bmax, int sigmaS, int sigmaE,
                            const float* density, int nx, int ny, int nz, float g);
int ora_camera_perspective(void* p, const float* m, float sensitivity, float aspect, float fovY, float lensRadius,
                           float imgPDist, float objPDist);
int ora_camera_equirect(void* p, const float* m, float sensitivity, float phiAngle, float thetaAngle);
int ora_build(void* p);
void* ora_scene_ptr(void* p);
}

namespace {
struct App {
    void* ref = nullptr;
    slrgpu_handle ctx = 0;
    std::unique_ptr<SLRGPU::SceneBuilder> gpu;
    ~App() {
        gpu.reset();
        if (ctx) slrgpu_context_destroy(ctx);
        if (ref) ora_scene_free(ref);
    }
};

// Both builders must hand out the same ids.
int same(int a, int b) { return a == b ? a : -100; }

template <typename F>
int guarded(F f) {
    try {
        return f();
    } catch (const std::exception &) {
        return -101;
    }
}
}  // namespace

extern "C" {

void* app_scene_new() {
    App* a = new App();
    a->ref = ora_scene_new();
    if (slrgpu_context_create(0, &a->ctx) != SLRGPU_OK) {
        delete a;
        return nullptr;
    }
    a->gpu.reset(new SLRGPU::SceneBuilder(a->ctx));
    return a;
}

void app_scene_free(void* p) { delete (App*)p; }

int app_spectrum_rgb(void* p, int t, float r, float g, float b) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_spectrum_rgb(a->ref, t, r, g, b), a->gpu->rgbSpectrum(t, r, g, b)); });
}
int app_spectrum_regular(void* p, float lo, float hi, const float* v, int n) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_spectrum_regular(a->ref, lo, hi, v, n), a->gpu->regularSpectrum(lo, hi, v, n)); });
}
int app_spectrum_irregular(void* p, const float* w, const float* v, int n) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_spectrum_irregular(a->ref, w, v, n), a->gpu->irregularSpectrum(w, v, n)); });
}
int app_material_matte(void* p, int r) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_material_matte(a->ref, r), a->gpu->matte(r)); });
}
int app_material_specular_reflection(void* p, int c, int e, int k) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_material_specular_reflection(a->ref, c, e, k), a->gpu->metal(c, e, k)); });
}
int app_material_specular_scattering(void* p, int c, int e0, int e1) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_material_specular_scattering(a->ref, c, e0, e1), a->gpu->glass(c, e0, e1)); });
}
int app_material_microfacet_reflection(void* p, int e, int k, float ax, float ay) {
    App* a = (App*)p;
    return guarded([&] {
        return same(ora_material_microfacet_reflection(a->ref, e, k, ax, ay), a->gpu->microfacetMetal(e, k, ax, ay));
    });
}
int app_material_microfacet_scattering(void* p, int e0, int e1, float ax, float ay) {
    App* a = (App*)p;
    return guarded([&] {
        return same(ora_material_microfacet_scattering(a->ref, e0, e1, ax, ay), a->gpu->microfacetGlass(e0, e1, ax, ay));
    });
}
int app_material_emitter(void* p, int base, int em) {
    App* a = (App*)p;
    return guarded([&] { return same(ora_material_emitter(a->ref, base, em), a->gpu->emitter(base, em)); });
}
int app_mesh(void* p, const float* pos, const float* nrm, const float* tan, const float* uv, int nv,
             const uint32_t* idx, int ntri, int material) {
    App* a = (App*)p;
    return guarded([&] {
        int r = ora_mesh(a->ref, pos, nrm, tan, uv, nv, idx, ntri, material);
        a->gpu->mesh(pos, nrm, tan, uv, (uint32_t)nv, idx, (uint32_t)ntri, material);
        return r;
    });
}
int app_env_ibl(void* p, const uint16_t* rgba, int w, int h, float scale) {
    App* a = (App*)p;
    return guarded([&] {
        a->gpu->environment(rgba, (uint32_t)w, (uint32_t)h, scale);
        return ora_env_ibl(a->ref, rgba, w, h, scale);
    });
}
int app_medium_density_grid(void* p, const float* bmin, const float* bmax, int ss, int se, const float* d, int nx,
                            int ny, int nz, float g) {
    App* a = (App*)p;
    return guarded([&] {
        a->gpu->densityGridMedium(bmin, bmax, ss, se, d, (uint32_t)nx, (uint32_t)ny, (uint32_t)nz, g);
        return ora_medium_density_grid(a->ref, bmin, bmax, ss, se, d, nx, ny, nz, g);
    });
}
int app_camera_perspective(void* p, const float* m, float sens, float aspect, float fovY, float lens, float ipd,
                           float opd) {
    App* a = (App*)p;
    return guarded([&] {
        a->gpu->perspectiveCamera(m, sens, aspect, fovY, lens, ipd, opd);
        return ora_camera_perspective(a->ref, m, sens, aspect, fovY, lens, ipd, opd);
    });
}
int app_camera_equirect(void* p, const float* m, float sens, float phi, float theta) {
    App* a = (App*)p;
    return guarded([&] {
        a->gpu->equirectangularCamera(m, sens, phi, theta);
        return ora_camera_equirect(a->ref, m, sens, phi, theta);
    });
}
int app_build(void* p) {
    App* a = (App*)p;
    return guarded([&] {
        int r = ora_build(a->ref);
        a->gpu->commit((const SLR::Scene*)ora_scene_ptr(a->ref));
        return r;
    });
}
// Builds the reference's scene only: its device twin is never committed, so
// the shim has no device scene registered for it.
int app_build_reference_only(void* p) { return ora_build(((App*)p)->ref); }

// The device scene, for rendering the same scene through slrgpu_render.
uint64_t app_device_scene(void* p) { return ((App*)p)->gpu->handle(); }

// kind: 0 PTRenderer, 1 VolumetricPTRenderer, 2 BPTRenderer, 3 VolumetricBPTRenderer.
// Renders through a const SLR::Renderer& and copies the camera sensor's
// pixels (16 bins each, row-major) to film.
int app_render(void* p, int kind, int spp, int maxDepth, int w, int h, int seed, float* film,
               unsigned long long* dropped) {
    App* a = (App*)p;
    return guarded([&] {
        std::unique_ptr<SLRGPU::PathTracingRenderer> r;
        if (kind == 0) r.reset(new SLRGPU::PathTracingRenderer(spp, maxDepth));
        else if (kind == 1) r.reset(new SLRGPU::VolumetricPathTracingRenderer(spp, maxDepth));
        else if (kind == 2) r.reset(new SLRGPU::BidirectionalPathTracingRenderer(spp, maxDepth));
        else r.reset(new SLRGPU::VolumetricBidirectionalPathTracingRenderer(spp, maxDepth));
        const SLR::Renderer &renderer = *r;
        SLR::RenderSettings settings;
        settings.addItem(SLR::RenderSettingItem::NumThreads, (int32_t)1);
        settings.addItem(SLR::RenderSettingItem::ImageWidth, (int32_t)w);
        settings.addItem(SLR::RenderSettingItem::ImageHeight, (int32_t)h);
        settings.addItem(SLR::RenderSettingItem::TimeStart, 0.0f);
        settings.addItem(SLR::RenderSettingItem::TimeEnd, 0.0f);
        settings.addItem(SLR::RenderSettingItem::Brightness, 1.0f);
        settings.addItem(SLR::RenderSettingItem::RNGSeed, (int32_t)seed);
        const SLR::Scene* scene = (const SLR::Scene*)ora_scene_ptr(a->ref);
        if (!scene) return -102;
        renderer.render(*scene, settings);
        SLR::ImageSensor* sensor = scene->getCamera()->getSensor();
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                SLR::DiscretizedSpectrum v = sensor->pixel(x, y).getValue().result;
                for (int i = 0; i < 16; ++i) film[((size_t)y * w + x) * 16 + i] = v[i];
            }
        if (dropped) *dropped = r->lastStats().dropped_samples;
        return 0;
    });
}
}
