// slrgpu_renderer.hpp - the GPU renderer behind the reference's own C++
// renderer interface.
//
// Header-only; compiled into an application that links the reference's
// libSLR and slr_gb300's libslrgpu.so.  It needs libSLR's include directory
// and include/ of this repository on the include path.
//
// * SLRGPU::SceneBuilder mirrors the node-API calls that build an SLR::Scene
//   (spectra, surface materials, TriangleMeshNode, InfiniteSphereNode,
//   DensityGridMediumNode, the camera nodes) into a device scene: the
//   reference keeps its scene state private (Scene.h:23, material members,
//   SBVH::m_nodes), so the application calls both builders with the same
//   arguments ("tee" building).  commit() registers the device scene for the
//   SLR::Scene it mirrors.
// * SLRGPU::PathTracingRenderer and its volumetric / bidirectional variants
//   implement SLR::Renderer::render(const Scene&, const RenderSettings&)
//   (libSLR/Core/renderer.h:15-19) for PTRenderer(spp)
//   (Renderer/PTRenderer.h:42-43), VolumetricPTRenderer(spp)
//   (VolumetricPTRenderer.h:43-44), BPTRenderer(spp) and
//   VolumetricBPTRenderer(spp): they render the registered device scene and
//   write the film into the camera's ImageSensor (ImageSensor.h:47-48), so
//   saveImage() and everything downstream stay unchanged.
//
// Errors: the reference's render() returns void; these throw
// std::runtime_error with slrgpu_last_error()'s text instead.
#ifndef SLRGPU_RENDERER_HPP
#define SLRGPU_RENDERER_HPP

#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "Core/renderer.h"
#include "Core/RenderSettings.h"
#include "Core/camera.h"
#include "Core/ImageSensor.h"
#include "Scene/Scene.h"
#include "slrgpu.h"

namespace SLRGPU {

inline void check(int rc) {
    if (rc != SLRGPU_OK) throw std::runtime_error(std::string("slrgpu: ") + slrgpu_last_error());
}

// Device scenes registered for the SLR::Scene objects they mirror.
class Registry {
public:
    static void put(const SLR::Scene* scene, slrgpu_handle dev) {
        std::lock_guard<std::mutex> lock(mu());
        map()[scene] = dev;
    }
    static void erase(const SLR::Scene* scene) {
        std::lock_guard<std::mutex> lock(mu());
        map().erase(scene);
    }
    static slrgpu_handle get(const SLR::Scene* scene) {
        std::lock_guard<std::mutex> lock(mu());
        auto it = map().find(scene);
        if (it == map().end())
            throw std::runtime_error("slrgpu: no device scene registered for this SLR::Scene "
                                     "(build it with SLRGPU::SceneBuilder and commit())");
        return it->second;
    }
private:
    static std::map<const SLR::Scene*, slrgpu_handle> &map() {
        static std::map<const SLR::Scene*, slrgpu_handle> m;
        return m;
    }
    static std::mutex &mu() {
        static std::mutex m;
        return m;
    }
};

// Mirrors the reference's node constructors one to one.  Spectrum and
// material ids are returned in creation order, starting at 0.
class SceneBuilder {
public:
    // ctx: a context from slrgpu_context_create (one per GPU).
    explicit SceneBuilder(slrgpu_handle ctx) { check(slrgpu_scene_create(ctx, &m_scene)); }
    ~SceneBuilder() {
        if (m_registered) Registry::erase(m_registered);
        if (m_scene) slrgpu_scene_destroy(m_scene);
    }
    SceneBuilder(const SceneBuilder &) = delete;
    SceneBuilder &operator=(const SceneBuilder &) = delete;

    // UpsampledContinuousSpectrum(type, sRGB, r, g, b) (spectrum_types.h:188);
    // type 0 reflectance, 1 light source, 2 index of refraction.
    int rgbSpectrum(int type, float r, float g, float b) {
        int id;
        check(slrgpu_spectrum_rgb(m_scene, type, r, g, b, &id));
        return id;
    }
    // RegularContinuousSpectrum(minWL, maxWL, values, n) (spectrum_types.h:99).
    int regularSpectrum(float minWL, float maxWL, const float* values, uint32_t n) {
        int id;
        check(slrgpu_spectrum_regular(m_scene, minWL, maxWL, values, n, &id));
        return id;
    }
    // IrregularContinuousSpectrum(wavelengths, values, n).
    int irregularSpectrum(const float* wavelengths, const float* values, uint32_t n) {
        int id;
        check(slrgpu_spectrum_irregular(m_scene, wavelengths, values, n, &id));
        return id;
    }
    // DiffuseReflectionSurfaceMaterial (basic_surface_materials.h:20-27).
    int matte(int reflectance) {
        int id;
        check(slrgpu_material_matte(m_scene, reflectance, &id));
        return id;
    }
    // SpecularReflectionSurfaceMaterial(coeff, eta, k).
    int metal(int coeff, int eta, int k) {
        int id;
        check(slrgpu_material_specular_reflection(m_scene, coeff, eta, k, &id));
        return id;
    }
    // SpecularScatteringSurfaceMaterial(coeff, etaExt, etaInt).
    int glass(int coeff, int etaExt, int etaInt) {
        int id;
        check(slrgpu_material_specular_scattering(m_scene, coeff, etaExt, etaInt, &id));
        return id;
    }
    // MicrofacetReflectionSurfaceMaterial(eta, k, GGX(alphaX, alphaY))
    // (microfacet_surface_materials.h:21-28).
    int microfacetMetal(int eta, int k, float alphaX, float alphaY) {
        int id;
        check(slrgpu_material_microfacet_reflection(m_scene, eta, k, alphaX, alphaY, &id));
        return id;
    }
    // MicrofacetScatteringSurfaceMaterial(etaExt, etaInt, GGX(alphaX, alphaY)).
    int microfacetGlass(int etaExt, int etaInt, float alphaX, float alphaY) {
        int id;
        check(slrgpu_material_microfacet_scattering(m_scene, etaExt, etaInt, alphaX, alphaY, &id));
        return id;
    }
    // EmitterSurfaceMaterial(base, DiffuseEmitterSurfaceProperty(emittance)).
    int emitter(int baseMaterial, int emittance) {
        int id;
        check(slrgpu_material_emitter(m_scene, baseMaterial, emittance, &id));
        return id;
    }
    // TriangleMeshNode with one material group; call with the same world-space
    // vertices (positions, normals, tangents: 3 floats each; uvs: 2) and
    // triangle indices given to the reference's node.  uv may be null.
    void mesh(const float* pos, const float* nrm, const float* tan, const float* uv, uint32_t numVertices,
              const uint32_t* triangles, uint32_t numTriangles, int material) {
        check(slrgpu_scene_add_mesh(m_scene, pos, nrm, tan, uv, numVertices, triangles, numTriangles, material));
    }
    // InfiniteSphereNode(scene, IBL texture, scale) (node.h:125-141): the
    // environment image as width x height RGBA IEEE half-float texels, the
    // same texels the reference's RGBA16Fx4 image holds.
    void environment(const uint16_t* rgbaHalf, uint32_t width, uint32_t height, float scale) {
        check(slrgpu_environment_ibl(m_scene, rgbaHalf, width, height, scale));
    }
    // DensityGridMediumNode(region, sigma_s, sigma_e, density, nx, ny, nz,
    // HenyeyGreensteinScatteringMediumMaterial(g)) (medium_nodes.h:33-48);
    // density is [nz][ny][nx].
    void densityGridMedium(const float bmin[3], const float bmax[3], int sigmaS, int sigmaE, const float* density,
                           uint32_t nx, uint32_t ny, uint32_t nz, float g) {
        check(slrgpu_medium_density_grid(m_scene, bmin, bmax, sigmaS, sigmaE, density, nx, ny, nz, g));
    }
    // PerspectiveCameraNode(sensitivity, aspect, fovY, lensRadius, imgPDist,
    // objPDist) under the row-major camera-to-world transform
    // (camera_nodes.h:16-31).
    void perspectiveCamera(const float camToWorld[16], float sensitivity, float aspect, float fovY, float lensRadius,
                           float imgPlaneDist, float objPlaneDist) {
        check(slrgpu_camera_perspective(m_scene, camToWorld, sensitivity, aspect, fovY, lensRadius, imgPlaneDist,
                                        objPlaneDist));
    }
    // EquirectangularCameraNode(sensitivity, phiAngle, thetaAngle)
    // (camera_nodes.h:38-54).
    void equirectangularCamera(const float camToWorld[16], float sensitivity, float phiAngle, float thetaAngle) {
        check(slrgpu_camera_equirect(m_scene, camToWorld, sensitivity, phiAngle, thetaAngle));
    }
    // After SLR::Scene::build: builds the SBVH (the reference's tree), the
    // wide BVH and the light and environment tables, uploads them, and
    // registers the device scene for refScene.
    slrgpu_bvh_stats commit(const SLR::Scene* refScene) {
        slrgpu_bvh_stats st;
        check(slrgpu_scene_commit(m_scene, &st));
        Registry::put(refScene, m_scene);
        m_registered = refScene;
        return st;
    }
    slrgpu_handle handle() const { return m_scene; }

private:
    slrgpu_handle m_scene = 0;
    const SLR::Scene* m_registered = nullptr;
};

// SLR::Renderer over the GPU path tracers.  maxDepth is the number of
// scattering vertices at which next-event estimation and BSDF sampling run
// (the reference's path tracer stops at 100 vertices, PTRenderer.cpp:172);
// for the bidirectional tracers it caps each subpath.
class PathTracingRenderer : public SLR::Renderer {
public:
    explicit PathTracingRenderer(uint32_t spp, uint32_t maxDepth = 100, bool volumetric = false,
                                 uint32_t flags = 0)
        : m_spp(spp), m_maxDepth(maxDepth), m_volumetric(volumetric), m_flags(flags) {}

    // Renders with ImageWidth, ImageHeight and RNGSeed of the settings
    // (RenderSettings.h:15-23); NumThreads, TimeStart/TimeEnd (static scenes)
    // and Brightness (used only by the reference's progressive saveImage) do
    // not apply.  The camera's sensor is re-initialised, as the reference's
    // renderers do, and holds per pixel the 16-bin sums over all samples.
    void render(const SLR::Scene &scene, const SLR::RenderSettings &settings) const override {
        slrgpu_handle dev = Registry::get(&scene);
        slrgpu_settings s = {};
        s.width = (uint32_t)settings.getInt(SLR::RenderSettingItem::ImageWidth);
        s.height = (uint32_t)settings.getInt(SLR::RenderSettingItem::ImageHeight);
        s.spp = m_spp;
        s.max_depth = m_maxDepth;
        s.seed = (uint32_t)settings.getInt(SLR::RenderSettingItem::RNGSeed);
        s.volumetric = m_volumetric ? 1u : 0u;
        s.flags = m_flags;
        std::vector<float> film((size_t)s.width * s.height * 16);
        check(slrgpu_render(dev, &s, film.data(), 0, &m_lastStats));
        SLR::ImageSensor* sensor = scene.getCamera()->getSensor();
        sensor->init(s.width, s.height);
        for (uint32_t y = 0; y < s.height; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                // SpectrumStorage::getValue() is the pixel's compensated sum
                // (spectrum_types.h:716-739, CompensatedSum.h:16-33); its
                // members are set directly (its operator= does not compile
                // for DiscretizedSpectrum)
                SLR::CompensatedSum<SLR::DiscretizedSpectrum> &v = sensor->pixel(x, y).getValue();
                v.result = SLR::DiscretizedSpectrum(&film[((size_t)y * s.width + x) * 16]);
                v.comp = SLR::DiscretizedSpectrum(0.0f);
            }
    }
    // Statistics of the last render (path samples, rays, dropped samples).
    const slrgpu_render_stats &lastStats() const { return m_lastStats; }

private:
    uint32_t m_spp, m_maxDepth;
    bool m_volumetric;
    uint32_t m_flags;
    mutable slrgpu_render_stats m_lastStats = {};
};

// VolumetricPTRenderer(spp) (Renderer/VolumetricPTRenderer.h:43-44).
class VolumetricPathTracingRenderer : public PathTracingRenderer {
public:
    explicit VolumetricPathTracingRenderer(uint32_t spp, uint32_t maxDepth = 100)
        : PathTracingRenderer(spp, maxDepth, true) {}
};

// BPTRenderer(spp) (Renderer/BPTRenderer.h): the light-tracing connections
// are summed into the film, where the reference keeps them in the sensor's
// separated buffers (ImageSensor.cpp:132-137); they land in pixel() and the
// separated buffers stay empty.
class BidirectionalPathTracingRenderer : public PathTracingRenderer {
public:
    explicit BidirectionalPathTracingRenderer(uint32_t spp, uint32_t maxDepth = 32)
        : PathTracingRenderer(spp, maxDepth, false, SLRGPU_FLAG_BPT) {}
};

// VolumetricBPTRenderer(spp) (Renderer/VolumetricBPTRenderer.h).
class VolumetricBidirectionalPathTracingRenderer : public PathTracingRenderer {
public:
    explicit VolumetricBidirectionalPathTracingRenderer(uint32_t spp, uint32_t maxDepth = 32)
        : PathTracingRenderer(spp, maxDepth, true, SLRGPU_FLAG_BPT) {}
};

}  // namespace SLRGPU

#endif  // SLRGPU_RENDERER_HPP
