// CPU oracle driver for SLR's path tracer.  TEST INFRASTRUCTURE ONLY.
//
// It builds scenes through the reference's own public node API
// (libSLR/Scene/TriangleMeshNode.h:37-73, Scene/node.h:42-66,
// Scene/camera_nodes.h:16-54, Scene/node.h:125-141) from plain arrays, and
// exposes extern "C" entry points so that tests and the CPU-baseline leg of
// bench.py can run, through ctypes:
//   * the reference renderers PTRenderer / VolumetricPTRenderer
//     (libSLR/Renderer/PTRenderer.cpp:26-101) and BPTRenderer
//     (libSLR/Renderer/BPTRenderer.cpp:25-101) and read back the 16-bin film;
//   * the reference SBVH (libSLR/Accelerator/SBVH.h:380-496) on explicit ray
//     sets (closest hit and any hit), plus its node dump for build parity;
//   * the reference BSDFs at fixed queries (libSLR/BSDF/*.cpp).
// The friend declaration `friend class QBVH;` in SBVH.h:19 lets the
// inspector class below (named SLR::QBVH, a class nothing else defines
// once the QBVH header include is dropped) read the built SBVH node arrays.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "defines.h"
#include "declarations.h"
#include "BasicTypes/spectrum_base.h"
#include "BasicTypes/spectrum_types.h"
#include "BasicTypes/spectrum_library.h"
#include "Core/geometry.h"
#include "Core/transform.h"
#include "Core/textures.h"
#include "Core/image_2d.h"
#include "Core/camera.h"
#include "Core/ImageSensor.h"
#include "Core/RenderSettings.h"
#include "Core/light_path_sampler.h"
#include "Core/surface_material.h"
#include "Core/surface_object.h"
#include "Core/directional_distribution_functions.h"
#include "Core/distributions.h"
#include "Accelerator/SBVH.h"
#include "MemoryAllocators/ArenaAllocator.h"
#include "Scene/Scene.h"
#include "Scene/node.h"
#include "Scene/TriangleMeshNode.h"
#include "Scene/camera_nodes.h"
#include "Scene/medium_nodes.h"
#include "MediumDistribution/DensityGridMediumDistribution.h"
#include "Texture/constant_textures.h"
#include "Texture/image_textures.h"
#include "SurfaceMaterial/basic_surface_materials.h"
#include "SurfaceMaterial/microfacet_surface_materials.h"
#include "SurfaceMaterial/basic_emitter_surface_properties.h"
#include "BSDF/basic_bsdfs.h"
#include "BSDF/microfacet_bsdfs.h"
#include "Renderer/PTRenderer.h"
#include "Renderer/VolumetricPTRenderer.h"
#include "Renderer/BPTRenderer.h"
#include "Renderer/VolumetricBPTRenderer.h"
#include "MediumMaterial/basic_medium_materials.h"
#include "Core/medium_material.h"
#include "Core/medium_object.h"

extern "C" unsigned int slr_oracle_max_depth = 100;
std::atomic<unsigned long long> slr_oracle_dropped_samples(0);
// Path tapes (build patch P12): while set, every uniform the reference's RNG
// returns is appended to slr_oracle_tape, and slr_oracle_path_begin() marks
// where each pixel sample's draws begin.  Used with one render thread only.
std::vector<float>* slr_oracle_tape = nullptr;
static std::vector<uint32_t>* g_pathStarts = nullptr;
extern "C" void slr_oracle_path_begin() {
    if (slr_oracle_tape && g_pathStarts) g_pathStarts->push_back((uint32_t)slr_oracle_tape->size());
}

namespace SLR {
    // Reads the private node arrays of a built SBVH through SBVH's friend
    // declaration (SBVH.h:19).
    class QBVH {
    public:
        static const SBVH::Node* nodes(const SBVH &b, size_t* n) { *n = b.m_nodes.size(); return b.m_nodes.data(); }
        static const std::vector<const SurfaceObject*> &leaves(const SBVH &b) { return b.m_objLists; }
        static uint32_t depth(const SBVH &b) { return b.m_depth; }
    };
}

using namespace SLR;

namespace {
    std::once_flag g_colorInit;

    struct OraScene {
        ArenaAllocator sceneMem;
        std::vector<std::unique_ptr<AssetSpectrum>> spectra;
        std::vector<std::unique_ptr<SpectrumTexture>> specTex;
        std::vector<std::unique_ptr<FloatTexture>> floatTex;
        std::vector<std::unique_ptr<SVMicrofacetDistribution>> dists;
        std::vector<std::unique_ptr<EmitterSurfaceProperty>> emitters;
        std::vector<std::unique_ptr<SurfaceMaterial>> materials;
        std::vector<std::unique_ptr<TriangleMeshNode>> meshes;
        std::vector<std::unique_ptr<Image2D>> images;
        std::unique_ptr<Texture2DMapping> mapping;
        std::unique_ptr<StaticTransform> identityTF, cameraTF;
        std::unique_ptr<InternalNode> root, cameraParent;
        std::unique_ptr<Node> cameraNode;
        std::unique_ptr<InfiniteSphereNode> envNode;
        const SpectrumTexture* envTex = nullptr;
        float envScale = 1.0f;
        std::vector<std::unique_ptr<MediumNode>> mediumNodes;
        std::vector<std::unique_ptr<MediumMaterial>> mediumMaterials;
        std::vector<std::vector<float>> densitySlices;   // must outlive the medium node
        // The medium's distribution again, standalone, for medium queries.
        int medSigmaS = -1, medSigmaE = -1, medN[3] = {0, 0, 0};
        float medBmin[3], medBmax[3];
        std::unique_ptr<DensityGridMediumDistribution> medDist;
        std::unique_ptr<SingleMediumObject> medObj;
        std::unique_ptr<MediumObjectAggregate> medAgg;
        std::unique_ptr<Scene> scene;
        bool built = false;
        bool bptRendered = false;
        // Standalone SBVH over the same surface objects, for ray queries.
        ArenaAllocator rayMem;
        std::vector<SurfaceObject*> rayObjs;
        std::unordered_map<const SurfaceObject*, uint32_t> objIndex;
        std::unique_ptr<SBVH> sbvh;
    };

    const SpectrumTexture* constTex(OraScene* s, int spectrum) {
        s->specTex.emplace_back(new ConstantSpectrumTexture(s->spectra.at(spectrum).get()));
        return s->specTex.back().get();
    }

    const FloatTexture* floatTex(OraScene* s, float v) {
        s->floatTex.emplace_back(new ConstantFloatTexture(v));
        return s->floatTex.back().get();
    }

    int addMaterial(OraScene* s, SurfaceMaterial* m) {
        s->materials.emplace_back(m);
        return (int)s->materials.size() - 1;
    }

    template <typename F>
    void parallelFor(int n, int threads, F f) {
        threads = std::max(1, threads);
        std::atomic<int> next(0);
        const int chunk = 1024;
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t)
            pool.emplace_back([&]() {
                for (;;) {
                    int b = next.fetch_add(chunk);
                    if (b >= n) break;
                    int e = std::min(n, b + chunk);
                    for (int i = b; i < e; ++i) f(i);
                }
            });
        for (auto &th : pool) th.join();
    }
}

extern "C" {

void* ora_scene_new() {
    std::call_once(g_colorInit, []() { initializeColorSystem(); });
    OraScene* s = new OraScene();
    s->identityTF.reset(new StaticTransform());
    s->root.reset(new InternalNode(s->identityTF.get()));
    s->mapping.reset(new Texture2DMapping());
    return s;
}

void ora_scene_free(void* p) {
    OraScene* s = (OraScene*)p;
    if (s->built)
        s->scene->destory();
    delete s;
}

// spType: 0 Reflectance, 1 LightSource, 2 IndexOfRefraction (spectrum_base.h:34-38)
int ora_spectrum_rgb(void* p, int spType, float r, float g, float b) {
    OraScene* s = (OraScene*)p;
    s->spectra.emplace_back(new UpsampledContinuousSpectrum((SpectrumType)spType, ColorSpace::sRGB, r, g, b));
    return (int)s->spectra.size() - 1;
}

int ora_spectrum_regular(void* p, float minWL, float maxWL, const float* vals, int n) {
    OraScene* s = (OraScene*)p;
    s->spectra.emplace_back(new RegularContinuousSpectrum(minWL, maxWL, vals, n));
    return (int)s->spectra.size() - 1;
}

int ora_spectrum_irregular(void* p, const float* wls, const float* vals, int n) {
    OraScene* s = (OraScene*)p;
    s->spectra.emplace_back(new IrregularContinuousSpectrum(wls, vals, n));
    return (int)s->spectra.size() - 1;
}

int ora_material_matte(void* p, int refl) {
    OraScene* s = (OraScene*)p;
    return addMaterial(s, new DiffuseReflectionSurfaceMaterial(constTex(s, refl), nullptr));
}

int ora_material_specular_reflection(void* p, int coeff, int eta, int k) {
    OraScene* s = (OraScene*)p;
    return addMaterial(s, new SpecularReflectionSurfaceMaterial(constTex(s, coeff), constTex(s, eta), constTex(s, k)));
}

int ora_material_specular_scattering(void* p, int coeff, int etaExt, int etaInt) {
    OraScene* s = (OraScene*)p;
    return addMaterial(s, new SpecularScatteringSurfaceMaterial(constTex(s, coeff), constTex(s, etaExt), constTex(s, etaInt)));
}

int ora_material_microfacet_reflection(void* p, int eta, int k, float ax, float ay) {
    OraScene* s = (OraScene*)p;
    s->dists.emplace_back(new GGXSVMicrofacetDistribution(floatTex(s, ax), floatTex(s, ay)));
    return addMaterial(s, new MicrofacetReflectionSurfaceMaterial(constTex(s, eta), constTex(s, k), s->dists.back().get()));
}

int ora_material_microfacet_scattering(void* p, int etaExt, int etaInt, float ax, float ay) {
    OraScene* s = (OraScene*)p;
    s->dists.emplace_back(new GGXSVMicrofacetDistribution(floatTex(s, ax), floatTex(s, ay)));
    return addMaterial(s, new MicrofacetScatteringSurfaceMaterial(constTex(s, etaExt), constTex(s, etaInt), s->dists.back().get()));
}

int ora_material_emitter(void* p, int baseMat, int emittance) {
    OraScene* s = (OraScene*)p;
    s->emitters.emplace_back(new DiffuseEmitterSurfaceProperty(constTex(s, emittance)));
    return addMaterial(s, new EmitterSurfaceMaterial(s->materials.at(baseMat).get(), s->emitters.back().get()));
}

// One TriangleMeshNode with a single material group; vertex positions are
// world-space (identity transform), so TriangleMeshNode::createRenderingData
// leaves them untouched (TriangleMeshNode.cpp:61-75).
int ora_mesh(void* p, const float* pos, const float* nrm, const float* tan, const float* uv,
             int nv, const uint32_t* idx, int ntri, int material) {
    OraScene* s = (OraScene*)p;
    TriangleMeshNode* mesh = new TriangleMeshNode(nv, 1, false, -1);
    Vertex* verts = mesh->getVertexArray();
    for (int i = 0; i < nv; ++i) {
        verts[i] = Vertex(Point3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                          Normal3D(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]),
                          Tangent3D(tan[3 * i], tan[3 * i + 1], tan[3 * i + 2]),
                          TexCoord2D(uv[2 * i], uv[2 * i + 1]));
    }
    MaterialGroupInTriangleMesh &grp = mesh->getMaterialGroupArray()[0];
    grp.material = s->materials.at(material).get();
    std::unique_ptr<Vertex*[]> refs(new Vertex*[3 * ntri]);
    for (int i = 0; i < 3 * ntri; ++i) {
        if (idx[i] >= (uint32_t)nv) { delete mesh; return -1; }
        refs[i] = verts + idx[i];
    }
    grp.setTriangles(refs, ntri);
    s->meshes.emplace_back(mesh);
    s->root->addChildNode(mesh);
    return (int)s->meshes.size() - 1;
}

// rgbaHalf: width*height*4 IEEE binary16 values (linear RGBA), stored by the
// reference as uvsA16Fx4 texels (image_2d.h:270-291).
int ora_env_ibl(void* p, const uint16_t* rgbaHalf, int w, int h, float scale) {
    OraScene* s = (OraScene*)p;
    s->images.emplace_back(new TiledImage2D(rgbaHalf, w, h, ColorFormat::RGBA16Fx4, &s->sceneMem,
                                            ImageStoreMode::AsIs, SpectrumType::LightSource));
    s->specTex.emplace_back(new ImageSpectrumTexture(s->images.back().get(), s->mapping.get()));
    s->envTex = s->specTex.back().get();
    s->envScale = scale;
    return 0;
}

// Density-grid medium over [bmin, bmax] with a Henyey-Greenstein phase
// function (Scene/medium_nodes.h:33-48, MediumMaterial/basic_medium_materials.h:25-32);
// density is [nz][ny][nx].
int ora_medium_density_grid(void* p, const float* bmin, const float* bmax, int sigmaS, int sigmaE,
                            const float* density, int nx, int ny, int nz, float g) {
    OraScene* s = (OraScene*)p;
    s->densitySlices.assign(nz, std::vector<float>());
    for (int z = 0; z < nz; ++z)
        s->densitySlices[z].assign(density + (size_t)z * nx * ny, density + (size_t)(z + 1) * nx * ny);
    s->mediumMaterials.emplace_back(new HenyeyGreensteinScatteringMediumMaterial(floatTex(s, g)));
    BoundingBox3D region(Point3D(bmin[0], bmin[1], bmin[2]), Point3D(bmax[0], bmax[1], bmax[2]));
    DensityGridMediumNode* node = new DensityGridMediumNode(region, s->spectra.at(sigmaS).get(), s->spectra.at(sigmaE).get(),
                                                            s->densitySlices, nx, ny, nz, s->mediumMaterials.back().get());
    s->mediumNodes.emplace_back(node);
    s->root->addChildNode(node);
    s->medSigmaS = sigmaS;
    s->medSigmaE = sigmaE;
    s->medN[0] = nx; s->medN[1] = ny; s->medN[2] = nz;
    for (int i = 0; i < 3; ++i) { s->medBmin[i] = bmin[i]; s->medBmax[i] = bmax[i]; }
    return 0;
}

// m: row-major 4x4 camera-to-world matrix.
int ora_camera_perspective(void* p, const float* m, float sensitivity, float aspect, float fovY,
                           float lensRadius, float imgPDist, float objPDist) {
    OraScene* s = (OraScene*)p;
    Matrix4x4 mat(Vector4D(m[0], m[4], m[8], m[12]), Vector4D(m[1], m[5], m[9], m[13]),
                  Vector4D(m[2], m[6], m[10], m[14]), Vector4D(m[3], m[7], m[11], m[15]));
    s->cameraTF.reset(new StaticTransform(mat));
    s->cameraParent.reset(new InternalNode(s->cameraTF.get()));
    s->cameraNode.reset(new PerspectiveCameraNode(sensitivity, aspect, fovY, lensRadius, imgPDist, objPDist));
    s->cameraParent->addChildNode(s->cameraNode.get());
    s->root->addChildNode(s->cameraParent.get());
    return 0;
}

int ora_camera_equirect(void* p, const float* m, float sensitivity, float phiAngle, float thetaAngle) {
    OraScene* s = (OraScene*)p;
    Matrix4x4 mat(Vector4D(m[0], m[4], m[8], m[12]), Vector4D(m[1], m[5], m[9], m[13]),
                  Vector4D(m[2], m[6], m[10], m[14]), Vector4D(m[3], m[7], m[11], m[15]));
    s->cameraTF.reset(new StaticTransform(mat));
    s->cameraParent.reset(new InternalNode(s->cameraTF.get()));
    s->cameraNode.reset(new EquirectangularCameraNode(sensitivity, phiAngle, thetaAngle));
    s->cameraParent->addChildNode(s->cameraNode.get());
    s->root->addChildNode(s->cameraParent.get());
    return 0;
}

// The built SLR::Scene, for applications that render it through another
// SLR::Renderer (null before ora_build).
void* ora_scene_ptr(void* p) {
    OraScene* s = (OraScene*)p;
    return s->built ? (void*)s->scene.get() : nullptr;
}

int ora_build(void* p) {
    OraScene* s = (OraScene*)p;
    if (s->built) return 0;
    s->scene.reset(new Scene(s->root.get()));
    // The environment node needs the scene for the world disc area used by
    // its EDF (IBLEmitterSurfaceProperty.cpp:20), so it is created here.
    if (s->envTex) {
        s->envNode.reset(new InfiniteSphereNode(s->scene.get(), s->envTex, s->envScale));
        s->scene->setEnvironmentNode(s->envNode.get());
    }
    s->scene->build(&s->sceneMem);
    s->built = true;
    return 0;
}

// Renders with PTRenderer (volumetric == 0) or VolumetricPTRenderer and
// copies the raw 16-bin film (sum over all samples, per pixel, row-major) to
// film[h][w][16].  Timing covers renderer.render() only.
int ora_render(void* p, int volumetric, int spp, int maxDepth, int w, int h, int threads, int seed,
               float* film, double* seconds) {
    OraScene* s = (OraScene*)p;
    if (!s->built || !s->scene->getCamera()) return -1;
    slr_oracle_max_depth = (unsigned)maxDepth;
    RenderSettings settings;
    settings.addItem(RenderSettingItem::NumThreads, (int32_t)threads);
    settings.addItem(RenderSettingItem::ImageWidth, (int32_t)w);
    settings.addItem(RenderSettingItem::ImageHeight, (int32_t)h);
    settings.addItem(RenderSettingItem::TimeStart, 0.0f);
    settings.addItem(RenderSettingItem::TimeEnd, 0.0f);
    settings.addItem(RenderSettingItem::Brightness, 1.0f);
    settings.addItem(RenderSettingItem::RNGSeed, (int32_t)seed);
    std::unique_ptr<Renderer> r;
    slr_oracle_dropped_samples.store(0);
    if (volumetric) r.reset(new VolumetricPTRenderer(spp));
    else r.reset(new PTRenderer(spp));
    auto t0 = std::chrono::steady_clock::now();
    r->render(*s->scene, settings);
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    const ImageSensor* sensor = s->scene->getCamera()->getSensor();
    if (film) {
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                DiscretizedSpectrum v = sensor->pixel(x, y);
                for (int b = 0; b < 16; ++b)
                    film[((size_t)y * w + x) * 16 + b] = v[b];
            }
    }
    return 0;
}

// A one-thread, one-sample PTRenderer render that records each path's
// uniforms in the reference's draw order (Job::kernel, PTRenderer.cpp:103-144,
// and Job::contribution, :146-276): tape[starts[k] .. starts[k + 1]) are the
// draws of the k-th pixel sample, in the renderer's tile order.  Returns -3
// when tapeCap or startsCap is too small (*nDraws, *nPaths then hold the sizes
// needed).
int ora_render_record(void* p, int maxDepth, int w, int h, int seed, float* film, float* tape, uint32_t tapeCap,
                      uint32_t* starts, uint32_t startsCap, uint32_t* nDraws, uint32_t* nPaths) {
    std::vector<float> t;
    std::vector<uint32_t> st;
    slr_oracle_tape = &t;
    g_pathStarts = &st;
    int rc = ora_render(p, 0, 1, maxDepth, w, h, 1, seed, film, nullptr);
    slr_oracle_tape = nullptr;
    g_pathStarts = nullptr;
    if (rc != 0) return rc;
    *nDraws = (uint32_t)t.size();
    *nPaths = (uint32_t)st.size();
    if (t.size() > tapeCap || st.size() > startsCap) return -3;
    std::copy(t.begin(), t.end(), tape);
    std::copy(st.begin(), st.end(), starts);
    return 0;
}

// Renders with BPTRenderer (volumetric == 0) or VolumetricBPTRenderer
// (VolumetricBPTRenderer.cpp:25-101) and copies the 16-bin film, main buffer plus the
// per-thread buffers that collect the light-tracing connections
// (BPTRenderer.cpp:268-276; ImageSensor::saveImage adds them the same way,
// ImageSensor.cpp:154-156).  ImageSensor::addSeparatedBuffers
// (ImageSensor.cpp:54-63) allocates buffers only beyond those it already
// has, into a new pointer array, so a second BPT render through the same
// sensor would clear unallocated buffers: one BPT render per scene (-2).
int ora_render_bpt(void* p, int volumetric, int spp, int maxDepth, int w, int h, int threads, int seed, float* film,
                   double* seconds) {
    OraScene* s = (OraScene*)p;
    if (!s->built || !s->scene->getCamera()) return -1;
    if (s->bptRendered) return -2;
    s->bptRendered = true;
    slr_oracle_max_depth = (unsigned)maxDepth;
    RenderSettings settings;
    settings.addItem(RenderSettingItem::NumThreads, (int32_t)threads);
    settings.addItem(RenderSettingItem::ImageWidth, (int32_t)w);
    settings.addItem(RenderSettingItem::ImageHeight, (int32_t)h);
    settings.addItem(RenderSettingItem::TimeStart, 0.0f);
    settings.addItem(RenderSettingItem::TimeEnd, 0.0f);
    settings.addItem(RenderSettingItem::Brightness, 1.0f);
    settings.addItem(RenderSettingItem::RNGSeed, (int32_t)seed);
    slr_oracle_dropped_samples.store(0);
    std::unique_ptr<Renderer> r;
    if (volumetric) r.reset(new VolumetricBPTRenderer(spp));
    else r.reset(new BPTRenderer(spp));
    auto t0 = std::chrono::steady_clock::now();
    r->render(*s->scene, settings);
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    const ImageSensor* sensor = s->scene->getCamera()->getSensor();
    if (film) {
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                DiscretizedSpectrum v = sensor->pixel(x, y);
                for (int t = 0; t < threads; ++t) v += sensor->pixel((uint32_t)t, x, y);
                for (int b = 0; b < 16; ++b)
                    film[((size_t)y * w + x) * 16 + b] = v[b];
            }
    }
    return 0;
}

// Non-finite samples dropped by the last ora_render call.
unsigned long long ora_dropped_samples() { return slr_oracle_dropped_samples.load(); }

// Builds a standalone SBVH over the scene's triangles, in the same object
// order as Scene::build (node order, then triangle order), and reports the
// fingerprint the reference prints at SBVH.h:415.
int ora_sbvh_build(void* p, uint32_t* numFragments, uint32_t* depth, float* cost, uint32_t* numNodes) {
    OraScene* s = (OraScene*)p;
    if (!s->sbvh) {
        RenderingData rd(nullptr);
        for (auto &m : s->meshes)
            m->createRenderingData(&s->rayMem, nullptr, &rd);
        s->rayObjs = rd.surfObjs;
        for (size_t i = 0; i < s->rayObjs.size(); ++i)
            s->objIndex[s->rayObjs[i]] = (uint32_t)i;
        s->sbvh.reset(new SBVH(s->rayObjs));
    }
    size_t n;
    QBVH::nodes(*s->sbvh, &n);
    if (numFragments) *numFragments = (uint32_t)QBVH::leaves(*s->sbvh).size();
    if (depth) *depth = QBVH::depth(*s->sbvh);
    if (cost) *cost = s->sbvh->costForIntersect();
    if (numNodes) *numNodes = (uint32_t)n;
    return 0;
}

// Node dump: per node 6 floats (minP, maxP) + 5 uints (c0, c1, offset,
// count, axis); leaf list as triangle indices.
int ora_sbvh_dump(void* p, float* boxes, uint32_t* words, uint32_t* leafPrims) {
    OraScene* s = (OraScene*)p;
    if (!s->sbvh) return -1;
    size_t n;
    const auto* nodes = QBVH::nodes(*s->sbvh, &n);
    for (size_t i = 0; i < n; ++i) {
        const auto &nd = nodes[i];
        boxes[6 * i + 0] = nd.bbox.minP.x; boxes[6 * i + 1] = nd.bbox.minP.y; boxes[6 * i + 2] = nd.bbox.minP.z;
        boxes[6 * i + 3] = nd.bbox.maxP.x; boxes[6 * i + 4] = nd.bbox.maxP.y; boxes[6 * i + 5] = nd.bbox.maxP.z;
        words[5 * i + 0] = nd.c0; words[5 * i + 1] = nd.c1;
        words[5 * i + 2] = nd.offsetFirstLeaf; words[5 * i + 3] = nd.numLeaves;
        words[5 * i + 4] = nd.numLeaves ? 0xffffffffu : (uint32_t)nd.axis;
    }
    const auto &leaves = QBVH::leaves(*s->sbvh);
    for (size_t i = 0; i < leaves.size(); ++i)
        leafPrims[i] = s->objIndex.at(leaves[i]);
    return 0;
}

// rays: 8 floats per ray (org.xyz, tmin, dir.xyz, tmax).  Closest hit
// (anyhit == 0): prim (0xffffffff on miss), t, b1, b2 of the Moller-Trumbore
// test (TriangleSurfaceShape.cpp:205-257; the interaction stores b0 = 1-b1-b2
// and b1, so b2 is recovered as 1 - b0 - b1).  Any hit: prim[i] = 1 when the
// segment is occluded (fractional visibility 0), else 0.
int ora_trace(void* p, const float* rays, int n, int anyhit, int threads,
              uint32_t* prim, float* t, float* b1, float* b2) {
    OraScene* s = (OraScene*)p;
    if (!s->sbvh) ora_sbvh_build(p, nullptr, nullptr, nullptr, nullptr);
    parallelFor(n, threads, [&](int i) {
        const float* r = rays + 8 * (size_t)i;
        Ray ray(Point3D(r[0], r[1], r[2]), Vector3D(r[4], r[5], r[6]), 0.0f);
        RaySegment seg(r[3], r[7]);
        if (anyhit) {
            float vis = s->sbvh->testVisibility(ray, seg);
            prim[i] = vis == 0.0f ? 1u : 0u;
            return;
        }
        thread_local IndependentLightPathSampler sampler(12345);
        SurfaceInteraction si;
        const SurfaceObject* obj = nullptr;
        if (s->sbvh->intersect(ray, seg, sampler, &si, &obj)) {
            prim[i] = s->objIndex.at(obj);
            t[i] = si.getDistance();
            float u, v;
            si.getSurfaceParameter(&u, &v);
            b1[i] = v;
            b2[i] = 1.0f - u - v;
        } else {
            prim[i] = 0xffffffffu;
            t[i] = INFINITY; b1[i] = 0; b2[i] = 0;
        }
    });
    return 0;
}

// BSDF known-answer queries on the reference BSDF classes, built directly as
// SLR_Test/bsdf_tests.cpp does.
//   kind 0: LambertianBRDF(R)                      spec0 = R
//   kind 1: SpecularBRDF(coeff, eta, k)            spec0 = coeff, spec1 = eta, spec2 = k
//   kind 2: SpecularBSDF(coeff, etaExt, etaInt, dispersive=1)
//   kind 3: MicrofacetBRDF(eta, k, GGX(ax, ay))    spec0 = eta, spec1 = k
//   kind 4: MicrofacetBSDF(etaExt, etaInt, GGX(ax, ay))
// Per query (q = 16 floats): dirLocal.xyz, gNormal.xyz, wlIdx, adjoint,
// uComponent, uDir0, uDir1, evalDir.xyz, pad, pad.
// Out (o = 40 floats): sampled fs[16], sampled dir.xyz, sampled pdf,
// sampledType, eval fs[16], eval pdf, pad...
int ora_bsdf_query(int kind, const float* spec0, const float* spec1, const float* spec2,
                   float ax, float ay, const float* q, int nq, float* o) {
    SampledSpectrum s0(spec0), s1(spec1 ? spec1 : spec0), s2(spec2 ? spec2 : spec0);
    GGXMicrofacetDistribution ggx(ax, ay);
    std::unique_ptr<BSDF> bsdf;
    switch (kind) {
        case 0: bsdf.reset(new LambertianBRDF(s0)); break;
        case 1: bsdf.reset(new SpecularBRDF(s0, s1, s2)); break;
        case 2: bsdf.reset(new SpecularBSDF(s0, s1, s2, true)); break;
        case 3: bsdf.reset(new MicrofacetBRDF(s0, s1, &ggx)); break;
        case 4: bsdf.reset(new MicrofacetBSDF(s0, s1, &ggx)); break;
        default: return -1;
    }
    for (int i = 0; i < nq; ++i) {
        const float* qi = q + 16 * (size_t)i;
        float* oi = o + 40 * (size_t)i;
        Vector3D dir(qi[0], qi[1], qi[2]);
        Normal3D gn(qi[3], qi[4], qi[5]);
        BSDFQuery query(dir, gn, (int16_t)qi[6], DirectionType::All, false, qi[7] != 0.0f);
        BSDFSample smp(qi[8], qi[9], qi[10]);
        BSDFQueryResult res;
        SampledSpectrum fs = bsdf->sample(query, smp, &res);
        for (int k = 0; k < 16; ++k) oi[k] = fs[k];
        oi[16] = res.dirLocal.x; oi[17] = res.dirLocal.y; oi[18] = res.dirLocal.z;
        oi[19] = res.dirPDF;
        oi[20] = (float)(uint32_t)res.sampledType.value;
        Vector3D ed(qi[11], qi[12], qi[13]);
        SampledSpectrum fe = bsdf->evaluate(query, ed);
        for (int k = 0; k < 16; ++k) oi[21 + k] = fe[k];
        oi[37] = bsdf->evaluatePDF(query, ed);
        oi[38] = 0.0f; oi[39] = 0.0f;
    }
    return 0;
}

}  // extern "C"

namespace {
// An RNG that replays a given stream of 32-bit values (then 0x80000000), so
// that the medium routines draw exactly the uniforms a test hands them; it
// stands in for the XORShift generator behind FreePathSampler
// (Core/light_path_sampler.h:55-61).
class ReplayRNG : public XORShiftRNG {
public:
    const uint32_t* vals = nullptr;
    uint32_t n = 0, used = 0;
    uint32_t getUInt() override {
        uint32_t v = used < n ? vals[used] : 0x80000000u;
        ++used;
        return v;
    }
};

class ReplayPathSampler : public LightPathSampler {
public:
    ReplayRNG rng;
    AlphaTestSampler alphaSampler;
    FreePathSampler freeSampler;
    ReplayPathSampler() : alphaSampler(rng), freeSampler(rng) { }
    float f() { return rng.getFloat0cTo1o(); }
    float getTimeSample(float b, float e) override { float v = f(); return b * (1 - v) + e * v; }
    PixelPosition getPixelPositionSample(uint32_t x, uint32_t y) override { float a = f(); return PixelPosition(x + a, y + f()); }
    float getWavelengthSample() override { return f(); }
    float getWLSelectionSample() override { return f(); }
    LensPosSample getLensPosSample() override { float a = f(); return LensPosSample(a, f()); }
    IDFSample getIDFSample() override { float a = f(); return IDFSample(a, f()); }
    BSDFSample getBSDFSample() override { float a = f(), b = f(); return BSDFSample(a, b, f()); }
    PFSample getPFSample() override { float a = f(); return PFSample(a, f()); }
    AlphaTestSampler &getAlphaTestSampler() override { return alphaSampler; }
    FreePathSampler &getFreePathSampler() override { return freeSampler; }
    float getPathTerminationSample() override { return f(); }
    float getLightSelectionSample() override { return f(); }
    SurfaceLightPosSample getSurfaceLightPosSample() override { float a = f(); return SurfaceLightPosSample(a, f()); }
    VolumetricLightPosSample getVolumetricLightPosSample() override { float a = f(), b = f(); return VolumetricLightPosSample(a, b, f()); }
    EDFSample getEDFSample() override { float a = f(), b = f(); return EDFSample(a, b, f()); }
};
}  // namespace

extern "C" {

// Medium queries on one segment inside the density-grid medium, with the
// free-path sampler replaying given uniforms.  mode 0:
// DensityGridMediumDistribution::interact (DensityGridMediumDistribution.cpp:402-575),
// mode 1: ::evaluateTransmittance (:577-744), mode 2: the extinction
// coefficient at a normalised position (rays[0..2]) (:756-759); modes 3 and
// 4: interact / evaluateTransmittance of the medium aggregate
// (Core/medium_object.cpp:287-402), which walks the medium's boundary
// crossings, on any segment.
// rays: n x 8 (org.xyz, distMin, dir.xyz, distMax); lambdas: n x 16;
// sel: n (selected index | 0x100 if the wavelength is already selected);
// vals: n x nvals uint32; out: n x 24 (hit, dist, param.xyz, values used,
// spectrum[16], 0, 0).
int ora_medium_query(void* p, int mode, int n, const float* rays, const float* lambdas, const int* sel,
                     const uint32_t* vals, int nvals, float* out) {
    OraScene* s = (OraScene*)p;
    if (s->medSigmaE < 0) return -1;
    if (!s->medDist) {
        BoundingBox3D region(Point3D(s->medBmin[0], s->medBmin[1], s->medBmin[2]),
                             Point3D(s->medBmax[0], s->medBmax[1], s->medBmax[2]));
        s->medDist.reset(new DensityGridMediumDistribution(region, s->spectra.at(s->medSigmaS).get(),
                                                           s->spectra.at(s->medSigmaE).get(), s->densitySlices,
                                                           s->medN[0], s->medN[1], s->medN[2]));
    }
    if (!s->medAgg) {
        s->medObj.reset(new SingleMediumObject(s->medDist.get(), s->mediumMaterials.back().get()));
        std::vector<MediumObject*> objs{s->medObj.get()};
        s->medAgg.reset(new MediumObjectAggregate(objs));
    }
    const DensityGridMediumDistribution* md = s->medDist.get();
    const MediumObjectAggregate* agg = s->medAgg.get();
    for (int i = 0; i < n; ++i) {
        const float* r = rays + 8 * (size_t)i;
        float* o = out + 24 * (size_t)i;
        std::memset(o, 0, 24 * sizeof(float));
        WavelengthSamples wls(lambdas + 16 * (size_t)i);
        wls.selectedLambdaIndex = (uint16_t)(sel[i] & 0xff);
        wls.flags = (sel[i] & 0x100) ? WavelengthSamples::WavelengthIsSelected : 0;
        ReplayPathSampler ps;
        ps.rng.vals = vals + (size_t)nvals * i;
        ps.rng.n = (uint32_t)nvals;
        Ray ray(Point3D(r[0], r[1], r[2]), Vector3D(r[4], r[5], r[6]), 0.0f);
        RaySegment seg(r[3], r[7]);
        SampledSpectrum v;
        bool single = false;
        if (mode == 0) {
            MediumInteraction mi;
            bool hit = md->interact(ray, seg, wls, ps, &mi, &v, &single);
            o[0] = hit ? 1.0f : 0.0f;
            if (hit) {
                o[1] = mi.getDistance();
                mi.getMediumParameter(&o[2], &o[3], &o[4]);
            }
        } else if (mode == 1) {
            v = md->evaluateTransmittance(ray, seg, wls, ps, &single);
        } else if (mode == 3) {
            MediumInteraction mi;
            bool hit = agg->interact(ray, seg, wls, ps, &mi, &v, &single);
            o[0] = hit ? 1.0f : 0.0f;
            if (hit) {
                o[1] = mi.getDistance();
                mi.getMediumParameter(&o[2], &o[3], &o[4]);
            }
        } else if (mode == 4) {
            v = agg->evaluateTransmittance(ray, seg, wls, ps, &single);
        } else {
            v = md->evaluateExtinctionCoefficient(Point3D(r[0], r[1], r[2]), wls);
        }
        o[5] = (float)ps.rng.used;
        for (int k = 0; k < 16; ++k) o[6 + k] = v[k];
    }
    return 0;
}

// Film output through the reference's own ImageSensor::saveImage
// (Core/ImageSensor.cpp:139-195): the film (width*height*16 floats, row
// major) is written into a sensor of the given sensitivity, then saved.
int ora_film_bmp(const float* film, int w, int h, float scale, float sensitivity, const char* path) {
    std::call_once(g_colorInit, []() { initializeColorSystem(); });
    ImageSensor sensor(sensitivity);
    sensor.init((uint32_t)w, (uint32_t)h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            CompensatedSum<DiscretizedSpectrum> &v = sensor.pixel((uint32_t)x, (uint32_t)y).getValue();
            v.result = DiscretizedSpectrum(film + 16 * ((size_t)y * w + x));
            v.comp = DiscretizedSpectrum(0.0f);
        }
    sensor.saveImage(path, scale);
    return 0;
}

// The discretised colour matching functions of the film
// (DiscretizedSpectrumTemplate::initialize): x[16], y[16], z[16], integral.
int ora_film_cmf(float* bins, float* integral) {
    std::call_once(g_colorInit, []() { initializeColorSystem(); });
    for (int i = 0; i < 16; ++i) {
        bins[i] = DiscretizedSpectrum::xbar[i];
        bins[16 + i] = DiscretizedSpectrum::ybar[i];
        bins[32 + i] = DiscretizedSpectrum::zbar[i];
    }
    *integral = DiscretizedSpectrum::integralCMF;
    return 0;
}

// Spectrum evaluation at explicit wavelength sets (16 per set), for the
// upsampled / regular / irregular spectrum parity checks.
int ora_spectrum_eval(void* p, int spectrum, const float* lambdas, int nsets, float* out) {
    OraScene* s = (OraScene*)p;
    const AssetSpectrum* sp = s->spectra.at(spectrum).get();
    for (int i = 0; i < nsets; ++i) {
        WavelengthSamples wls(lambdas + 16 * (size_t)i);
        SampledSpectrum v = sp->evaluate(wls);
        for (int k = 0; k < 16; ++k) out[16 * (size_t)i + k] = v[k];
    }
    return 0;
}

}  // extern "C"
