/*
 * slrgpu.h - C ABI of the GB300 path tracer (drop-in for SLR's PTRenderer and
 * VolumetricPTRenderer).
 *
 * Plain C: opaque 64-bit handles, plain pointers and sizes, int status codes
 * (0 = success, negative = error; slrgpu_last_error() returns the message of
 * the calling thread's last failure).  Arrays passed in are copied before the
 * call returns; the caller keeps ownership.  One context per GPU; calls on
 * different scenes may come from different threads.
 *
 * The entry points replace the reference's C++ interfaces as follows (paths
 * are relative to the reference project):
 *   scene construction  - libSLR/Scene/Scene.h:31-36 (Scene(root), build),
 *                         libSLR/Scene/TriangleMeshNode.h:37-73,
 *                         libSLR/Scene/node.h:125-141 (InfiniteSphereNode),
 *                         libSLR/Scene/medium_nodes.h:33-48 (DensityGridMediumNode),
 *                         libSLR/Scene/camera_nodes.h:16-54
 *   spectra             - libSLR/BasicTypes/spectrum_types.h:90-190
 *                         (Regular/Irregular/UpsampledContinuousSpectrum)
 *   materials           - libSLR/SurfaceMaterial/basic_surface_materials.h:20-57,
 *                         microfacet_surface_materials.h:21-37,
 *                         libSLR/Core/surface_material.h:55-69 (EmitterSurfaceMaterial)
 *   rendering           - libSLR/Core/renderer.h:15-19 (Renderer::render),
 *                         libSLR/Renderer/PTRenderer.h:42-43,
 *                         libSLR/Renderer/VolumetricPTRenderer.h:43-44
 *   film                - libSLR/Core/ImageSensor.h:47-48 (pixel(x, y))
 *   ray queries         - libSLR/Core/accelerator.h:16-30 (intersect / testVisibility)
 */
#ifndef SLRGPU_H
#define SLRGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SLRGPU_OK 0
#define SLRGPU_ERR_INVALID_ARGUMENT (-1)
#define SLRGPU_ERR_INVALID_HANDLE   (-2)
#define SLRGPU_ERR_CUDA             (-3)
#define SLRGPU_ERR_OUT_OF_MEMORY    (-4)
#define SLRGPU_ERR_NOT_COMMITTED    (-5)
#define SLRGPU_ERR_STATE            (-6)
#define SLRGPU_ERR_TIMEOUT          (-7)
#define SLRGPU_ERR_UNSUPPORTED      (-8)   /* a valid request this library does not implement */
#define SLRGPU_ERR_CANCELLED        (-9)   /* a server request cancelled by slrgpu_server_cancel */

typedef uint64_t slrgpu_handle;

/* Spectrum types (libSLR/BasicTypes/spectrum_base.h:34-38). */
#define SLRGPU_SPECTRUM_REFLECTANCE 0
#define SLRGPU_SPECTRUM_LIGHT_SOURCE 1
#define SLRGPU_SPECTRUM_INDEX_OF_REFRACTION 2

typedef struct slrgpu_bvh_stats {
    uint32_t num_triangles;   /* input primitives */
    uint32_t num_fragments;   /* SBVH leaf references after spatial splits */
    uint32_t depth;           /* binary SBVH depth */
    uint32_t num_binary_nodes;
    uint32_t num_wide_nodes;  /* after collapse to the wide layout */
    uint32_t width;           /* children per wide node (4 or 8) */
    float sah_cost;           /* SAH cost as printed at SBVH.h:415 */
    float build_seconds;
} slrgpu_bvh_stats;

typedef struct slrgpu_settings {
    uint32_t width, height;       /* film size in pixels */
    uint32_t spp;                 /* samples per pixel */
    uint32_t max_depth;           /* scattering vertices with NEE + BSDF sampling */
    uint32_t seed;                /* RNG seed (RenderSettingItem::RNGSeed) */
    uint32_t volumetric;          /* 0: PTRenderer, 1: VolumetricPTRenderer */
    uint32_t samples_per_wave;    /* 0: automatic; paths in flight = this times
                                     the sample grid (W and H rounded up to
                                     multiples of 8) */
    uint32_t flags;               /* SLRGPU_FLAG_* */
    uint32_t sample_base;         /* index of the first sample: renders of disjoint
                                     ranges [sample_base, sample_base + spp) of one
                                     image (e.g. one per GPU) sum to the film of
                                     the whole range */
} slrgpu_settings;

/* settings.flags: record CUDA events around every launch and report the
 * device time per kernel class in slrgpu_render_stats.kernel_ms. */
#define SLRGPU_FLAG_PROFILE_KERNELS 1u
/* settings.flags: watertight ray-triangle test (Woop, Benthin, Wald 2013)
 * instead of the reference's Moller-Trumbore order, which can let a ray
 * through the shared edge of two triangles; hits then differ from the
 * reference only for rays within rounding of an edge or vertex. */
#define SLRGPU_FLAG_WATERTIGHT 2u
/* settings.flags: bidirectional path tracing, BPTRenderer(spp)
 * (libSLR/Renderer/BPTRenderer.h:117-123, BPTRenderer.cpp:25-431), or with
 * volumetric = 1 VolumetricBPTRenderer(spp) (VolumetricBPTRenderer.cpp),
 * instead of the path tracers.  max_depth (1..63) then caps each subpath at
 * max_depth vertices after its first (the reference ends subpaths by Russian
 * roulette only).  Surface lights and the environment.  Contributions
 * through the lens vertex land on the pixel they project to;
 * slrgpu_render_stats.dropped_samples counts non-finite contributions.  The
 * allocation-free render and the server return SLRGPU_ERR_UNSUPPORTED. */
#define SLRGPU_FLAG_BPT 4u

/* Kernel classes of the wavefront (index into kernel_ms / kernel_count). */
#define SLRGPU_KERNEL_RAYGEN 0
#define SLRGPU_KERNEL_EXTEND 1
#define SLRGPU_KERNEL_SHADE 2
#define SLRGPU_KERNEL_SHADOW 3
#define SLRGPU_KERNEL_ACCUMULATE 4
#define SLRGPU_KERNEL_CLASSES 8

typedef struct slrgpu_render_stats {
    double seconds;               /* wall time of the call */
    double kernel_seconds;        /* device time of the render kernels */
    uint64_t path_samples;        /* sample grid positions * spp */
    uint64_t extension_rays;      /* closest-hit queries traced */
    uint64_t shadow_rays;         /* any-hit queries traced */
    uint64_t dropped_samples;     /* non-finite contributions dropped */
    uint64_t kernel_launches;
    double kernel_ms[SLRGPU_KERNEL_CLASSES];      /* with SLRGPU_FLAG_PROFILE_KERNELS */
    uint64_t kernel_count[SLRGPU_KERNEL_CLASSES];
} slrgpu_render_stats;

/* Context ------------------------------------------------------------- */
int slrgpu_context_create(int device, slrgpu_handle* ctx);
int slrgpu_context_destroy(slrgpu_handle ctx);
const char* slrgpu_last_error(void);
int slrgpu_version(void);

/* Scene --------------------------------------------------------------- */
int slrgpu_scene_create(slrgpu_handle ctx, slrgpu_handle* scene);
int slrgpu_scene_destroy(slrgpu_handle scene);

/* Spectra: each returns a scene-local spectrum id in *id. */
int slrgpu_spectrum_rgb(slrgpu_handle scene, int spectrum_type, float r, float g, float b, int* id);
int slrgpu_spectrum_regular(slrgpu_handle scene, float min_wl, float max_wl,
                            const float* values, uint32_t num_values, int* id);
int slrgpu_spectrum_irregular(slrgpu_handle scene, const float* wavelengths, const float* values,
                              uint32_t num_values, int* id);

/* Materials: each returns a scene-local material id in *id. */
int slrgpu_material_matte(slrgpu_handle scene, int reflectance, int* id);
int slrgpu_material_specular_reflection(slrgpu_handle scene, int coeff, int eta, int k, int* id);
int slrgpu_material_specular_scattering(slrgpu_handle scene, int coeff, int eta_ext, int eta_int, int* id);
int slrgpu_material_microfacet_reflection(slrgpu_handle scene, int eta, int k,
                                          float alpha_x, float alpha_y, int* id);
int slrgpu_material_microfacet_scattering(slrgpu_handle scene, int eta_ext, int eta_int,
                                          float alpha_x, float alpha_y, int* id);
int slrgpu_material_emitter(slrgpu_handle scene, int base_material, int emittance, int* id);

/* Geometry: world-space vertices (positions/normals/tangents xyz, uvs uv),
 * triangles as vertex index triples. */
int slrgpu_scene_add_mesh(slrgpu_handle scene, const float* positions, const float* normals,
                          const float* tangents, const float* uvs, uint32_t num_vertices,
                          const uint32_t* indices, uint32_t num_triangles, int material);

/* Image-based environment: width*height linear RGBA texels as IEEE binary16
 * bit patterns; emitted radiance is texel * scale. */
int slrgpu_environment_ibl(slrgpu_handle scene, const uint16_t* rgba_half, uint32_t width,
                           uint32_t height, float scale);

/* Heterogeneous medium over an axis-aligned box: density[nz][ny][nx]
 * multiplies the sigma_s / sigma_e spectra; Henyey-Greenstein phase g. */
int slrgpu_medium_density_grid(slrgpu_handle scene, const float* bounds_min, const float* bounds_max,
                               int sigma_s, int sigma_e, const float* density, uint32_t nx,
                               uint32_t ny, uint32_t nz, float hg_g);

/* The same from the reference's raw density-grid file (the scene-graph
 * loader's format, libSLRSceneGraph/API.cpp:966-989): uint32 nx, ny, nz, then
 * nz slices of ny rows of nx float32, native byte order.  A short or
 * malformed file is an error (SLRGPU_ERR_INVALID_ARGUMENT). */
int slrgpu_medium_density_grid_file(slrgpu_handle scene, const char* path, const float* bounds_min,
                                    const float* bounds_max, int sigma_s, int sigma_e, float hg_g);

/* Cameras: cam_to_world is a row-major 4x4 matrix. */
int slrgpu_camera_perspective(slrgpu_handle scene, const float* cam_to_world, float sensitivity,
                              float aspect, float fov_y, float lens_radius, float img_plane_dist,
                              float obj_plane_dist);
int slrgpu_camera_equirect(slrgpu_handle scene, const float* cam_to_world, float sensitivity,
                           float phi_angle, float theta_angle);

/* Builds the SBVH, collapses it to the wide layout and uploads the scene to
 * device memory.  stats may be NULL. */
int slrgpu_scene_commit(slrgpu_handle scene, slrgpu_bvh_stats* stats);

/* Copies every device array of a committed scene again from its pinned host
 * mirror (stream-ordered before the next render); *bytes receives the bytes
 * copied.  This is the host-to-device part of an end-to-end render in which
 * the scene lives on the host. */
int slrgpu_scene_reupload(slrgpu_handle scene, uint64_t* bytes);

/* Rendering ----------------------------------------------------------- */
/* Blocking render.  film receives width*height*16 floats: per pixel (row
 * major) the 16-bin spectral sum over all samples, the value the reference's
 * ImageSensor::pixel(x, y) returns after PTRenderer::render.  As in the
 * reference, the sensor is sampled in whole 8 x 8 tiles: when width or height
 * is not a multiple of 8, the samples of the overhanging tile positions land
 * in the last column / row (PTRenderer.cpp:104-110, ImageSensor.cpp:125-130),
 * and stats->path_samples counts them.  film is a host pointer, or a device
 * pointer when film_on_device is nonzero. */
int slrgpu_render(slrgpu_handle scene, const slrgpu_settings* settings, float* film,
                  int film_on_device, slrgpu_render_stats* stats);

/* Path-level replay (diagnostics; no counterpart in the reference): one
 * sample per pixel of the surface path tracer in which the path of grid
 * position i (the tile-padded grid, row-major) draws its uniforms from
 * tapes[256 i .. 256 i + 256) instead of the renderer's own generator (draws
 * past 256 read 0.5).  Fed with the uniforms a reference path drew (recorded
 * in the reference's draw order: time, pixel, wavelength, wavelength
 * selection, lens; per vertex: Russian roulette after the first, light
 * selection, light position, BSDF), the GPU traces the same path, so films
 * can be compared path by path.  spp must be 1, sample_base 0, no
 * volumetric, watertight or bidirectional flag (SLRGPU_ERR_UNSUPPORTED);
 * max_depth at most 35 keeps a path's draws within its 256.  Allocates a
 * device copy of the tapes for the call. */
/* Diagnostics (no counterpart in the reference): the queue counters of the
 * last path-tracer wave rendered on the context, one row of 11 per bounce
 * (rows = max_depth + 2 of the context's path state): [0..4] paths shaded
 * per material kind, [5] paths that left the scene, [6] medium scattering
 * points, [7] paths in the bounce's extension queue, [8] shadow rays, [9]
 * shadow rays waiting for their transmittance, [10] a work counter.  These
 * are the units of each wave kernel's launch (for profiles).  capacity is
 * the size of counts in uint32. */
int slrgpu_context_queue_counts(slrgpu_handle ctx, uint32_t* counts, uint32_t capacity, uint32_t* rows);

int slrgpu_render_replay(slrgpu_handle scene, const slrgpu_settings* settings, const float* tapes, float* film,
                         slrgpu_render_stats* stats);

/* Checkpointed rendering (no counterpart in the reference, whose renderer
 * runs all passes in one call): renders samples [sample_base, sample_base +
 * spp) and adds them, in sample order, to the compensated film sums held in
 * film_state (host memory, 2 x 16 x width x height floats: the sum planes
 * [bin][pixel], then the compensation planes; all zeros for a fresh film),
 * updated in place.  film (host, optional) receives the film
 * (width*height*16 floats, the layout of slrgpu_render).  A film rendered
 * over consecutive sample ranges, the state saved and restored between the
 * calls, equals the one-call film bit for bit: the ranges are additive and
 * a sample's random numbers depend only on (seed, sample, pixel).  Path
 * tracers only (SLRGPU_FLAG_BPT: SLRGPU_ERR_UNSUPPORTED). */
int slrgpu_render_continue(slrgpu_handle scene, const slrgpu_settings* settings, float* film_state, float* film,
                           slrgpu_render_stats* stats);

/* Render that allocates nothing.  It has no counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc while they run: a real-time loop
 * with a fixed device-memory budget, a host application that owns the GPU's
 * allocator, or an embedding runtime that forbids allocation after start-up.
 * slrgpu_render needs per-context path-state buffers that it allocates (and
 * grows) on demand; this variant keeps the path state, queues, counters and
 * film sums in one fixed file-scope device array of
 * slrgpu_render_noalloc_scratch_bytes() bytes (about 29 MiB), which every GPU
 * that loads the library holds until the process exits.
 *
 * Limits: the sample grid, width and height each rounded up to a multiple
 * of 8 (the reference samples its sensor in whole 8 x 8 tiles), holds <= 65536
 * positions, and max_depth <= 64 (settings beyond them are rejected with
 * SLRGPU_ERR_INVALID_ARGUMENT and a message); each wave holds grid positions *
 * samples_per_wave <= 65536 paths (0 picks the largest).  film_device receives width*height*16 floats in the layout of
 * slrgpu_render.  The call is stream-ordered on `stream` (a cudaStream_t, or
 * NULL for the legacy default stream) and returns without waiting; the caller
 * synchronizes before reading the film.  The scene's own arrays were
 * allocated by slrgpu_scene_commit.
 *
 * The first call on a device, with that device current, looks up the device
 * address of the scratch array; make that first call before any stream
 * capture.  Every call shares the one array and clears what must start at
 * zero, so calls that overlap on the GPU (concurrent streams or threads)
 * race: serialize them.  With the same settings and samples_per_wave the
 * film equals slrgpu_render's.  SLRGPU_FLAG_PROFILE_KERNELS has no effect
 * here (there are no statistics to fill), and SLRGPU_FLAG_BPT is refused
 * (SLRGPU_ERR_UNSUPPORTED). */
int slrgpu_render_noalloc(slrgpu_handle scene, const slrgpu_settings* settings, float* film_device, void* stream);
uint64_t slrgpu_render_noalloc_scratch_bytes(void);

/* Serving ------------------------------------------------------------- *
 * No counterpart in the reference, whose renderers take one blocking render
 * call at a time.  A server renders queued requests (any committed scene of
 * its context, any resolution, spp and max depth) with continuous batching:
 * requests are admitted oldest first while their films fit the HBM budget;
 * in SLRGPU_SERVER_BATCHED mode each wave of launches carries the next
 * samples of up to 32 admitted requests with the same integrator and max
 * depth: for the surface path tracer, requests of up to 8 different scenes,
 * whose paths share one set of extension, shading and shadow queues (each
 * path finds its scene in the wave's scene table); for the volumetric path
 * tracer, requests of one scene.  Several waves run concurrently on separate
 * streams and path-state slots, a request in one wave at a time; requests
 * that arrive while others are on the GPU join the next wave.  SLRGPU_SERVER_PLAIN renders one request at a time, like
 * slrgpu_render.  A request's film is bit-identical in both modes and to
 * slrgpu_render with the same settings: its random numbers depend only on
 * (seed, sample, pixel) and its samples are accumulated in order.  A scene
 * cannot be destroyed while it has unfinished requests.
 *
 * The HBM budget covers everything the server holds on the device for its
 * requests: its path-state slots (charged at creation; creation fails if
 * they alone exceed it), each resident scene an admitted request renders
 * (charged once while any of its admitted requests is alive) and the
 * admitted requests' films (released by slrgpu_server_wait).  A request
 * whose film and scene can never fit is refused at submission. */
#define SLRGPU_SERVER_PLAIN 0u
#define SLRGPU_SERVER_BATCHED 1u

#define SLRGPU_REQUEST_QUEUED 0
#define SLRGPU_REQUEST_RUNNING 1
#define SLRGPU_REQUEST_DONE 2

typedef struct slrgpu_server_config {
    uint32_t mode;              /* SLRGPU_SERVER_PLAIN or SLRGPU_SERVER_BATCHED */
    uint32_t slots;             /* path-state slots = waves in flight; 0: 4 (plain: 1) */
    uint32_t paths_per_slot;    /* 0: 4 Mi paths (about 2 GB per slot) */
    uint32_t max_depth;         /* largest max_depth accepted; 0: 64 */
    uint64_t hbm_budget_bytes;  /* device bytes for slots, scenes and films (above); 0: 150 GB */
} slrgpu_server_config;

typedef struct slrgpu_request_info {
    int32_t status;             /* SLRGPU_REQUEST_* or a negative error code */
    uint32_t spp_done;
    double submit_seconds;      /* since the server's creation */
    double start_seconds;       /* admission */
    double done_seconds;
    uint64_t path_samples;      /* sample grid positions * spp done */
    uint64_t dropped_samples;
} slrgpu_request_info;

typedef struct slrgpu_server_stats {
    uint64_t requests_done;
    uint64_t path_samples_done;
    uint64_t waves;
    uint64_t kernel_launches;
    uint64_t bytes_in_use;      /* charged to the budget: slots, scenes, admitted films */
    uint32_t queued, active;
    double first_start_seconds;
    double last_done_seconds;
    uint64_t mixed_scene_waves; /* waves whose paths came from more than one scene */
} slrgpu_server_stats;

int slrgpu_server_create(slrgpu_handle ctx, const slrgpu_server_config* config, slrgpu_handle* server);
/* Finishes the waves on the GPU; queued requests end with an error status. */
int slrgpu_server_destroy(slrgpu_handle server);
int slrgpu_server_submit(slrgpu_handle server, slrgpu_handle scene, const slrgpu_settings* settings,
                         uint64_t* request);
int slrgpu_server_poll(slrgpu_handle server, uint64_t request, slrgpu_request_info* info);
/* Blocks until the request is done (timeout_seconds < 0: no limit;
 * SLRGPU_ERR_TIMEOUT otherwise), copies its film (width*height*16 floats,
 * the layout of slrgpu_render; film may be NULL) to host memory and
 * releases the request. */
int slrgpu_server_wait(slrgpu_handle server, uint64_t request, float* film, slrgpu_request_info* info,
                       double timeout_seconds);
int slrgpu_server_get_stats(slrgpu_handle server, slrgpu_server_stats* stats);
/* Cancels a queued or running request (no counterpart in the reference): a
 * queued request ends at once, a running one gets no more samples and ends
 * when its waves on the GPU finish; its status becomes SLRGPU_ERR_CANCELLED
 * and slrgpu_server_wait returns that code and releases it.  A request that
 * has finished, or whose film is already being converted, is left alone
 * (SLRGPU_ERR_STATE). */
int slrgpu_server_cancel(slrgpu_handle server, uint64_t request);
/* Sets a deadline, seconds from now: a request not finished by then is
 * cancelled by the server with status SLRGPU_ERR_TIMEOUT (checked at least
 * every 50 ms). */
int slrgpu_server_set_deadline(slrgpu_handle server, uint64_t request, double seconds);

/* Host-side fault injection for tests of the serving loop (no counterpart
 * in the reference): the next `count` film allocations
 * (SLRGPU_FAULT_SERVER_FILM_ALLOC) or wave launches
 * (SLRGPU_FAULT_SERVER_WAVE_LAUNCH) of any server in the process fail as if
 * the CUDA call had failed; nothing is injected on the GPU.  count 0 clears
 * the site. */
#define SLRGPU_FAULT_SERVER_FILM_ALLOC 0
#define SLRGPU_FAULT_SERVER_WAVE_LAUNCH 1
int slrgpu_debug_inject_fault(int site, uint32_t count);

/* Film output --------------------------------------------------------- *
 * ImageSensor::saveImage (libSLR/Core/ImageSensor.cpp:139-195) on the GPU: the
 * film (width*height*16 floats, the layout slrgpu_render writes) times
 * scale x sensitivity (an infinite sensitivity counts as 1) -> XYZ with the
 * CIE 1931 2-degree colour matching functions integrated over the 16 bins ->
 * sRGB -> 1 - exp(-x) -> sRGB gamma -> 8 bits.  pixels (optional) receives
 * the BMP pixel array: bottom-up rows of B, G, R bytes, each row padded to a
 * multiple of 4 bytes with zeros ((3*width + width%4) * height bytes); path
 * (optional) receives a 24-bit BMP file laid out as the reference's
 * (Helper/bmp_exporter.cpp:15-53). */
int slrgpu_film_to_bmp(const float* film, uint32_t width, uint32_t height, int film_on_device, float scale,
                       float sensitivity, uint8_t* pixels, const char* path);
/* The 16 film bins of the colour matching functions (x[16], y[16], z[16])
 * and their y integral (DiscretizedSpectrumTemplate::initialize,
 * spectrum_types.cpp:945-995).  Host only. */
int slrgpu_film_cmf(float* bins, float* integral);

/* Ray queries on the committed scene (device pointers).  rays: n x 8 floats
 * (org.xyz, tmin, dir.xyz, tmax).  any_hit bit 0: any hit (prim = 1 when
 * occluded, else 0), otherwise closest hit filling prim (0xffffffff on miss),
 * t, b1, b2 (barycentric weights of the second and third vertex); bit 1: the
 * watertight triangle test instead of the reference's.  stream is a
 * cudaStream_t or NULL. */
int slrgpu_trace(slrgpu_handle scene, const float* rays, uint32_t n, int any_hit, uint32_t* prim,
                 float* t, float* b1, float* b2, void* stream);

/* BSDF queries on the GPU at fixed inputs (the reference's BSDF::sample /
 * evaluate / evaluatePDF, directional_distribution_functions.h:295-349, on
 * LambertianBRDF, SpecularBRDF, SpecularBSDF, MicrofacetBRDF, MicrofacetBSDF;
 * kind 0..4 in that order).  spec0..2: 16 values each (R | coeff, eta, k |
 * coeff, etaExt, etaInt | eta, k | etaExt, etaInt).  Per query 16 floats:
 * dir.xyz, gnormal.xyz, wavelength index, adjoint (0), uComponent, uDir0,
 * uDir1, eval dir.xyz, 0, 0.  Per result 40 floats: sampled fs[16], sampled
 * dir.xyz, sampled pdf, sampled direction type, evaluated fs[16], evaluated
 * pdf, 0, 0.  Host arrays. */
int slrgpu_bsdf_query(int kind, const float* spec0, const float* spec1, const float* spec2, float alpha_x,
                      float alpha_y, const float* queries, uint32_t n, float* out);

/* Medium queries on the GPU on segments inside the committed scene's
 * density-grid medium, with the free-path sampler replaying given 32-bit
 * values as uniforms (value >> 9 as the mantissa, as the reference's
 * RandomNumberGenerator::getFloat0cTo1o; 0x80000000 once a query's values run
 * out).  mode 0: DensityGridMediumDistribution::interact
 * (DensityGridMediumDistribution.cpp:402-575), 1: ::evaluateTransmittance
 * (:577-744), 2: ::evaluateExtinctionCoefficient at the normalised position
 * rays[0..2] (:756-759); 3 and 4: MediumObjectAggregate::interact /
 * ::evaluateTransmittance (medium_object.cpp:287-402), which walk the
 * medium's boundary crossings, on segments anywhere.  rays: n x 8 (org.xyz, dist_min, dir.xyz, dist_max);
 * lambdas: n x 16 wavelengths; sel: n (selected index, | 0x100 when the
 * wavelength is already selected); vals: n x num_vals; out: n x 24 (hit,
 * distance, normalised position xyz, values drawn, spectrum[16], 0, 0).
 * Host arrays. */
int slrgpu_medium_query(slrgpu_handle scene, int mode, uint32_t n, const float* rays, const float* lambdas,
                        const int* sel, const uint32_t* vals, uint32_t num_vals, float* out);

/* Diagnostics (host side, no GPU needed) ------------------------------ */
/* Builds the SBVH and the other host tables without uploading
 * (the part of SurfaceObjectAggregate's constructor, surface_object.cpp:373-399,
 * and Scene::build, Scene.cpp:17-38, that runs on the CPU). */
int slrgpu_scene_build_host(slrgpu_handle scene, slrgpu_bvh_stats* stats);
/* Binary SBVH node dump (SBVH.h:21-43 node fields): per node boxes[6]
 * (min xyz, max xyz) and words[5] (c0, c1, first leaf, leaf count,
 * split axis or 0xffffffff for leaves); leaf_prims[num_fragments]. */
int slrgpu_scene_sbvh_dump(slrgpu_handle scene, float* boxes, uint32_t* words, uint32_t* leaf_prims);
/* Host evaluation of a spectrum at num_sets x 16 wavelengths
 * (ContinuousSpectrum::evaluate, spectrum_types.h:72-80). */
int slrgpu_spectrum_evaluate(slrgpu_handle scene, int id, const float* lambdas, uint32_t num_sets, float* out);
/* Environment importance map (image_textures.cpp:142-195,
 * distributions.cpp:215-281): row pdf [map_h][map_w], row cdf
 * [map_h][map_w + 1], top pdf [map_h], top cdf [map_h + 1], and per texel
 * (adjacency bits, s, t, scale) of its upsampled spectrum. */
int slrgpu_environment_tables(slrgpu_handle scene, uint32_t* map_w, uint32_t* map_h, float* row_pdf, float* row_cdf,
                              float* top_pdf, float* top_cdf, float* texel_params);
/* The alias tables the GPU samples lights and the environment with (Vose;
 * bin i is kept with probability prob[i], else alias[i] is taken), built
 * from the CDFs above, so they carry the same PMFs: surface lights
 * (num_lights entries), the environment's rows (map_h) and the bins of each
 * row (map_h x map_w).  Host only; any output may be NULL. */
int slrgpu_scene_alias_tables(slrgpu_handle scene, uint32_t* num_lights, float* light_prob, uint32_t* light_alias,
                              float* top_prob, uint32_t* top_alias, float* row_prob, uint32_t* row_alias);

#ifdef __cplusplus
}
#endif

#endif /* SLRGPU_H */
