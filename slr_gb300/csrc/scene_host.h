// Host-side scene representation and builders (spectra, environment tables,
// SBVH, wide-BVH collapse).  Compiled with -ffp-contract=off so that every
// float operation rounds exactly as the reference's build does.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <vector_types.h>

#include "slrgpu_types.h"

namespace slrgpu {

// ---- IEEE binary16 ---------------------------------------------------------
// float -> half with the reference's default rounding (half.hpp
// HALF_ROUND_STYLE = round_indeterminate: truncation toward zero, overflow to
// infinity).
uint16_t floatToHalfTrunc(float f);
float halfToFloat(uint16_t h);

// ---- spectra ---------------------------------------------------------------
int upsNumPoints();
const float* upsSpectra();                       // [numPoints][95]
void upsComputeAdjacents(float u, float v, uint32_t* adj, float* s, float* t);
void srgbToUVS(int spType, const float rgb[3], float uvs[3]);
void uvsToSRGB(int spType, const float uvs[3], float rgb[3]);
DevSpectrum upsampledFromRGB(int spType, float r, float g, float b);
// Host evaluation of a spectrum at 16 wavelengths (same arithmetic as the
// device code); used by tests through the C ABI helper.
void evaluateSpectrum(const DevSpectrum &sp, const float* values, const float* lambdas, float* out);

// ---- SBVH --------------------------------------------------------------------
struct SbvhNode {
    float bmin[3], bmax[3];
    uint32_t c0, c1, offset, count;   // leaf: leafPrims[offset..offset+count)
    uint32_t axis;
    uint32_t leaf;                    // 1 for leaves (a leaf may hold 0 prims)
};

struct SbvhResult {
    std::vector<SbvhNode> nodes;
    std::vector<uint32_t> leafPrims;
    uint32_t depth = 0;
    uint32_t numFragments = 0;
    float cost = 0.0f;
    float bmin[3], bmax[3];
};

// Builds the binned-SAH BVH with spatial splits over triangles given as
// positions[3 * nt][3] (float).
bool buildSbvh(const float* triPositions, uint32_t numTris, SbvhResult* out, std::string* err);

// ---- wide BVH -----------------------------------------------------------------
struct WideBvh {
    std::vector<BvhNode> nodes;
    std::vector<TriFrag> frags;
};
void collapseToWide(const SbvhResult &b, const float* triPositions, WideBvh* out);

// ---- environment ----------------------------------------------------------------
struct HostEnvironment {
    uint32_t width = 0, height = 0;
    float scale = 1.0f;
    std::vector<EnvTexel> texels;          // row-major
    uint32_t mapW = 0, mapH = 0;
    std::vector<float> rowPDF, rowCDF, rowIntegral, topPDF, topCDF;
    std::vector<AliasEntry> rowAlias, topAlias;
    float integral = 0.0f;
};
void buildEnvironment(const uint16_t* rgbaHalf, uint32_t w, uint32_t h, float scale, HostEnvironment* env);
// Alias table with the PMF cdf[i + 1] - cdf[i] of the n bins of a CDF.
void buildAlias(const float* cdf, uint32_t n, AliasEntry* out);

// ---- scene ---------------------------------------------------------------------
struct HostMesh {
    std::vector<float> pos, nrm, tan, uv;
    std::vector<uint32_t> idx;
    int material;
};

struct HostMedium {
    bool present = false;
    float bmin[3], bmax[3];
    int sigmaS = -1, sigmaE = -1;
    uint32_t nx = 0, ny = 0, nz = 0;
    std::vector<float> density;
    float g = 0.0f;
};

struct HostScene {
    std::vector<DevSpectrum> spectra;
    std::vector<float> specValues;
    std::vector<DevMaterial> materials;
    std::vector<HostMesh> meshes;
    bool envPresent = false;
    std::vector<uint16_t> envRGBA;
    uint32_t envW = 0, envH = 0;
    float envScale = 1.0f;
    bool cameraPresent = false;
    uint32_t cameraKind = 0;
    float camMatrix[16];
    float camSensitivity = 1, camAspect = 1, camFovY = 1, camLensRadius = 0, camImgDist = 1, camObjDist = 1;
    float camPhiAngle = 0, camThetaAngle = 0;
    HostMedium medium;
};

// Super-voxel majorant grid of a density medium.
struct HostSuperVoxels {
    uint32_t svx = 0, svy = 0, svz = 0;
    float width[3];
    std::vector<float> corners;    // [svz][svy][svx]
    std::vector<float> maxDiff;    // [svz-1][svy-1][svx-1]
};
void buildSuperVoxels(const HostMedium &m, HostSuperVoxels* sv);
// Trilinear density at a normalised position in [0,1]^3 (0 outside).
float densityAt(const HostMedium &m, const float param[3]);

// Flattened, device-ready arrays produced by commit.
struct BuiltScene {
    HostSuperVoxels superVoxels;
    SbvhResult sbvh;
    WideBvh wide;
    std::vector<DevPrim> prims;
    std::vector<float4> vpos, vnrm, vtan;
    std::vector<uint32_t> lightPrims;
    std::vector<float> lightCDF, lightPMF;
    std::vector<AliasEntry> lightAlias;
    HostEnvironment env;
    DevCamera camera;
    float worldCenter[3], worldRadius, worldDiscArea;
    float buildSeconds = 0.0f;
};

bool buildScene(const HostScene &s, BuiltScene* out, std::string* err);

// The colour matching functions integrated over the 16 film bins and the
// sum of the y bins (the reference's DiscretizedSpectrum::xbar/ybar/zbar and
// integralCMF).
void discretizedCmf(float xbar[16], float ybar[16], float zbar[16], float* integral);

}  // namespace slrgpu
