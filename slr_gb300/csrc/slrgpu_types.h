// Device-resident scene layout shared by the host build code and the kernels.
// Plain structs only; every array lives in HBM and is read-only during a
// render.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SLRGPU_HD __host__ __device__ __forceinline__
#else
#define SLRGPU_HD inline
#endif

namespace slrgpu {

// 16 hero wavelengths over [360, 830) nm with equal offsets and a 16-bin
// film (libSLR/declarations.h:50-51, BasicTypes/spectrum_base.h:110-111).
constexpr int kNumLambda = 16;
constexpr float kWavelengthLow = 360.0f;
constexpr float kWavelengthHigh = 830.0f;
// Ray epsilon of the reference (libSLR/BasicTypes/Ray.h:29).
constexpr float kRayEpsilon = 1e-4f;
// Spectral upsampling grid (spectrum_types.cpp:391-394).
constexpr int kUpsNumSamples = 95;
constexpr int kUpsGridWidth = 12;
constexpr int kUpsGridHeight = 14;

enum SpectrumKind : uint32_t { kSpecUpsampled = 0, kSpecRegular = 1, kSpecIrregular = 2 };

// One input spectrum (32 B).
//   upsampled: adj = packed adjacent data-point indices (4 x u8; 0xFF in the
//              top byte means a 3-point barycentric cell), p0/p1 = s/t weights,
//              scale = brightness / EqualEnergyReflectance.
//   regular:   count samples at values[offset..], p0/p1 = min/max wavelength.
//   irregular: count samples; wavelengths at values[offset..], values at
//              values[offset + count..].
struct DevSpectrum {
    uint32_t kind;
    uint32_t adj;
    uint32_t offset;
    uint32_t count;
    float p0, p1;
    float scale;
    float pad;
};

enum MaterialKind : uint32_t {
    kMatMatte = 0,          // LambertianBRDF(R)                    spec[0] = R
    kMatSpecularReflection, // SpecularBRDF(coeff, eta, k)          spec = coeff, eta, k
    kMatSpecularScattering, // SpecularBSDF(coeff, etaExt, etaInt)  spec = coeff, etaExt, etaInt
    kMatGGXReflection,      // MicrofacetBRDF(eta, k, GGX)          spec = eta, k
    kMatGGXScattering,      // MicrofacetBSDF(etaExt, etaInt, GGX)  spec = etaExt, etaInt
    kMatNull,               // no BSDF (environment)
};

struct DevMaterial {        // 32 B
    uint32_t kind;
    int32_t spec[3];
    float alphaX, alphaY;
    int32_t emit;           // emittance spectrum, -1 when not emitting
    uint32_t pad;
};

// Per input triangle (32 B): vertex indices, material, geometric normal
// normalize(cross(p1 - p0, p2 - p0)) and 1 / area.
struct DevPrim {
    uint32_t v0, v1, v2, material;
    float ngx, ngy, ngz, invArea;
};

// Wide BVH node: kBvhWidth children (4 or 8, a compile-time tuning constant
// shared by the host build and the kernels), SoA boxes: one 128-byte line
// for 4-wide, two for 8-wide, read as 128-bit loads.
// child[k]: 0xffffffff = empty; bit 31 set = leaf with first fragment in
// bits [0, 26) and (count - 1) in bits [26, 31); else internal node index.
#ifndef SLRGPU_BVH_WIDTH
#define SLRGPU_BVH_WIDTH 4
#endif
constexpr int kBvhWidth = SLRGPU_BVH_WIDTH;
static_assert(kBvhWidth == 4 || kBvhWidth == 8, "BVH width 4 or 8");
constexpr uint32_t kChildEmpty = 0xffffffffu;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kLeafCountShift = 26;
constexpr uint32_t kLeafFirstMask = (1u << kLeafCountShift) - 1;
constexpr int kMaxLeafCount = 32;

struct alignas(128) BvhNode {
    float lox[kBvhWidth], hix[kBvhWidth], loy[kBvhWidth], hiy[kBvhWidth], loz[kBvhWidth], hiz[kBvhWidth];
    uint32_t child[kBvhWidth];
    uint32_t pad[kBvhWidth];
};
static_assert(sizeof(BvhNode) == 32 * kBvhWidth, "whole cache lines");

// Traversal fragment (48 B, leaf order): v0.xyz + prim id bits, e01 = p1 - p0,
// e02 = p2 - p0 (precomputed with the same float subtraction as the test).
struct TriFrag {
    float v0x, v0y, v0z;
    uint32_t prim;
    float e1x, e1y, e1z, pad0;
    float e2x, e2y, e2z, pad1;
};

struct DevCamera {
    uint32_t kind;          // 0 perspective (thin lens), 1 equirectangular
    float sensitivity;
    float org[3];           // lens centre (world)
    float ex[3], ey[3], ez[3];  // lens frame (world): x, y = cross(z, x), z = lens normal
    float opWidth, opHeight, objPlaneDist, imgPlaneDist, imgPlaneArea, lensRadius;
    float phiAngle, thetaAngle;
};

// Environment texel: upsampled spectrum per texel (16 B).
struct EnvTexel {
    uint32_t adj;
    float s, t, scale;
};

// Heterogeneous medium: density grid over an axis-aligned box with a
// super-voxel majorant grid (DensityGridMediumDistribution).
struct DevMedium {
    uint32_t present;
    uint32_t nx, ny, nz;          // density samples per axis
    uint32_t svx, svy, svz;       // super-voxel corners per axis
    float bmin[3], bmax[3];
    float svWidth[3];             // (bmax - bmin) / (sv - 1)
    float invSvWidth[3];          // 1 / svWidth
    float invExtent[3];           // 1 / (bmax - bmin)
    const float* density;         // [nz][ny][nx]
    const float* superVoxels;     // [svz][svy][svx]
    const float* maxDiff;         // [svz-1][svy-1][svx-1]
    int32_t sigmaS, sigmaE;       // spectrum ids
    float g;                      // Henyey-Greenstein asymmetry
    float importance;             // emitting media weight (0: none emit)
};

// Alias table entry (Vose): bin i is kept with probability prob, else its
// alias is taken; built from a CDF, so the bins keep the CDF's PMF.
struct AliasEntry {
    float prob;
    uint32_t alias;
};

struct DevScene {
    // geometry / traversal
    const BvhNode* nodes;
    const TriFrag* frags;
    const float4* wtVerts;  // per fragment: v0 (w = prim id bits), v1, v2 as given (watertight test)
    uint32_t watertight;    // 1: watertight triangle test instead of the reference's
    // path-level replay (slrgpu_render_replay): kRngTapeStride uniforms per
    // grid position that the path tracer draws instead of its own; null
    // otherwise
    const float* rngTape;
    const DevPrim* prims;
    const float4* vpos;     // xyz, u
    const float4* vnrm;     // xyz, v
    const float4* vtan;     // xyz, 0
    uint32_t numPrims;
    uint32_t numNodes;
    // materials / spectra
    const DevMaterial* materials;
    const DevSpectrum* spectra;
    const float* specValues;
    const float* upsSpectra;   // [numPoints][95]
    // surface lights: emitting prims in aggregate order, CDF over them
    const uint32_t* lightPrims;
    const float* lightCDF;     // numLights + 1
    const float* lightPMF;     // numLights
    const AliasEntry* lightAlias;   // numLights
    uint32_t numLights;
    float surfImportance;      // SurfaceObjectAggregate::importance()
    float envImportance;       // 1 when an environment is present, else 0
    // environment
    uint32_t envPresent;
    uint32_t envWidth, envHeight;
    float envScale;
    const EnvTexel* envTexels;
    uint32_t envMapW, envMapH;
    const float* envRowPDF;    // [mapH][mapW]
    const float* envRowCDF;    // [mapH][mapW + 1]
    const float* envTopPDF;    // [mapH]
    const float* envTopCDF;    // [mapH + 1]
    const AliasEntry* envRowAlias;  // [mapH][mapW]
    const AliasEntry* envTopAlias;  // [mapH]
    float worldRadius;
    float worldDiscArea;
    float worldCenter[3];
    DevCamera camera;
    DevMedium medium;
};

}  // namespace slrgpu
