// Host-side scene builders.  Compiled with -ffp-contract=off: the spectral
// upsampling, environment tables and SBVH build reproduce the reference's
// float arithmetic operation by operation, so that identical inputs give
// bit-identical spectra, importance maps and BVH trees.
#include "scene_host.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace slrgpu {

#include "upsampling_table.inc"

namespace {
constexpr double kPi = 3.14159265358979323846;
// 1 / integral of a CMF (spectrum_types.h:207; UPSAMPLED_CONTINOUS_SPECTRUM_SCALE_FACTOR).
constexpr float kEqualEnergyReflectance = 0.009355121400914532f;
constexpr double kUvsScaleFactor = 0.009355121400914532;

float bitsToFloat(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }
float4 f4(float x, float y, float z, float w) { float4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }

struct UpsTables {
    float uv[SLRGPU_UPS_NUM_POINTS][2];
    float spectra[SLRGPU_UPS_NUM_POINTS][95];
    UpsTables() {
        for (int i = 0; i < SLRGPU_UPS_NUM_POINTS; ++i) {
            uv[i][0] = bitsToFloat(kUpsPointUVBits[i][0]);
            uv[i][1] = bitsToFloat(kUpsPointUVBits[i][1]);
            for (int k = 0; k < 95; ++k)
                spectra[i][k] = bitsToFloat(kUpsPointSpectrumBits[i][k]);
        }
    }
};
const UpsTables &ups() { static UpsTables t; return t; }
}  // namespace

// ============================================================================
// binary16
// ============================================================================
uint16_t floatToHalfTrunc(float f) {
    uint32_t bits;
    std::memcpy(&bits, &f, 4);
    uint16_t sign = (uint16_t)((bits >> 16) & 0x8000u);
    uint32_t e = (bits >> 23) & 0xffu;
    uint32_t mant = bits & 0x7fffffu;
    uint16_t h;
    if (e == 255u)
        h = (uint16_t)(0x7c00u + (mant >> 13));
    else if (e >= 143u)
        h = 0x7c00u;                                  // overflow -> infinity
    else if (e >= 113u)
        h = (uint16_t)(((e - 112u) << 10) + (mant >> 13));
    else if (e >= 103u)
        h = (uint16_t)((0x400u >> (113u - e)) + (mant >> (126u - e)));
    else
        h = 0;
    return (uint16_t)(sign | h);
}

float halfToFloat(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    uint32_t bits;
    if (e == 0) {
        if (m == 0) {
            bits = sign;
        } else {
            int shift = 0;
            while ((m & 0x400u) == 0) { m <<= 1; ++shift; }
            m &= 0x3ffu;
            bits = sign | ((uint32_t)(113 - shift) << 23) | (m << 13);
        }
    } else if (e == 31) {
        bits = sign | 0x7f800000u | (m << 13);
    } else {
        bits = sign | ((e + 112u) << 23) | (m << 13);
    }
    return bitsToFloat(bits);
}

// ============================================================================
// Spectral upsampling (Meng et al. 2015) - the arithmetic of
// UpsampledContinuousSpectrumTemplate (spectrum_types.cpp:424-543,
// spectrum_types.h:205-260).
// ============================================================================
int upsNumPoints() { return SLRGPU_UPS_NUM_POINTS; }
const float* upsSpectra() { return &ups().spectra[0][0]; }

void upsComputeAdjacents(float u, float v, uint32_t* adj, float* s, float* t) {
    u = std::min(std::max(u, 0.0f), (float)kUpsGridWidth);
    v = std::min(std::max(v, 0.0f), (float)kUpsGridHeight);
    int32_t ui = (int32_t)u;
    int32_t vi = (int32_t)v;
    // u == 12 or v == 14 would index past the grid; clamp to the last cell.
    ui = std::min(ui, kUpsGridWidth - 1);
    vi = std::min(vi, kUpsGridHeight - 1);
    const unsigned char* cell = kUpsGridCells[ui + kUpsGridWidth * vi];
    const unsigned char inside = cell[0], numPoints = cell[1];
    const unsigned char* indices = cell + 2;
    const UpsTables &T = ups();
    if (inside) {
        *adj = ((uint32_t)indices[3] << 24) | ((uint32_t)indices[2] << 16) |
               ((uint32_t)indices[1] << 8) | (uint32_t)indices[0];
        *s = u - ui;
        *t = v - vi;
        return;
    }
    // Triangle fan around indices[0]: find the triangle containing (u, v).
    const float ex = u - T.uv[indices[0]][0];
    const float ey = v - T.uv[indices[0]][1];
    float e0x = T.uv[indices[1]][0] - T.uv[indices[0]][0];
    float e0y = T.uv[indices[1]][1] - T.uv[indices[0]][1];
    float uu = e0x * ey - ex * e0y;
    bool found = false;
    for (int i = 1; i < numPoints; ++i) {
        uint32_t idx = indices[i % (numPoints - 1) + 1];
        float e1x = T.uv[idx][0] - T.uv[indices[0]][0];
        float e1y = T.uv[idx][1] - T.uv[indices[0]][1];
        float vv = ex * e1y - e1x * ey;
        const float area = e0x * e1y - e1x * e0y;
        const float b0 = uu / area;
        const float b1 = vv / area;
        float b2 = 1.0f - b0 - b1;
        if (b0 < -1e-6f || b1 < -1e-6f || b2 < -1e-6f) {
            uu = -vv;
            e0x = e1x;
            e0y = e1y;
            continue;
        }
        *adj = (0xffu << 24) | ((uint32_t)indices[0] << 16) | ((uint32_t)indices[i] << 8) | idx;
        *s = b0;
        *t = b1;
        found = true;
        break;
    }
    if (!found) {
        // Outside the quantised spectral locus: fall back to the fan centre.
        *adj = (0xffu << 24) | ((uint32_t)indices[0] << 16) | ((uint32_t)indices[0] << 8) | indices[0];
        *s = 1.0f;
        *t = 0.0f;
    }
}

namespace {
void xyToUV(const float xy[2], float uv[2]) {
    uv[0] = (float)(16.730260708356887 * xy[0] + 7.7801960340706 * xy[1] - 2.170152247475828);
    uv[1] = (float)(-7.530081094743006 * xy[0] + 16.192422314095225 * xy[1] + 1.1125529268825947);
}
void uvToXY(const float uv[2], float xy[2]) {
    xy[0] = (float)(0.0491440520940413 * uv[0] - 0.02361291916573777 * uv[1] + 0.13292069743203658);
    xy[1] = (float)(0.022853819546830627 * uv[0] + 0.05077639329371236 * uv[1] - 0.006895157122499944);
}
// sRGB (D65 white) and equal-energy-white sRGB matrices (spectrum_base.h:61-86).
void srgbToXYZ(const float rgb[3], float xyz[3]) {
    xyz[0] = (float)(0.4124564 * rgb[0] + 0.3575761 * rgb[1] + 0.1804375 * rgb[2]);
    xyz[1] = (float)(0.2126729 * rgb[0] + 0.7151522 * rgb[1] + 0.0721750 * rgb[2]);
    xyz[2] = (float)(0.0193339 * rgb[0] + 0.1191920 * rgb[1] + 0.9503041 * rgb[2]);
}
void xyzToSRGB(const float xyz[3], float rgb[3]) {
    rgb[0] = (float)(3.2404542 * xyz[0] - 1.5371385 * xyz[1] - 0.4985314 * xyz[2]);
    rgb[1] = (float)(-0.9692660 * xyz[0] + 1.8760108 * xyz[1] + 0.0415560 * xyz[2]);
    rgb[2] = (float)(0.0556434 * xyz[0] - 0.2040259 * xyz[1] + 1.0572252 * xyz[2]);
}
void srgbEToXYZ(const float rgb[3], float xyz[3]) {
    xyz[0] = (float)(0.4969 * rgb[0] + 0.3391 * rgb[1] + 0.1640 * rgb[2]);
    xyz[1] = (float)(0.2562 * rgb[0] + 0.6782 * rgb[1] + 0.0656 * rgb[2]);
    xyz[2] = (float)(0.0233 * rgb[0] + 0.1130 * rgb[1] + 0.8637 * rgb[2]);
}
void xyzToSRGBE(const float xyz[3], float rgb[3]) {
    rgb[0] = (float)(2.6897 * xyz[0] - 1.2759 * xyz[1] - 0.4138 * xyz[2]);
    rgb[1] = (float)(-1.0221 * xyz[0] + 1.9783 * xyz[1] + 0.0438 * xyz[2]);
    rgb[2] = (float)(0.0612 * xyz[0] - 0.2245 * xyz[1] + 1.1633 * xyz[2]);
}
float srgbToLuminance(float r, float g, float b) {
    return (float)(0.2126729 * r + 0.7151522 * g + 0.0721750 * b);
}
}  // namespace

void srgbToUVS(int spType, const float rgb[3], float uvs[3]) {
    float xyz[3] = {0, 0, 0};
    if (spType == 1) srgbToXYZ(rgb, xyz);
    else srgbEToXYZ(rgb, xyz);
    float xy[2];
    float b = xyz[0] + xyz[1] + xyz[2];
    xy[0] = xyz[0] / b;
    xy[1] = xyz[1] / b;
    if (b == 0)
        xy[0] = xy[1] = (float)(1.0f / 3.0);
    xyToUV(xy, uvs);
    uvs[2] = b / kEqualEnergyReflectance;
}

void uvsToSRGB(int spType, const float uvs[3], float rgb[3]) {
    float xy[2];
    uvToXY(uvs, xy);
    float b = uvs[2] * kEqualEnergyReflectance;
    float XYZ[3];
    XYZ[0] = xy[0] * b;
    XYZ[1] = xy[1] * b;
    XYZ[2] = b - XYZ[0] - XYZ[1];
    if (spType == 1) xyzToSRGB(XYZ, rgb);
    else xyzToSRGBE(XYZ, rgb);
}

DevSpectrum upsampledFromRGB(int spType, float r, float g, float b) {
    DevSpectrum sp{};
    sp.kind = kSpecUpsampled;
    float rgb[3] = {r, g, b};
    float XYZ[3];
    if (spType == 1) srgbToXYZ(rgb, XYZ);
    else srgbEToXYZ(rgb, XYZ);
    float brightness = XYZ[0] + XYZ[1] + XYZ[2];
    if (brightness == 0) {
        sp.scale = 0;
        upsComputeAdjacents(6, 4, &sp.adj, &sp.p0, &sp.p1);
        return sp;
    }
    float xy[2] = {XYZ[0] / brightness, XYZ[1] / brightness};
    sp.scale = brightness / kEqualEnergyReflectance;
    float uv[2];
    xyToUV(xy, uv);
    upsComputeAdjacents(uv[0], uv[1], &sp.adj, &sp.p0, &sp.p1);
    return sp;
}

void evaluateSpectrum(const DevSpectrum &sp, const float* values, const float* lambdas, float* out) {
    if (sp.kind == kSpecUpsampled) {
        uint8_t a[4] = {(uint8_t)(sp.adj & 0xff), (uint8_t)((sp.adj >> 8) & 0xff),
                        (uint8_t)((sp.adj >> 16) & 0xff), (uint8_t)(sp.adj >> 24)};
        float w[4];
        int n;
        if (a[3] != 0xff) {
            w[0] = (1 - sp.p0) * (1 - sp.p1); w[1] = sp.p0 * (1 - sp.p1);
            w[2] = (1 - sp.p0) * sp.p1; w[3] = sp.p0 * sp.p1; n = 4;
        } else {
            w[0] = sp.p0; w[1] = sp.p1; w[2] = 1.0f - sp.p0 - sp.p1; n = 3;
        }
        const UpsTables &T = ups();
        for (int i = 0; i < kNumLambda; ++i) {
            float p = (lambdas[i] - 360.0f) / (830.0f - 360.0f);
            p = std::min(std::max(p, 0.0f), 1.0f);
            float sBinF = p * (float)(kUpsNumSamples - 1);
            uint32_t sBin = std::min((uint32_t)sBinF, (uint32_t)(kUpsNumSamples - 1));
            uint32_t sBinNext = std::min(sBin + 1, (uint32_t)(kUpsNumSamples - 1));
            float t = sBinF - sBin;
            float acc = 0.0f;
            for (int j = 0; j < n; ++j)
                acc += w[j] * (T.spectra[a[j]][sBin] * (1 - t) + T.spectra[a[j]][sBinNext] * t);
            out[i] = acc * sp.scale;
        }
    } else if (sp.kind == kSpecRegular) {
        const float* v = values + sp.offset;
        for (int i = 0; i < kNumLambda; ++i) {
            float binF = (lambdas[i] - sp.p0) / (sp.p1 - sp.p0) * (float)(sp.count - 1);
            if (binF <= 0.0f) { out[i] = v[0]; continue; }
            if (binF >= (float)(sp.count - 1)) { out[i] = v[sp.count - 1]; continue; }
            int32_t bin = (int32_t)binF;
            float t = binF - bin;
            out[i] = (1 - t) * v[bin] + t * v[bin + 1];
        }
    } else {
        const float* wl = values + sp.offset;
        const float* v = wl + sp.count;
        uint32_t base = 0;
        for (int i = 0; i < kNumLambda; ++i) {
            int32_t low = std::max((int32_t)(std::lower_bound(wl + base, wl + sp.count, lambdas[i]) - wl) - 1, 0);
            base = (uint32_t)low;
            if (low >= (int32_t)sp.count - 1) { out[i] = v[sp.count - 1]; continue; }
            float t = (lambdas[i] - wl[low]) / (wl[low + 1] - wl[low]);
            if (t <= 0.0f) { out[i] = v[0]; continue; }
            out[i] = (1 - t) * v[low] + t * v[low + 1];
        }
    }
}

// ============================================================================
// Environment: RGBA16F -> uvs texels (image_2d.h:270-291), per-texel
// upsampled spectrum, and the luminance importance map over (W/4) x (H/4)
// area-averaged blocks weighted by sin(theta) (image_textures.cpp:142-195,
// image_2d.cpp:205-305, distributions.cpp:215-281).
// ============================================================================
namespace {
struct UvsA { uint16_t u, v, s, a; };

struct Kahan {
    float result = 0.0f, comp = 0.0f;
    void add(float value) {
        float cInput = value - comp;
        float sumTemp = result + cInput;
        comp = (sumTemp - result) - cInput;
        result = sumTemp;
    }
};

UvsA areaAverageUvs(const std::vector<UvsA> &img, uint32_t w, float xLeft, float xRight, float yTop, float yBottom) {
    uint32_t xLeftPix = (uint32_t)xLeft;
    uint32_t xRightPix = (uint32_t)std::ceil(xRight) - 1;
    uint32_t yTopPix = (uint32_t)yTop;
    uint32_t yBottomPix = (uint32_t)std::ceil(yBottom) - 1;
    float area = (yBottom - yTop) * (xRight - xLeft);
    float cc[4] = {(xLeftPix + 1 - xLeft) * (yTopPix + 1 - yTop), (xRight - xRightPix) * (yTopPix + 1 - yTop),
                   (xLeftPix + 1 - xLeft) * (yBottom - yBottomPix), (xRight - xRightPix) * (yBottom - yBottomPix)};
    float ce[4] = {yTopPix + 1 - yTop, xLeftPix + 1 - xLeft, xRight - xRightPix, yBottom - yBottomPix};
    Kahan sr, sg, sb, sa;
    auto add = [&](uint32_t x, uint32_t y, float coeff, bool weighted) {
        const UvsA &p = img[(size_t)y * w + x];
        float uvs[3] = {halfToFloat(p.u), halfToFloat(p.v), halfToFloat(p.s)};
        float rgb[3];
        uvsToSRGB(1, uvs, rgb);
        if (weighted) {
            sr.add(coeff * rgb[0]); sg.add(coeff * rgb[1]); sb.add(coeff * rgb[2]); sa.add(coeff * halfToFloat(p.a));
        } else {
            sr.add(rgb[0]); sg.add(rgb[1]); sb.add(rgb[2]); sa.add(halfToFloat(p.a));
        }
    };
    uint32_t corners[8] = {xLeftPix, yTopPix, xRightPix, yTopPix, xLeftPix, yBottomPix, xRightPix, yBottomPix};
    for (int i = 0; i < 4; ++i) add(corners[2 * i], corners[2 * i + 1], cc[i], true);
    for (uint32_t x = xLeftPix + 1; x < xRightPix; ++x) { add(x, yTopPix, ce[0], true); add(x, yBottomPix, ce[3], true); }
    for (uint32_t y = yTopPix + 1; y < yBottomPix; ++y) { add(xLeftPix, y, ce[1], true); add(xRightPix, y, ce[2], true); }
    for (uint32_t y = yTopPix + 1; y < yBottomPix; ++y)
        for (uint32_t x = xLeftPix + 1; x < xRightPix; ++x) add(x, y, 0.0f, false);
    float rgb[3] = {sr.result / area, sg.result / area, sb.result / area};
    float uvs[3];
    srgbToUVS(1, rgb, uvs);
    UvsA ret{floatToHalfTrunc(uvs[0]), floatToHalfTrunc(uvs[1]), floatToHalfTrunc(uvs[2]),
             floatToHalfTrunc(sa.result / area)};
    return ret;
}

// RegularConstantContinuousDistribution1D construction (distributions.cpp:168-190).
void build1D(const std::vector<float> &vals, float* pdf, float* cdf, float* integral) {
    const uint32_t n = (uint32_t)vals.size();
    for (uint32_t i = 0; i < n; ++i) pdf[i] = vals[i];
    Kahan sum;
    cdf[0] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        sum.add(pdf[i] / n);
        cdf[i + 1] = sum.result;
    }
    *integral = sum.result;
    if (sum.result > 0) {
        for (uint32_t i = 0; i < n; ++i) {
            pdf[i] /= sum.result;
            cdf[i + 1] /= sum.result;
        }
    }
}
}  // namespace

// Vose's alias method in double precision: the bins' probabilities are the
// CDF's increments (the PMF the CDF inversion samples), scaled to mean 1;
// bins below 1 take an alias among those above.
void buildAlias(const float* cdf, uint32_t n, AliasEntry* out) {
    std::vector<double> q(n);
    double total = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        q[i] = std::max(0.0, (double)cdf[i + 1] - (double)cdf[i]);
        total += q[i];
    }
    for (uint32_t i = 0; i < n; ++i) q[i] = total > 0 ? q[i] * n / total : 1.0;
    std::vector<uint32_t> small, large;
    for (uint32_t i = 0; i < n; ++i) (q[i] < 1.0 ? small : large).push_back(i);
    for (uint32_t i = 0; i < n; ++i) out[i] = AliasEntry{1.0f, i};
    while (!small.empty() && !large.empty()) {
        uint32_t s = small.back(), l = large.back();
        small.pop_back();
        out[s] = AliasEntry{(float)q[s], l};
        q[l] = (q[l] + q[s]) - 1.0;
        if (q[l] < 1.0) {
            large.pop_back();
            small.push_back(l);
        }
    }
    // leftovers (rounding) keep themselves with probability 1
    for (uint32_t i : large) out[i] = AliasEntry{1.0f, i};
    for (uint32_t i : small) out[i] = AliasEntry{1.0f, i};
}

void buildEnvironment(const uint16_t* rgbaHalf, uint32_t w, uint32_t h, float scale, HostEnvironment* env) {
    env->width = w;
    env->height = h;
    env->scale = scale;
    std::vector<UvsA> img((size_t)w * h);
    env->texels.resize((size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        float rgb[3] = {std::max(halfToFloat(rgbaHalf[4 * i + 0]), 0.0f), std::max(halfToFloat(rgbaHalf[4 * i + 1]), 0.0f),
                        std::max(halfToFloat(rgbaHalf[4 * i + 2]), 0.0f)};
        float uvs[3];
        srgbToUVS(1, rgb, uvs);
        img[i] = UvsA{floatToHalfTrunc(uvs[0]), floatToHalfTrunc(uvs[1]),
                      floatToHalfTrunc((float)(uvs[2] * kUvsScaleFactor)), rgbaHalf[4 * i + 3]};
        // Lookup-time spectrum: UpsampledContinuousSpectrum(u, v, s / factor)
        // (image_textures.cpp:29-33).
        EnvTexel &t = env->texels[i];
        float u = halfToFloat(img[i].u), v = halfToFloat(img[i].v);
        t.scale = (float)(halfToFloat(img[i].s) / kUvsScaleFactor);
        upsComputeAdjacents(u, v, &t.adj, &t.s, &t.t);
    }
    const uint32_t mapW = w / 4, mapH = h / 4;
    env->mapW = mapW;
    env->mapH = mapH;
    const float deltaX = (float)(w / mapW), deltaY = (float)(h / mapH);
    env->rowPDF.assign((size_t)mapW * mapH, 0.0f);
    env->rowCDF.assign((size_t)(mapW + 1) * mapH, 0.0f);
    env->rowIntegral.assign(mapH, 0.0f);
    Kahan total;
    std::vector<float> vals(mapW);
    for (uint32_t y = 0; y < mapH; ++y) {
        for (uint32_t x = 0; x < mapW; ++x) {
            UvsA avg = areaAverageUvs(img, w, x * deltaX, (x + 1) * deltaX, y * deltaY, (y + 1) * deltaY);
            float uvs[3] = {halfToFloat(avg.u), halfToFloat(avg.v), halfToFloat(avg.s)};
            float rgb[3];
            uvsToSRGB(1, uvs, rgb);
            float lum = srgbToLuminance(rgb[0], rgb[1], rgb[2]);
            vals[x] = (float)(std::sin(kPi * (double)(y + 0.5f) / (double)mapH) * (double)lum);
        }
        build1D(vals, &env->rowPDF[(size_t)y * mapW], &env->rowCDF[(size_t)y * (mapW + 1)], &env->rowIntegral[y]);
        total.add(env->rowIntegral[y]);
    }
    env->integral = total.result;
    env->topPDF.assign(mapH, 0.0f);
    env->topCDF.assign(mapH + 1, 0.0f);
    float topIntegral;
    build1D(env->rowIntegral, env->topPDF.data(), env->topCDF.data(), &topIntegral);
    env->rowAlias.resize((size_t)mapW * mapH);
    for (uint32_t y = 0; y < mapH; ++y)
        buildAlias(&env->rowCDF[(size_t)y * (mapW + 1)], mapW, &env->rowAlias[(size_t)y * mapW]);
    env->topAlias.resize(mapH);
    buildAlias(env->topCDF.data(), mapH, env->topAlias.data());
}

// ============================================================================
// SBVH: binned SAH (32 object bins on the widest centroid axis) with spatial
// splits (16 bins on the widest bounds axis) when the object split's child
// overlap exceeds 1e-5 of the root area; traversal cost 1.2, unit triangle
// cost, leaf when cheaper than both splits.  The same steps and float
// arithmetic as libSLR/Accelerator/SBVH.h:57-417, so the resulting tree (and
// the fingerprint printed at SBVH.h:415) is identical for the same input.
// ============================================================================
namespace {
struct Box {
    float mn[3], mx[3];
    Box() { mn[0] = mn[1] = mn[2] = INFINITY; mx[0] = mx[1] = mx[2] = -INFINITY; }
    static Box point(const float p[3]) { Box b; for (int k = 0; k < 3; ++k) { b.mn[k] = p[k]; b.mx[k] = p[k]; } return b; }
    void unify(const Box &o) { for (int k = 0; k < 3; ++k) { mn[k] = std::fmin(mn[k], o.mn[k]); mx[k] = std::fmax(mx[k], o.mx[k]); } }
    void unifyPoint(const float p[3]) { for (int k = 0; k < 3; ++k) { mn[k] = std::fmin(mn[k], p[k]); mx[k] = std::fmax(mx[k], p[k]); } }
    float sa() const {
        float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        return 2 * (dx * dy + dy * dz + dz * dx);
    }
    bool valid() const { return (mx[0] - mn[0]) >= 0 && (mx[1] - mn[1]) >= 0 && (mx[2] - mn[2]) >= 0; }
    int widestAxis() const {
        float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        if (dx > dy && dx > dz) return 0;
        if (dy > dz) return 1;
        return 2;
    }
    float center(int a) const { return (mn[a] + mx[a]) * 0.5f; }
    void centroid(float c[3]) const { for (int k = 0; k < 3; ++k) c[k] = (mn[k] + mx[k]) * 0.5f; }
};

Box intersect(const Box &a, const Box &b) {
    Box r;
    for (int k = 0; k < 3; ++k) { r.mn[k] = std::fmax(a.mn[k], b.mn[k]); r.mx[k] = std::fmin(a.mx[k], b.mx[k]); }
    return r;
}

struct Frag {
    uint32_t prim;
    Box box;
    float cost;
};

struct P3 { float v[3]; };

class SbvhBuilder {
public:
    SbvhBuilder(const float* tris, uint32_t n) : m_tris(tris), m_n(n) {}

    bool run(SbvhResult* out, std::string* err) {
        if (m_n == 0) {
            SbvhNode leaf{};
            for (int k = 0; k < 3; ++k) { leaf.bmin[k] = INFINITY; leaf.bmax[k] = -INFINITY; }
            leaf.offset = 0xffffffffu;
            leaf.count = 0;
            leaf.leaf = 1;
            out->nodes.assign(1, leaf);
            out->depth = 1;
            out->cost = 0;
            out->numFragments = 0;
            for (int k = 0; k < 3; ++k) { out->bmin[k] = INFINITY; out->bmax[k] = -INFINITY; }
            return true;
        }
        const uint32_t budget = 5 * m_n;
        m_frags.resize(budget);
        for (uint32_t i = 0; i < m_n; ++i) {
            m_frags[i].prim = i;
            m_frags[i].box = triBounds(i);
            m_frags[i].cost = 1.0f;
            m_bounds.unify(m_frags[i].box);
        }
        m_budget = budget;
        std::vector<Frag> all(m_frags.begin(), m_frags.begin() + m_n);
        std::vector<Frag>().swap(m_frags);
        SubTree tree;
        const int threads = (int)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        subtreeParallel(std::move(all), threads, &tree);
        if (tree.overflow || tree.leaves.size() > budget) {
            *err = "SBVH fragment budget (5x triangles) exceeded";
            return false;
        }
        out->nodes = std::move(tree.nodes);
        out->leafPrims = std::move(tree.leaves);
        out->depth = tree.depth;
        out->numFragments = (uint32_t)out->leafPrims.size();
        out->cost = sahCost(out->nodes);
        for (int k = 0; k < 3; ++k) { out->bmin[k] = m_bounds.mn[k]; out->bmax[k] = m_bounds.mx[k]; }
        return true;
    }

private:
    const float* vert(uint32_t tri, int k) const { return m_tris + 9 * (size_t)tri + 3 * k; }

    Box triBounds(uint32_t t) const {
        Box b = Box::point(vert(t, 0));
        b.unifyPoint(vert(t, 1));
        b.unifyPoint(vert(t, 2));
        return b;
    }

    void sortedVerts(uint32_t t, int axis, P3 p[3]) const {
        for (int k = 0; k < 3; ++k) std::memcpy(p[k].v, vert(t, k), 12);
        std::sort(p, p + 3, [axis](const P3 &a, const P3 &b) { return a.v[axis] < b.v[axis]; });
    }

    static void lerpPoint(const P3 &pa, const P3 &pb, float t, float out[3]) {
        const float omt = 1 - t;
        for (int k = 0; k < 3; ++k) out[k] = omt * pa.v[k] + t * pb.v[k];
    }

    // Bounds of the part of triangle t inside the slab [lo, hi) on axis
    // (TriangleSurfaceShape.cpp:44-96).
    Box choppedBounds(uint32_t t, int axis, float lo, float hi) const {
        P3 p[3];
        sortedVerts(t, axis, p);
        const float chop[2] = {lo, hi};
        float minPos = p[0].v[axis], maxPos = p[2].v[axis];
        Box base = triBounds(t);
        if (minPos >= hi || maxPos <= lo) return Box();
        if (minPos >= lo && maxPos <= hi) return base;
        float isect[4][3];
        uint32_t n = 0;
        for (int from = 0; from < 2; ++from)
            for (int to = from + 1; to < 3; ++to) {
                float dAB = p[to].v[axis] - p[from].v[axis];
                for (int c = 0; c < 2; ++c) {
                    float dAP = chop[c] - p[from].v[axis];
                    float dPB = chop[c] - p[to].v[axis];
                    float tt = dAP / dAB;
                    if (dAP > 0 && dPB <= 0 && n < 4) lerpPoint(p[from], p[to], tt, isect[n++]);
                }
            }
        Box r;
        if (p[1].v[axis] >= lo && p[1].v[axis] < hi) r.unifyPoint(p[1].v);
        for (uint32_t i = 0; i < n; ++i) r.unifyPoint(isect[i]);
        if (n == 2) r.unifyPoint(maxPos < hi ? p[2].v : p[0].v);
        return r;
    }

    // Bounds of the two parts of triangle t split at pos (TriangleSurfaceShape.cpp:98-153).
    void splitBounds(uint32_t t, int axis, float pos, Box* b0, Box* b1) const {
        P3 p[3];
        sortedVerts(t, axis, p);
        float minPos = p[0].v[axis], maxPos = p[2].v[axis];
        Box base = triBounds(t);
        if (pos <= minPos) { *b0 = Box(); *b1 = base; return; }
        if (pos >= maxPos) { *b0 = base; *b1 = Box(); return; }
        float isect[2][3];
        uint32_t n = 0;
        for (int from = 0; from < 2; ++from)
            for (int to = from + 1; to < 3; ++to) {
                float dAB = p[to].v[axis] - p[from].v[axis];
                float dAP = pos - p[from].v[axis];
                float dPB = pos - p[to].v[axis];
                float tt = dAP / dAB;
                if (dAP > 0 && dPB <= 0 && n < 2) lerpPoint(p[from], p[to], tt, isect[n++]);
            }
        *b0 = Box::point(p[0].v);
        *b1 = Box::point(p[2].v);
        if (p[1].v[axis] < pos) b0->unifyPoint(p[1].v);
        else b1->unifyPoint(p[1].v);
        for (uint32_t i = 0; i < n; ++i) { b0->unifyPoint(isect[i]); b1->unifyPoint(isect[i]); }
    }

    // ---- one node's decision (SBVH.h:57-250): leaf, object split or spatial
    // split, from the node's fragments alone.  The cost sums add fragment
    // costs of 1 (exact in float for any order) and the boxes are min/max
    // unions, so the decision does not depend on the fragments' order or on
    // how the binning is divided between threads.
    struct Decision {
        enum Kind { kLeaf, kObject, kSpatial } kind;
        Box parent;
        int axis;
        float pivot;                  // object split
        uint32_t splitSP;             // spatial split
        float pMin, pMax, binWidth;
    };

    struct Bins {
        static constexpr uint32_t kObjBins = 32, kSBins = 16;
        Box parent, parentCentroid;
        float leafCost = 0.0f;
        Box objBox[kObjBins];
        float objCost[kObjBins] = {};
        Box sBox[kSBins];
        float sEntryCost[kSBins] = {}, sExitCost[kSBins] = {};
        void merge(const Bins &o, bool obj, bool spatial) {
            parent.unify(o.parent);
            parentCentroid.unify(o.parentCentroid);
            leafCost += o.leafCost;
            if (obj)
                for (uint32_t i = 0; i < kObjBins; ++i) { objBox[i].unify(o.objBox[i]); objCost[i] += o.objCost[i]; }
            if (spatial)
                for (uint32_t i = 0; i < kSBins; ++i) {
                    sBox[i].unify(o.sBox[i]);
                    sEntryCost[i] += o.sEntryCost[i];
                    sExitCost[i] += o.sExitCost[i];
                }
        }
    };

    // Runs fn(lo, hi, partial) over [0, n) on up to `threads` threads and
    // merges the partial bins in chunk order.
    template <typename Fn>
    static void parallelBins(uint32_t n, int threads, Bins* out, bool obj, bool spatial, Fn fn) {
        const uint32_t kMinChunk = 16384;
        int t = (int)std::min<uint32_t>((uint32_t)std::max(1, threads), std::max(1u, n / kMinChunk));
        if (t <= 1) {
            fn(0u, n, out);
            return;
        }
        std::vector<Bins> part(t);
        std::vector<std::thread> pool;
        for (int k = 0; k < t; ++k) {
            uint32_t lo = (uint32_t)((uint64_t)n * k / t), hi = (uint32_t)((uint64_t)n * (k + 1) / t);
            pool.emplace_back([&, lo, hi, k]() { fn(lo, hi, &part[k]); });
        }
        for (std::thread &th : pool) th.join();
        for (int k = 0; k < t; ++k) out->merge(part[k], obj, spatial);
    }

    Decision decide(const Frag* f, uint32_t n, int threads) const {
        Decision d;
        Bins bins;
        parallelBins(n, threads, &bins, false, false, [&](uint32_t lo, uint32_t hi, Bins* b) {
            for (uint32_t i = lo; i < hi; ++i) {
                b->parent.unify(f[i].box);
                float c[3];
                f[i].box.centroid(c);
                b->parentCentroid.unifyPoint(c);
                b->leafCost += f[i].cost;
            }
        });
        const Box parent = bins.parent, parentCentroid = bins.parentCentroid;
        const float leafCost = bins.leafCost;
        d.parent = parent;
        d.kind = Decision::kLeaf;
        if (n == 1) return d;
        const int axisOP = parentCentroid.widestAxis();
        const int axisSP = parent.widestAxis();
        const float saParent = parent.sa();
        const float pcMin = parentCentroid.mn[axisOP], pcMax = parentCentroid.mx[axisOP];
        const float pMin = parent.mn[axisSP], pMax = parent.mx[axisSP];
        const float travCost = 1.2f;
        constexpr uint32_t kObjBins = Bins::kObjBins, kSBins = Bins::kSBins;

        // Object binning.
        uint32_t splitOP = 0;
        float minCostOP = INFINITY;
        if ((pcMax - pcMin) > 0) {
            parallelBins(n, threads, &bins, true, false, [&](uint32_t lo, uint32_t hi, Bins* b) {
                for (uint32_t i = lo; i < hi; ++i) {
                    uint32_t bin = (uint32_t)(kObjBins * ((f[i].box.center(axisOP) - pcMin) / (pcMax - pcMin)));
                    bin = std::min(bin, kObjBins - 1);
                    b->objCost[bin] += f[i].cost;
                    b->objBox[bin].unify(f[i].box);
                }
            });
            for (uint32_t i = 0; i < kObjBins - 1; ++i) {
                Box b0, b1;
                float c0 = 0.0f, c1 = 0.0f;
                for (uint32_t j = 0; j <= i; ++j) { b0.unify(bins.objBox[j]); c0 += bins.objCost[j]; }
                for (uint32_t j = i + 1; j < kObjBins; ++j) { b1.unify(bins.objBox[j]); c1 += bins.objCost[j]; }
                float cost = travCost + (b0.sa() * c0 + b1.sa() * c1) / saParent;
                if (cost < minCostOP) { minCostOP = cost; splitOP = i; }
            }
        }
        Box leftOP, rightOP;
        for (uint32_t j = 0; j <= splitOP; ++j) leftOP.unify(bins.objBox[j]);
        for (uint32_t j = splitOP + 1; j < kObjBins; ++j) rightOP.unify(bins.objBox[j]);
        Box overlap = intersect(leftOP, rightOP);
        float overlapSA = 0;
        if (overlap.valid()) overlapSA = overlap.sa();

        // Spatial binning.
        const float binWidth = (parent.mx[axisSP] - parent.mn[axisSP]) / kSBins;
        uint32_t splitSP = 0;
        float minCostSP = INFINITY;
        const float alpha = 1e-5f;
        if (overlapSA / m_bounds.sa() > alpha) {
            parallelBins(n, threads, &bins, false, true, [&](uint32_t lo, uint32_t hi, Bins* b) {
                for (uint32_t i = lo; i < hi; ++i) {
                    uint32_t entry = binIndex(f[i].box.mn[axisSP], pMin, pMax);
                    uint32_t exit = binIndex(f[i].box.mx[axisSP], pMin, pMax);
                    b->sEntryCost[entry] += f[i].cost;
                    b->sExitCost[exit] += f[i].cost;
                    for (uint32_t k = entry; k <= exit; ++k) {
                        float blo = k * binWidth + pMin;
                        Box chopped = choppedBounds(f[i].prim, axisSP, blo, blo + binWidth);
                        b->sBox[k].unify(intersect(chopped, f[i].box));
                    }
                }
            });
            for (uint32_t i = 0; i < kSBins - 1; ++i) {
                Box b0, b1;
                float c0 = 0.0f, c1 = 0.0f;
                for (uint32_t j = 0; j <= i; ++j) { b0.unify(bins.sBox[j]); c0 += bins.sEntryCost[j]; }
                for (uint32_t j = i + 1; j < kSBins; ++j) { b1.unify(bins.sBox[j]); c1 += bins.sExitCost[j]; }
                float cost = travCost + (b0.sa() * c0 + b1.sa() * c1) / saParent;
                if (cost < minCostSP) { minCostSP = cost; splitSP = i; }
            }
        }
        if (leafCost < minCostOP && leafCost < minCostSP) return d;
        if (minCostOP < minCostSP) {
            d.kind = Decision::kObject;
            d.axis = axisOP;
            d.pivot = pcMin + (pcMax - pcMin) / kObjBins * (splitOP + 1);
            return d;
        }
        d.kind = Decision::kSpatial;
        d.axis = axisSP;
        d.splitSP = splitSP;
        d.pMin = pMin;
        d.pMax = pMax;
        d.binWidth = binWidth;
        return d;
    }

    // Object split: partitions [first, last) in place (std::partition, as
    // SBVH.h:252-257) and returns the split offset (at least 1).
    static uint32_t objectPartition(Frag* first, Frag* last, const Decision &d) {
        const int axis = d.axis;
        const float pivot = d.pivot;
        Frag* mid = std::partition(first, last, [axis, pivot](const Frag &f) { return f.box.center(axis) < pivot; });
        return std::max((uint32_t)(mid - first), 1u);
    }

    // Spatial split (SBVH.h:276-330): fragments straddling the plane become
    // two, clipped to each side.
    void spatialSplit(const Frag* f, uint32_t n, const Decision &d, std::vector<Frag>* left,
                      std::vector<Frag>* right) const {
        left->reserve(n);
        right->reserve(n);
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t entry = binIndex(f[i].box.mn[d.axis], d.pMin, d.pMax);
            uint32_t exit = binIndex(f[i].box.mx[d.axis], d.pMin, d.pMax);
            if (exit <= d.splitSP) {
                left->push_back(f[i]);
            } else if (entry > d.splitSP) {
                right->push_back(f[i]);
            } else {
                float splitPos = (d.splitSP + 1) * d.binWidth + d.pMin;
                Box sl, sr;
                splitBounds(f[i].prim, d.axis, splitPos, &sl, &sr);
                if (sl.valid()) left->push_back(Frag{f[i].prim, intersect(sl, f[i].box), f[i].cost});
                if (sr.valid()) right->push_back(Frag{f[i].prim, intersect(sr, f[i].box), f[i].cost});
            }
        }
    }

    // ---- in-place build of one (small) subtree, as SBVH.h:57-349: nodes in
    // pre-order, leaf references in the same order.
    uint32_t build(uint32_t currentSize, uint32_t start, uint32_t end, uint32_t depth, uint32_t* numAdded) {
        *numAdded = 0;
        const uint32_t nodeIdx = (uint32_t)m_nodes.size();
        m_nodes.emplace_back();
        if (++depth > m_depth) m_depth = depth;
        const uint32_t numObjs = end - start;
        const Decision d = decide(m_frags.data() + start, numObjs, 1);
        if (d.kind == Decision::kLeaf) {
            makeLeaf(nodeIdx, d.parent, start, end);
            return nodeIdx;
        }
        if (d.kind == Decision::kObject) {
            uint32_t splitIdx = objectPartition(m_frags.data() + start, m_frags.data() + end, d) + start;
            uint32_t addL, addR;
            uint32_t c0 = build(currentSize, start, splitIdx, depth, &addL);
            uint32_t c1 = build(currentSize + addL, splitIdx + addL, end + addL, depth, &addR);
            makeInternal(nodeIdx, d.parent, c0, c1, d.axis);
            *numAdded += addL + addR;
            return nodeIdx;
        }
        std::vector<Frag> left, right;
        spatialSplit(m_frags.data() + start, numObjs, d, &left, &right);
        const uint32_t numLeft = (uint32_t)left.size(), numRight = (uint32_t)right.size();
        *numAdded = (numLeft + numRight) - numObjs;
        if (currentSize + *numAdded > (uint32_t)m_frags.size()) {
            m_overflow = true;
            makeLeaf(nodeIdx, d.parent, start, end);
            *numAdded = 0;
            return nodeIdx;
        }
        std::copy_backward(m_frags.begin() + end, m_frags.begin() + currentSize,
                           m_frags.begin() + currentSize + *numAdded);
        std::copy(left.begin(), left.end(), m_frags.begin() + start);
        std::copy(right.begin(), right.end(), m_frags.begin() + start + numLeft);
        uint32_t splitIdx = start + numLeft;
        uint32_t addL, addR;
        uint32_t c0 = build(currentSize + *numAdded, start, splitIdx, depth, &addL);
        uint32_t c1 = build(currentSize + *numAdded + addL, splitIdx + addL, end + *numAdded + addL, depth, &addR);
        makeInternal(nodeIdx, d.parent, c0, c1, d.axis);
        *numAdded += addL + addR;
        return nodeIdx;
    }

    // ---- parallel build of the top of the tree.  A node's subtree depends
    // only on its own fragments (in order), so the two children build
    // concurrently into separate arrays, concatenated afterwards in the
    // sequential pre-order; the result equals the sequential build's.
    struct SubTree {
        std::vector<SbvhNode> nodes;     // pre-order, child / leaf indices local
        std::vector<uint32_t> leaves;
        uint32_t depth = 0;
        bool overflow = false;
    };

    void subtreeSequential(std::vector<Frag> &&frags, SubTree* out) const {
        // Fragment headroom grows until the subtree fits (the reference's
        // decisions never depend on it).
        for (size_t room = frags.size() * 5 + 64;; room *= 2) {
            SbvhBuilder local(m_tris, 0);
            local.m_bounds = m_bounds;
            local.m_frags = frags;
            local.m_frags.resize(room);
            local.m_depth = 0;
            local.m_overflow = false;
            uint32_t added = 0;
            local.build((uint32_t)frags.size(), 0, (uint32_t)frags.size(), 0, &added);
            if (local.m_overflow && room < ((size_t)1 << 31)) continue;
            out->nodes = std::move(local.m_nodes);
            out->leaves = std::move(local.m_leaves);
            out->depth = local.m_depth;
            out->overflow = local.m_overflow;
            return;
        }
    }

    static void append(SubTree* dst, const SubTree &src) {
        const uint32_t nodeBase = (uint32_t)dst->nodes.size(), leafBase = (uint32_t)dst->leaves.size();
        for (SbvhNode n : src.nodes) {
            if (n.leaf) {
                if (n.offset != 0xffffffffu) n.offset += leafBase;
            } else {
                n.c0 += nodeBase;
                n.c1 += nodeBase;
            }
            dst->nodes.push_back(n);
        }
        dst->leaves.insert(dst->leaves.end(), src.leaves.begin(), src.leaves.end());
    }

    void subtreeParallel(std::vector<Frag> &&frags, int threads, SubTree* out) const {
        const uint32_t kSequentialBelow = 1u << 14;
        const uint32_t n = (uint32_t)frags.size();
        if (n <= kSequentialBelow || threads <= 1) {
            subtreeSequential(std::move(frags), out);
            return;
        }
        const Decision d = decide(frags.data(), n, threads);
        if (d.kind == Decision::kLeaf) {
            subtreeSequential(std::move(frags), out);
            return;
        }
        std::vector<Frag> left, right;
        if (d.kind == Decision::kObject) {
            uint32_t split = objectPartition(frags.data(), frags.data() + n, d);
            left.assign(frags.begin(), frags.begin() + split);
            right.assign(frags.begin() + split, frags.end());
        } else {
            spatialSplit(frags.data(), n, d, &left, &right);
        }
        std::vector<Frag>().swap(frags);
        SubTree l, r;
        const int tl = threads / 2, tr = threads - tl;
        std::thread th([&]() { subtreeParallel(std::move(left), std::max(1, tl), &l); });
        subtreeParallel(std::move(right), std::max(1, tr), &r);
        th.join();
        SbvhNode node{};
        for (int k = 0; k < 3; ++k) { node.bmin[k] = d.parent.mn[k]; node.bmax[k] = d.parent.mx[k]; }
        node.axis = (uint32_t)d.axis;
        node.leaf = 0;
        out->nodes.clear();
        out->nodes.push_back(node);
        out->nodes[0].c0 = 1;
        out->nodes[0].c1 = 1 + (uint32_t)l.nodes.size();
        append(out, l);
        append(out, r);
        out->depth = 1 + std::max(l.depth, r.depth);
        out->overflow = l.overflow || r.overflow;
    }

    static uint32_t binIndex(float x, float lo, float hi) {
        const uint32_t kSBins = 16;
        float f = kSBins * ((x - lo) / (hi - lo));
        uint32_t b = (f >= 0.0f && f < 4294967040.0f) ? (uint32_t)f : 0u;
        return std::min(b, kSBins - 1);
    }

    void makeLeaf(uint32_t nodeIdx, const Box &b, uint32_t start, uint32_t end) {
        SbvhNode &n = m_nodes[nodeIdx];
        for (int k = 0; k < 3; ++k) { n.bmin[k] = b.mn[k]; n.bmax[k] = b.mx[k]; }
        n.c0 = n.c1 = 0;
        n.offset = (uint32_t)m_leaves.size();
        n.count = end - start;
        n.axis = 0;
        n.leaf = 1;
        for (uint32_t i = start; i < end; ++i) m_leaves.push_back(m_frags[i].prim);
    }

    void makeInternal(uint32_t nodeIdx, const Box &b, uint32_t c0, uint32_t c1, int axis) {
        SbvhNode &n = m_nodes[nodeIdx];
        for (int k = 0; k < 3; ++k) { n.bmin[k] = b.mn[k]; n.bmax[k] = b.mx[k]; }
        n.c0 = c0;
        n.c1 = c1;
        n.offset = 0;
        n.count = 0;
        n.axis = (uint32_t)axis;
        n.leaf = 0;
    }

    static float boxSA(const SbvhNode &n) {
        float dx = n.bmax[0] - n.bmin[0], dy = n.bmax[1] - n.bmin[1], dz = n.bmax[2] - n.bmin[2];
        return 2 * (dx * dy + dy * dz + dz * dx);
    }

    // SBVH.h:319-347.
    static float sahCost(const std::vector<SbvhNode> &nodes) {
        const float Ci = 1.2f, Cl = 0.0f;
        float costInt = 0.0f, costLeaf = 0.0f, costObj = 0.0f;
        for (const SbvhNode &n : nodes) {
            float sa = boxSA(n);
            if (!n.leaf || n.count == 0) {
                costInt += sa;
            } else {
                costLeaf += sa;
                float prims = 0.0f;
                for (uint32_t j = 0; j < n.count; ++j) prims += 1.0f;
                costObj += sa * prims;
            }
        }
        float rootSA = boxSA(nodes[0]);
        costInt *= Ci / rootSA;
        costLeaf *= Cl / rootSA;
        costObj /= rootSA;
        return costInt + costLeaf + costObj;
    }

    const float* m_tris;
    uint32_t m_n;
    uint32_t m_budget = 0;
    bool m_overflow = false;
    std::vector<Frag> m_frags;
    std::vector<SbvhNode> m_nodes;
    std::vector<uint32_t> m_leaves;
    uint32_t m_depth = 0;
    Box m_bounds;
};
}  // namespace

bool buildSbvh(const float* triPositions, uint32_t numTris, SbvhResult* out, std::string* err) {
    SbvhBuilder b(triPositions, numTris);
    return b.run(out, err);
}

// ============================================================================
// Wide BVH: each wide node takes a binary node's children and repeatedly
// opens its largest-area internal child until it has kBvhWidth children.
// Boxes stay the SBVH's own boxes, so traversal tests the same slabs.
// ============================================================================
namespace {
struct WideBuilder {
    const SbvhResult &b;
    const float* tris;
    WideBvh* out;

    static float sa(const SbvhNode &n) {
        float dx = n.bmax[0] - n.bmin[0], dy = n.bmax[1] - n.bmin[1], dz = n.bmax[2] - n.bmin[2];
        return dx * dy + dy * dz + dz * dx;
    }

    uint32_t emitLeaf(uint32_t offset, uint32_t count) {
        uint32_t first = (uint32_t)out->frags.size();
        for (uint32_t i = 0; i < count; ++i) {
            uint32_t prim = b.leafPrims[offset + i];
            const float* p = tris + 9 * (size_t)prim;
            TriFrag f;
            f.v0x = p[0]; f.v0y = p[1]; f.v0z = p[2];
            f.prim = prim;
            f.e1x = p[3] - p[0]; f.e1y = p[4] - p[1]; f.e1z = p[5] - p[2]; f.pad0 = 0;
            f.e2x = p[6] - p[0]; f.e2y = p[7] - p[1]; f.e2z = p[8] - p[2]; f.pad1 = 0;
            out->frags.push_back(f);
        }
        return kLeafBit | ((count - 1) << kLeafCountShift) | first;
    }

    void setBox(BvhNode &n, int slot, const SbvhNode &s) {
        n.lox[slot] = s.bmin[0]; n.hix[slot] = s.bmax[0];
        n.loy[slot] = s.bmin[1]; n.hiy[slot] = s.bmax[1];
        n.loz[slot] = s.bmin[2]; n.hiz[slot] = s.bmax[2];
    }

    // Returns the child word for binary node `bi` referenced from a wide node.
    uint32_t child(uint32_t bi) {
        const SbvhNode &s = b.nodes[bi];
        if (s.leaf) {
            if (s.count == 0)
                return kChildEmpty;
            if (s.count <= (uint32_t)kMaxLeafCount)
                return emitLeaf(s.offset, s.count);
            // Oversized leaf: a wide node whose children are chunks of it,
            // all with the leaf's box.
            uint32_t idx = (uint32_t)out->nodes.size();
            out->nodes.emplace_back();
            uint32_t remaining = s.count, off = s.offset;
            BvhNode tmp;
            initNode(tmp);
            int slot = 0;
            while (remaining > 0 && slot < kBvhWidth) {
                uint32_t c = (slot == kBvhWidth - 1) ? remaining : std::min(remaining, (uint32_t)kMaxLeafCount);
                if (c > (uint32_t)kMaxLeafCount) {
                    // Recurse through a synthetic leaf node for the rest.
                    SbvhNode rest = s;
                    rest.offset = off;
                    rest.count = c;
                    tmp.child[slot] = childOfSynthetic(rest);
                } else {
                    tmp.child[slot] = emitLeaf(off, c);
                }
                setBox(tmp, slot, s);
                off += c;
                remaining -= c;
                ++slot;
            }
            out->nodes[idx] = tmp;
            return idx;
        }
        return buildWide(bi);
    }

    uint32_t childOfSynthetic(const SbvhNode &s) {
        std::vector<SbvhNode> &nodes = const_cast<std::vector<SbvhNode> &>(b.nodes);
        nodes.push_back(s);
        return child((uint32_t)nodes.size() - 1);
    }

    static void initNode(BvhNode &n) {
        for (int k = 0; k < kBvhWidth; ++k) {
            n.lox[k] = n.loy[k] = n.loz[k] = INFINITY;
            n.hix[k] = n.hiy[k] = n.hiz[k] = -INFINITY;
            n.child[k] = kChildEmpty;
            n.pad[k] = 0;
        }
    }

    uint32_t buildWide(uint32_t bi) {
        uint32_t idx = (uint32_t)out->nodes.size();
        out->nodes.emplace_back();
        std::vector<uint32_t> kids = {b.nodes[bi].c0, b.nodes[bi].c1};
        while ((int)kids.size() < kBvhWidth) {
            int best = -1;
            float bestSA = -1.0f;
            for (size_t k = 0; k < kids.size(); ++k) {
                const SbvhNode &n = b.nodes[kids[k]];
                if (!n.leaf && sa(n) > bestSA) { bestSA = sa(n); best = (int)k; }
            }
            if (best < 0) break;
            uint32_t open = kids[best];
            kids[best] = b.nodes[open].c0;
            kids.insert(kids.begin() + best + 1, b.nodes[open].c1);
        }
        BvhNode node;
        initNode(node);
        int slot = 0;
        for (size_t k = 0; k < kids.size(); ++k) {
            uint32_t w = child(kids[k]);
            if (w == kChildEmpty) continue;
            setBox(node, slot, b.nodes[kids[k]]);
            node.child[slot++] = w;
        }
        out->nodes[idx] = node;
        return idx;
    }
};
}  // namespace

void collapseToWide(const SbvhResult &b, const float* triPositions, WideBvh* out) {
    out->nodes.clear();
    out->frags.clear();
    SbvhResult copy = b;   // oversized-leaf handling may append synthetic nodes
    WideBuilder wb{copy, triPositions, out};
    const SbvhNode &root = copy.nodes[0];
    if (root.leaf) {
        // Root is a leaf (or the scene is empty): one wide node with it.
        out->nodes.emplace_back();
        BvhNode node;
        WideBuilder::initNode(node);
        if (root.count > 0) {
            wb.setBox(node, 0, root);
            node.child[0] = wb.child(0);
        }
        out->nodes[0] = node;
        return;
    }
    wb.buildWide(0);
}

// ============================================================================
// Density-grid medium: trilinear density and the super-voxel majorant grid
// (max(n / 16, 4) corners per axis plus, per cell, the largest amount by which
// the trilinear density exceeds the trilinear corner interpolation), the
// steps of DensityGridMediumDistribution::setupSuperVoxels
// (MediumDistribution/DensityGridMediumDistribution.cpp:16-204).
// ============================================================================
namespace {
inline float trilinear(const float* grid, uint32_t nx, uint32_t ny, uint32_t nz, const float p[3]) {
    uint32_t lx = std::min((uint32_t)(p[0] * (nx - 1)), nx - 1), ux = std::min(lx + 1, nx - 1);
    uint32_t ly = std::min((uint32_t)(p[1] * (ny - 1)), ny - 1), uy = std::min(ly + 1, ny - 1);
    uint32_t lz = std::min((uint32_t)(p[2] * (nz - 1)), nz - 1), uz = std::min(lz + 1, nz - 1);
    float wux = p[0] * (nx - 1) - lx, wlx = 1 - wux;
    float wuy = p[1] * (ny - 1) - ly, wly = 1 - wuy;
    float wuz = p[2] * (nz - 1) - lz, wlz = 1 - wuz;
    const size_t sl = (size_t)nx * ny;
    const float* zl = grid + sl * lz;
    const float* zu = grid + sl * uz;
    return zl[nx * ly + lx] * wlz * wly * wlx + zl[nx * ly + ux] * wlz * wly * wux +
           zl[nx * uy + lx] * wlz * wuy * wlx + zl[nx * uy + ux] * wlz * wuy * wux +
           zu[nx * ly + lx] * wuz * wly * wlx + zu[nx * ly + ux] * wuz * wly * wux +
           zu[nx * uy + lx] * wuz * wuy * wlx + zu[nx * uy + ux] * wuz * wuy * wux;
}

inline bool outsideUnit(const float p[3]) {
    return p[0] < 0 || p[1] < 0 || p[2] < 0 || p[0] > 1 || p[1] > 1 || p[2] > 1;
}
}  // namespace

float densityAt(const HostMedium &m, const float param[3]) {
    if (outsideUnit(param)) return 0.0f;
    return trilinear(m.density.data(), m.nx, m.ny, m.nz, param);
}

void buildSuperVoxels(const HostMedium &m, HostSuperVoxels* sv) {
    const uint32_t svx = std::max(m.nx / 16, 4u), svy = std::max(m.ny / 16, 4u), svz = std::max(m.nz / 16, 4u);
    sv->svx = svx; sv->svy = svy; sv->svz = svz;
    const uint32_t sv1[3] = {svx - 1, svy - 1, svz - 1};
    for (int k = 0; k < 3; ++k) sv->width[k] = (m.bmax[k] - m.bmin[k]) / (float)sv1[k];
    sv->corners.assign((size_t)svx * svy * svz, 0.0f);
    const size_t ncell = (size_t)(svx - 1) * (svy - 1) * (svz - 1);
    sv->maxDiff.assign(ncell, 0.0f);
    for (uint32_t z = 0; z < svz; ++z)
        for (uint32_t y = 0; y < svy; ++y)
            for (uint32_t x = 0; x < svx; ++x) {
                float p[3] = {(float)x / (svx - 1), (float)y / (svy - 1), (float)z / (svz - 1)};
                sv->corners[(size_t)z * svy * svx + y * svx + x] = densityAt(m, p);
            }
    // Coarse (corner-interpolated) density; the maximum differences are still
    // zero while they are being computed.
    auto coarse = [&](const float p[3]) -> float {
        if (outsideUnit(p)) return 0.0f;
        return trilinear(sv->corners.data(), svx, svy, svz, p);
    };
    const uint32_t nx = m.nx, ny = m.ny, nz = m.nz;
    std::vector<float> diffs(ncell, 0.0f);
    for (uint32_t cz = 0; cz < svz - 1; ++cz) {
        float lpz = (float)cz / (svz - 1), upz = (float)(cz + 1) / (svz - 1);
        uint32_t liz = (uint32_t)std::floor(lpz * (nz - 1)), uiz = (uint32_t)std::ceil(upz * (nz - 1));
        for (uint32_t cy = 0; cy < svy - 1; ++cy) {
            float lpy = (float)cy / (svy - 1), upy = (float)(cy + 1) / (svy - 1);
            uint32_t liy = (uint32_t)std::floor(lpy * (ny - 1)), uiy = (uint32_t)std::ceil(upy * (ny - 1));
            for (uint32_t cx = 0; cx < svx - 1; ++cx) {
                float lpx = (float)cx / (svx - 1), upx = (float)(cx + 1) / (svx - 1);
                uint32_t lix = (uint32_t)std::floor(lpx * (nx - 1)), uix = (uint32_t)std::ceil(upx * (nx - 1));
                float maxDiff = 0;
                for (uint32_t iz = liz; iz <= uiz; ++iz) {
                    float pz = (float)iz / (nz - 1);
                    for (uint32_t iy = liy; iy <= uiy; ++iy) {
                        float py = (float)iy / (ny - 1);
                        for (uint32_t ix = lix; ix <= uix; ++ix) {
                            float px = (float)ix / (nx - 1);
                            if (iz > liz && iz < uiz && iy > liy && iy < uiy && ix > lix && ix < uix) {
                                float p[3] = {px, py, pz};
                                float actual = m.density[(size_t)iz * nx * ny + (size_t)nx * iy + ix];
                                maxDiff = std::max(maxDiff, actual - coarse(p));
                            } else {
                                // Interpolated samples may exceed the coarse value at cell faces.
                                int nzI = (iz > liz && iz < uiz) ? 1 : 2;
                                int nyI = (iy > liy && iy < uiy) ? 1 : 2;
                                int nxI = (ix > lix && ix < uix) ? 1 : 2;
                                int zb = (int)iz, yb = (int)iy, xb = (int)ix;
                                if (nzI == 2) zb = iz == liz ? (int)liz : (int)uiz - 1;
                                if (nyI == 2) yb = iy == liy ? (int)liy : (int)uiy - 1;
                                if (nxI == 2) xb = ix == lix ? (int)lix : (int)uix - 1;
                                for (int dz = 0; dz < nzI; ++dz) {
                                    float ppz = std::min(std::max((float)(zb + dz) / (nz - 1), lpz), upz);
                                    for (int dy = 0; dy < nyI; ++dy) {
                                        float ppy = std::min(std::max((float)(yb + dy) / (ny - 1), lpy), upy);
                                        for (int dx = 0; dx < nxI; ++dx) {
                                            float ppx = std::min(std::max((float)(xb + dx) / (nx - 1), lpx), upx);
                                            float p[3] = {ppx, ppy, ppz};
                                            maxDiff = std::max(maxDiff, densityAt(m, p) - coarse(p));
                                        }
                                    }
                                }
                            }
                        }
                    }
                }
                diffs[(size_t)(svx - 1) * (svy - 1) * cz + (size_t)(svx - 1) * cy + cx] = maxDiff;
            }
        }
    }
    sv->maxDiff = diffs;
}

// ============================================================================
// Scene build
// ============================================================================
namespace {
void mat4MulPoint(const float m[16], const float p[3], float out[3]) {
    for (int r = 0; r < 3; ++r)
        out[r] = m[4 * r + 0] * p[0] + m[4 * r + 1] * p[1] + m[4 * r + 2] * p[2] + m[4 * r + 3];
}
void mat4MulVec(const float m[16], const float v[3], float out[3]) {
    for (int r = 0; r < 3; ++r)
        out[r] = m[4 * r + 0] * v[0] + m[4 * r + 1] * v[1] + m[4 * r + 2] * v[2];
}
bool invert4(const float m[16], double inv[16]) {
    double a[16];
    for (int i = 0; i < 16; ++i) a[i] = m[i];
    double r[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int i = c + 1; i < 4; ++i)
            if (std::fabs(a[4 * i + c]) > std::fabs(a[4 * piv + c])) piv = i;
        if (a[4 * piv + c] == 0) return false;
        for (int k = 0; k < 4; ++k) { std::swap(a[4 * c + k], a[4 * piv + k]); std::swap(r[4 * c + k], r[4 * piv + k]); }
        double d = a[4 * c + c];
        for (int k = 0; k < 4; ++k) { a[4 * c + k] /= d; r[4 * c + k] /= d; }
        for (int i = 0; i < 4; ++i) {
            if (i == c) continue;
            double f = a[4 * i + c];
            for (int k = 0; k < 4; ++k) { a[4 * i + k] -= f * a[4 * c + k]; r[4 * i + k] -= f * r[4 * c + k]; }
        }
    }
    for (int i = 0; i < 16; ++i) inv[i] = r[i];
    return true;
}
void normalize3(float v[3]) {
    float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    float r = 1.0f / l;
    v[0] *= r; v[1] *= r; v[2] *= r;
}
}  // namespace

bool buildScene(const HostScene &s, BuiltScene* out, std::string* err) {
    auto t0 = std::chrono::steady_clock::now();
    // Triangles in insertion order (mesh order, then triangle order), as the
    // reference's Scene::build orders its surface objects.
    uint32_t nt = 0, nv = 0;
    for (const HostMesh &m : s.meshes) { nt += (uint32_t)(m.idx.size() / 3); nv += (uint32_t)(m.pos.size() / 3); }
    std::vector<float> tris((size_t)nt * 9);
    out->prims.resize(nt);
    out->vpos.resize(nv);
    out->vnrm.resize(nv);
    out->vtan.resize(nv);
    uint32_t tBase = 0, vBase = 0;
    for (const HostMesh &m : s.meshes) {
        uint32_t mv = (uint32_t)(m.pos.size() / 3), mt = (uint32_t)(m.idx.size() / 3);
        for (uint32_t i = 0; i < mv; ++i) {
            out->vpos[vBase + i] = f4(m.pos[3 * i], m.pos[3 * i + 1], m.pos[3 * i + 2], m.uv[2 * i]);
            out->vnrm[vBase + i] = f4(m.nrm[3 * i], m.nrm[3 * i + 1], m.nrm[3 * i + 2], m.uv[2 * i + 1]);
            out->vtan[vBase + i] = f4(m.tan[3 * i], m.tan[3 * i + 1], m.tan[3 * i + 2], 0.0f);
        }
        for (uint32_t t = 0; t < mt; ++t) {
            uint32_t i0 = m.idx[3 * t], i1 = m.idx[3 * t + 1], i2 = m.idx[3 * t + 2];
            const float* p0 = &m.pos[3 * i0];
            const float* p1 = &m.pos[3 * i1];
            const float* p2 = &m.pos[3 * i2];
            float* dst = &tris[9 * (size_t)(tBase + t)];
            std::memcpy(dst, p0, 12);
            std::memcpy(dst + 3, p1, 12);
            std::memcpy(dst + 6, p2, 12);
            float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
            float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            float area = 0.5f * len;
            normalize3(n);
            DevPrim &pr = out->prims[tBase + t];
            pr.v0 = vBase + i0; pr.v1 = vBase + i1; pr.v2 = vBase + i2;
            pr.material = (uint32_t)m.material;
            pr.ngx = n[0]; pr.ngy = n[1]; pr.ngz = n[2];
            pr.invArea = 1.0f / area;
        }
        tBase += mt;
        vBase += mv;
    }
    if (!buildSbvh(tris.data(), nt, &out->sbvh, err)) return false;
    collapseToWide(out->sbvh, tris.data(), &out->wide);

    // Surface lights: emitting triangles in object order, importance 1 each
    // (surface_object.cpp:57-59, 379-391).
    out->lightPrims.clear();
    for (uint32_t i = 0; i < nt; ++i)
        if (s.materials[out->prims[i].material].emit >= 0) out->lightPrims.push_back(i);
    const uint32_t nl = (uint32_t)out->lightPrims.size();
    out->lightPMF.assign(nl, 1.0f);
    out->lightCDF.assign(nl + 1, 0.0f);
    {
        Kahan sum;
        for (uint32_t i = 0; i < nl; ++i) { sum.add(out->lightPMF[i]); out->lightCDF[i + 1] = sum.result; }
        for (uint32_t i = 0; i < nl; ++i) { out->lightPMF[i] /= sum.result; out->lightCDF[i + 1] /= sum.result; }
        out->lightAlias.resize(nl);
        buildAlias(out->lightCDF.data(), nl, out->lightAlias.data());
    }

    if (s.envPresent) buildEnvironment(s.envRGBA.data(), s.envW, s.envH, s.envScale, &out->env);
    if (s.medium.present) buildSuperVoxels(s.medium, &out->superVoxels);

    // World bounds: surfaces and media (Scene.cpp:30-36).
    Box world;
    if (nt > 0) {
        for (int k = 0; k < 3; ++k) { world.mn[k] = out->sbvh.bmin[k]; world.mx[k] = out->sbvh.bmax[k]; }
    }
    if (s.medium.present) {
        Box mb;
        for (int k = 0; k < 3; ++k) { mb.mn[k] = s.medium.bmin[k]; mb.mx[k] = s.medium.bmax[k]; }
        world.unify(mb);
    }
    if (world.valid()) {
        world.centroid(out->worldCenter);
        float d[3] = {world.mx[0] - out->worldCenter[0], world.mx[1] - out->worldCenter[1], world.mx[2] - out->worldCenter[2]};
        out->worldRadius = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    } else {
        out->worldCenter[0] = out->worldCenter[1] = out->worldCenter[2] = 0.0f;
        out->worldRadius = 0.0f;
    }
    out->worldDiscArea = (float)(kPi * out->worldRadius * out->worldRadius);

    // Camera (PerspectiveCamera.cpp:17-62, EquirectangularCamera.cpp:25-51).
    DevCamera &c = out->camera;
    std::memset(&c, 0, sizeof(c));
    if (s.cameraPresent) {
        c.kind = s.cameraKind;
        c.sensitivity = s.camSensitivity;
        const float* M = s.camMatrix;
        float zero[3] = {0, 0, 0};
        mat4MulPoint(M, zero, c.org);
        double inv[16];
        if (!invert4(M, inv)) { *err = "camera transform is singular"; return false; }
        // Normal (0, 0, 1) through the inverse transpose: the third row of the inverse.
        float nz[3] = {(float)inv[8], (float)inv[9], (float)inv[10]};
        normalize3(nz);
        float ex[3], xv[3] = {1, 0, 0};
        mat4MulVec(M, xv, ex);
        normalize3(ex);
        std::memcpy(c.ez, nz, 12);
        std::memcpy(c.ex, ex, 12);
        c.ey[0] = nz[1] * ex[2] - nz[2] * ex[1];
        c.ey[1] = nz[2] * ex[0] - nz[0] * ex[2];
        c.ey[2] = nz[0] * ex[1] - nz[1] * ex[0];
        c.lensRadius = s.camLensRadius;
        c.objPlaneDist = s.camObjDist;
        c.imgPlaneDist = s.camImgDist;
        c.opHeight = 2.0f * s.camObjDist * std::tan(s.camFovY * 0.5f);
        c.opWidth = c.opHeight * s.camAspect;
        c.imgPlaneArea = (float)(c.opWidth * c.opHeight * std::pow(s.camImgDist / s.camObjDist, 2));
        c.phiAngle = s.camPhiAngle;
        c.thetaAngle = s.camThetaAngle;
    }
    out->buildSeconds = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
    return true;
}

// ---------------------------------------------------------------------------
// Film colour: the CIE 1931 2-degree colour matching functions integrated
// over the 16 film bins (DiscretizedSpectrumTemplate::initialize,
// BasicTypes/spectrum_types.cpp:945-995), in float and in the same order, so
// the bins equal the reference's bit for bit.
// ---------------------------------------------------------------------------
#include "cmf_table.inc"

void discretizedCmf(float xbar[16], float ybar[16], float zbar[16], float* integral) {
    const int numSamples = 471, numBins = 16;
    auto val = [](const unsigned int* bits, int i) {
        float f;
        std::memcpy(&f, &bits[i], sizeof(f));
        return f;
    };
    uint32_t sBin = 0;
    float nextP = float(sBin + 1) / numBins;
    float xSum = 0, xPrev = val(kCmfXBits, 0);
    float ySum = 0, yPrev = val(kCmfYBits, 0);
    float zSum = 0, zPrev = val(kCmfZBits, 0);
    const float interval = 1;
    for (int i = 1; i < numSamples; ++i) {
        float curP = float(i) / (numSamples - 1);
        float width = interval;
        float xCur = val(kCmfXBits, i), yCur = val(kCmfYBits, i), zCur = val(kCmfZBits, i);
        if (curP >= nextP) {
            width = (curP - nextP) * (830.0f - 360.0f);
            float t = 1 - width / interval;
            float xIn = xPrev * (1 - t) + xCur * t;
            float yIn = yPrev * (1 - t) + yCur * t;
            float zIn = zPrev * (1 - t) + zCur * t;
            xSum += (xPrev + xIn) * (interval - width) * 0.5f;
            ySum += (yPrev + yIn) * (interval - width) * 0.5f;
            zSum += (zPrev + zIn) * (interval - width) * 0.5f;
            if (sBin < (uint32_t)numBins) {
                xbar[sBin] = xSum;
                ybar[sBin] = ySum;
                zbar[sBin] = zSum;
            }
            xSum = ySum = zSum = 0;
            xPrev = xIn;
            yPrev = yIn;
            zPrev = zIn;
            ++sBin;
            nextP = float(sBin + 1) / numBins;
        }
        xSum += (xPrev + xCur) * width * 0.5f;
        ySum += (yPrev + yCur) * width * 0.5f;
        zSum += (zPrev + zCur) * width * 0.5f;
        xPrev = xCur;
        yPrev = yCur;
        zPrev = zCur;
    }
    float sum = 0.0f;
    for (int i = 0; i < numBins; ++i) sum += ybar[i];
    *integral = sum;
}

}  // namespace slrgpu
