// ORACLE — test infrastructure only (see glsl.hpp for the parity status).
//
// The host light sampler that feeds every pass its per-iteration light
// samples, restated from the reference's C++:
//   LightSampler::GenerateRandomSamples   gpugi/scene/lightsampler.cpp:18-95
//   Scene::LoadLightSources               gpugi/scene/scene.cpp:244-293
//   Scene::ComputePointLightTable         gpugi/scene/scene.cpp:295-307
//   Xorshift (64-bit xorshift*), XorshiftF gpugi/utilities/random.cpp:26-49
// The epsilon library's surface(Triangle) and normalize(Vec3) are not in the
// reference tree; they are written from their definitions (half the length
// of the edge cross product; v / sqrt(dot(v, v))) and are unpinned.
//
// Light triangles are taken in the order of the scene's triangle array
// (for a bvhmake file: the leaf slots, which is the order its `triangles`
// chunk stores them), skipping invalid slots (v0 == v1) and materials whose
// emissivity is zero, as LoadLightSources does.
//
// Directional lights are an addition of this project (the reference has
// area and point lights only); their share of the samples is restated here
// as the library defines it: numSamples * nd / (nd + others) samples (others
// = 1 if area lights exist, plus the point lights; all samples when there
// are no others; at least one), placed after the area and point samples,
// sample i of them for light i mod nd with irradiance / (that light's share).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl.hpp"

using namespace glsl;

namespace {

uint64_t Xorshift64(uint64_t rndState) {
    rndState ^= rndState >> 12;
    rndState ^= rndState << 25;
    rndState ^= rndState >> 27;
    return rndState * UINT64_C(2685821657736338717);
}

float XorshiftF(uint64_t& rndState) {
    rndState = Xorshift64(rndState);
    return static_cast<float>(rndState % 8388593) / 8388593.0f;
}

struct LightTriangle {
    vec3 v0, v1, v2;
    vec3 luminance;
};

const float kPi = 3.14159265358979f;

float TriangleSurface(const vec3& a, const vec3& b, const vec3& c) {
    vec3 cr = cross(b - a, c - a);
    return 0.5f * std::sqrt(dot(cr, cr));
}

}  // namespace

extern "C" {

// positions: 3 floats per vertex; slots: 4 int32 per triangle slot
// {v0, v1, v2, material}; materials: 24 floats per material (emissivity at
// floats 12..14); points: 6 floats each {position, intensity}; dirs: 6 floats
// each {towards the light (unit), irradiance}. Writes 8 floats per sample.
int oracle_light_samples(const float* positions, const int32_t* slots, uint32_t numSlots, const float* materials,
                         const float* points, uint32_t numPoints, const float* dirs, uint32_t numDirs,
                         uint64_t* rngState, uint32_t numSamples, float* out) {
    // LoadLightSources
    std::vector<LightTriangle> lightTriangles;
    std::vector<float> lightSummedArea;
    float totalAreaLightFlux = 0.0f, sum = 0.0f;
    for (uint32_t i = 0; i < numSlots; ++i) {
        const int32_t* tri = slots + 4 * (size_t)i;
        if (tri[0] == tri[1] || !materials) continue;
        const float* e = materials + 24 * (size_t)tri[3] + 12;
        if (e[0] == 0.0f && e[1] == 0.0f && e[2] == 0.0f) continue;
        LightTriangle lt;
        lt.luminance = vec3(e[0], e[1], e[2]);
        const float* p0 = positions + 3 * (size_t)tri[0];
        const float* p1 = positions + 3 * (size_t)tri[1];
        const float* p2 = positions + 3 * (size_t)tri[2];
        lt.v0 = vec3(p0[0], p0[1], p0[2]);
        lt.v1 = vec3(p1[0], p1[1], p1[2]);
        lt.v2 = vec3(p2[0], p2[1], p2[2]);
        lightTriangles.push_back(lt);
        float area = TriangleSurface(lt.v0, lt.v1, lt.v2);
        totalAreaLightFlux += dot(vec3(0.2126f, 0.7152f, 0.0722f), lt.luminance) * area * kPi;
        sum += area;
        lightSummedArea.push_back(sum);
    }
    float lightAreaSum = 0.0f;
    if (!lightSummedArea.empty()) {
        lightAreaSum = lightSummedArea.back();
        for (float& v : lightSummedArea) v /= lightAreaSum;
    }
    // ComputePointLightTable
    float totalPointLightFlux = 0.0f;
    std::vector<float> pointLightSummedFlux;
    for (uint32_t i = 0; i < numPoints; ++i) {
        const float* in = points + 6 * (size_t)i + 3;
        float flux = dot(vec3(0.2126f, 0.7152f, 0.0722f), vec3(in[0], in[1], in[2])) * 4 * kPi;
        totalPointLightFlux += std::log(1.0f + flux);
        pointLightSummedFlux.push_back(totalPointLightFlux);
    }
    for (float& v : pointLightSummedFlux) v /= totalPointLightFlux;

    std::memset(out, 0, sizeof(float) * 8 * (size_t)numSamples);
    // directional share (addition)
    uint32_t numDir = 0;
    if (numDirs) {
        const uint32_t others = (lightTriangles.empty() ? 0u : 1u) + numPoints;
        numDir = others ? (uint32_t)((uint64_t)numSamples * numDirs / (numDirs + others)) : numSamples;
        if (numDir == 0) numDir = 1;
        for (uint32_t i = 0; i < numDir; ++i) {
            const uint32_t l = i % numDirs;
            const uint32_t share = numDir / numDirs + (l < numDir % numDirs ? 1u : 0u);
            const float* d = dirs + 6 * (size_t)l;
            float* o = out + 8 * (size_t)(numSamples - numDir + i);
            o[0] = d[0];
            o[1] = d[1];
            o[2] = d[2];
            o[3] = 0.0f;
            for (int c = 0; c < 3; ++c) o[4 + c] = d[3 + c] / (float)share;
            o[7] = 3.0f;
        }
    }
    const uint32_t rest = numSamples - numDir;
    // GenerateRandomSamples: black dummies without area or point lights
    if (totalAreaLightFlux + totalPointLightFlux == 0.0f || rest == 0) return 0;
    float pointLightPercentage = totalPointLightFlux / (totalAreaLightFlux + totalPointLightFlux);
    unsigned numPointSamples = unsigned(pointLightPercentage * rest);
    unsigned numAreaSamples = rest - numPointSamples;
    float sampleWeight = lightAreaSum / numAreaSamples;
    float* dst = out;
    for (unsigned s = 0; s < numAreaSamples; ++s, dst += 8) {
        float randomTriangle = XorshiftF(*rngState);
        const float* at = std::lower_bound(lightSummedArea.data(), lightSummedArea.data() + lightSummedArea.size(),
                                           randomTriangle);
        size_t triangleIdx = (size_t)(at - lightSummedArea.data());
        if (triangleIdx >= lightTriangles.size()) return 1;  // the reference asserts here
        float xi0 = XorshiftF(*rngState);
        float xi1 = XorshiftF(*rngState);
        xi0 = std::sqrt(xi0);
        float alpha = 1.0f - xi0;
        float beta = xi0 * (1.0f - xi1);
        float gamma = xi0 * xi1;
        const LightTriangle& lt = lightTriangles[triangleIdx];
        vec3 position = lt.v0 * alpha + lt.v1 * beta + lt.v2 * gamma;
        vec3 normal = normalize(cross(lt.v0 - lt.v1, lt.v0 - lt.v2));
        position += normal * 1.0e-4f;  // _positionBias default (lightsampler.hpp:27)
        dst[0] = position.x;
        dst[1] = position.y;
        dst[2] = position.z;
        dst[3] = std::atan2(normal.y, normal.x);
        vec3 intensity = lt.luminance * sampleWeight;
        dst[4] = intensity.x;
        dst[5] = intensity.y;
        dst[6] = intensity.z;
        dst[7] = normal.z;
    }
    for (unsigned s = 0; s < numPointSamples; ++s, dst += 8) {
        float randomPointLight = XorshiftF(*rngState);
        const float* at = std::lower_bound(pointLightSummedFlux.data(),
                                           pointLightSummedFlux.data() + pointLightSummedFlux.size(), randomPointLight);
        size_t lightIdx = (size_t)(at - pointLightSummedFlux.data());
        if (lightIdx >= numPoints) return 1;  // the reference asserts here
        sampleWeight = *at;
        if (lightIdx > 0) sampleWeight -= pointLightSummedFlux[lightIdx - 1];
        const float* pl = points + 6 * lightIdx;
        dst[0] = pl[0];
        dst[1] = pl[1];
        dst[2] = pl[2];
        dst[3] = 0.0f;
        for (int c = 0; c < 3; ++c) dst[4 + c] = pl[3 + c] / (numPointSamples * sampleWeight);
        dst[7] = 2.0f;
    }
    return 0;
}

}  // extern "C"
