// Host-side parts of the renderer boundary: camera parameters, the scene's
// light tables and the per-iteration light sampler. Plain C++ (no kernels).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ctx.cuh"

namespace gpugi {

// 64-bit xorshift* (gpugi/utilities/random.cpp:26-43) and XorshiftF (:45-49).
static inline uint64_t xorshift64(uint64_t s) {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return s * UINT64_C(2685821657736338717);
}
static inline float xorshiftF(uint64_t& s) {
    s = xorshift64(s);
    return static_cast<float>(s % 8388593) / 8388593.0f;
}

struct HV {
    float x, y, z;
};
static inline HV hsub(HV a, HV b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline HV hcross(HV a, HV b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline float hdot(HV a, HV b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline HV hnorm(HV a) {
    float l = std::sqrt(hdot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}

// Scene::LoadLightSources (gpugi/scene/scene.cpp:244-293): every valid
// triangle whose material emits becomes a light triangle; the summed area
// table is normalised to [0, 1]. Triangles are visited in leaf-slot order.
void build_light_tables(gpugi_scene* sc) {
    if (sc->lightsReady) return;
    sc->lightTris.clear();
    sc->lightSummedArea.clear();
    sc->totalAreaLightFlux = 0.0f;
    float sum = 0.0f;
    const size_t nSlots = sc->hostSlots.size() / 4;
    for (size_t i = 0; i < nSlots; ++i) {
        const int32_t* t = &sc->hostSlots[4 * i];
        if (t[0] == t[1] || sc->hostMaterials.empty()) continue;
        const float* m = &sc->hostMaterials[24 * (size_t)t[3]];
        if (m[12] == 0.0f && m[13] == 0.0f && m[14] == 0.0f) continue;
        LightTriangle lt;
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) lt.v[k][c] = sc->hostPositions[3 * (size_t)t[k] + c];
        lt.lum[0] = m[12];
        lt.lum[1] = m[13];
        lt.lum[2] = m[14];
        HV a{lt.v[0][0], lt.v[0][1], lt.v[0][2]}, b{lt.v[1][0], lt.v[1][1], lt.v[1][2]},
            c{lt.v[2][0], lt.v[2][1], lt.v[2][2]};
        HV cr = hcross(hsub(b, a), hsub(c, a));
        float area = 0.5f * std::sqrt(hdot(cr, cr));
        sc->totalAreaLightFlux += (0.2126f * lt.lum[0] + 0.7152f * lt.lum[1] + 0.0722f * lt.lum[2]) * area * 3.14159265f;
        sum += area;
        sc->lightTris.push_back(lt);
        sc->lightSummedArea.push_back(sum);
    }
    sc->lightAreaSum = sum;
    if (sum > 0.0f)
        for (float& v : sc->lightSummedArea) v /= sum;
    sc->lightsReady = true;
}

// Scene::ComputePointLightTable (gpugi/scene/scene.cpp:295-307).
static void point_light_table(gpugi_scene* sc) {
    sc->totalPointLightFlux = 0.0f;
    sc->pointLightSummedFlux.clear();
    for (const PointLight& p : sc->pointLights) {
        float flux = (0.2126f * p.intensity[0] + 0.7152f * p.intensity[1] + 0.0722f * p.intensity[2]) * 4 * 3.14159265f;
        sc->totalPointLightFlux += std::log(1.0f + flux);
        sc->pointLightSummedFlux.push_back(sc->totalPointLightFlux);
    }
    for (float& v : sc->pointLightSummedFlux) v /= sc->totalPointLightFlux;
}

// LightSampler::GenerateRandomSamples (gpugi/scene/lightsampler.cpp:18-95).
// Directional lights (an addition) take a share of the samples proportional
// to their count among all light sources when other lights exist, or all of
// them otherwise; each directional sample carries irradiance / numSamplesOfIt.
void generate_light_samples(gpugi_scene* sc, uint64_t& rng, uint32_t numSamples, float* out) {
    build_light_tables(sc);
    std::memset(out, 0, sizeof(float) * 8 * numSamples);
    uint32_t numDir = 0;
    const size_t nd = sc->dirLights.size();
    if (nd) {
        const size_t others = (sc->lightTris.empty() ? 0 : 1) + sc->pointLights.size();
        numDir = others ? (uint32_t)((uint64_t)numSamples * nd / (nd + others)) : numSamples;
        if (numDir == 0) numDir = 1;
        for (uint32_t i = 0; i < numDir; ++i) {
            const DirLight& d = sc->dirLights[i % nd];
            const uint32_t share = numDir / (uint32_t)nd + (i % nd < numDir % nd ? 1u : 0u);
            float* o = out + 8 * (size_t)(numSamples - numDir + i);
            o[0] = d.dir[0];
            o[1] = d.dir[1];
            o[2] = d.dir[2];
            o[3] = 0.0f;
            for (int c = 0; c < 3; ++c) o[4 + c] = d.irradiance[c] / (float)share;
            o[7] = 3.0f;  // directional marker
        }
    }
    const uint32_t rest = numSamples - numDir;
    if (sc->totalAreaLightFlux + sc->totalPointLightFlux == 0.0f || rest == 0) return;  // black dummies
    float pointPct = sc->totalPointLightFlux / (sc->totalAreaLightFlux + sc->totalPointLightFlux);
    uint32_t numPoint = (uint32_t)(pointPct * rest);
    uint32_t numArea = rest - numPoint;
    float sampleWeight = sc->lightAreaSum / (float)numArea;
    float* o = out;
    const size_t nl = sc->lightTris.size();
    for (uint32_t k = 0; k < numArea; ++k, o += 8) {
        float r = xorshiftF(rng);
        size_t idx = (size_t)(std::lower_bound(sc->lightSummedArea.begin(), sc->lightSummedArea.end(), r) -
                              sc->lightSummedArea.begin());
        if (idx >= nl) idx = nl - 1;
        float xi0 = xorshiftF(rng);
        float xi1 = xorshiftF(rng);
        xi0 = std::sqrt(xi0);
        float alpha = 1.0f - xi0, beta = xi0 * (1.0f - xi1), gamma = xi0 * xi1;
        const LightTriangle& lt = sc->lightTris[idx];
        HV a{lt.v[0][0], lt.v[0][1], lt.v[0][2]}, b{lt.v[1][0], lt.v[1][1], lt.v[1][2]},
            c{lt.v[2][0], lt.v[2][1], lt.v[2][2]};
        HV p{a.x * alpha + b.x * beta + c.x * gamma, a.y * alpha + b.y * beta + c.y * gamma,
             a.z * alpha + b.z * beta + c.z * gamma};
        HV n = hnorm(hcross(hsub(a, b), hsub(a, c)));
        const float bias = 1.0e-4f;
        o[0] = p.x + n.x * bias;
        o[1] = p.y + n.y * bias;
        o[2] = p.z + n.z * bias;
        o[3] = std::atan2(n.y, n.x);
        for (int ch = 0; ch < 3; ++ch) o[4 + ch] = lt.lum[ch] * sampleWeight;
        o[7] = n.z;
    }
    for (uint32_t k = 0; k < numPoint; ++k, o += 8) {
        float r = xorshiftF(rng);
        size_t idx = (size_t)(std::lower_bound(sc->pointLightSummedFlux.begin(), sc->pointLightSummedFlux.end(), r) -
                              sc->pointLightSummedFlux.begin());
        if (idx >= sc->pointLights.size()) idx = sc->pointLights.size() - 1;
        float w = sc->pointLightSummedFlux[idx];
        if (idx > 0) w -= sc->pointLightSummedFlux[idx - 1];
        const PointLight& pl = sc->pointLights[idx];
        o[0] = pl.position[0];
        o[1] = pl.position[1];
        o[2] = pl.position[2];
        o[3] = 0.0f;
        for (int ch = 0; ch < 3; ++ch) o[4 + ch] = pl.intensity[ch] / ((float)numPoint * w);
        o[7] = 2.0f;
    }
}

}  // namespace gpugi

using namespace gpugi;

extern "C" {

gpugi_status gpugi_camera_lookat(const float position[3], const float lookat[3], const float up[3],
                                 float yFovDegrees, uint32_t width, uint32_t height, gpugi_camera* out) {
    if (!position || !lookat || !up || !out || width == 0 || height == 0) return GPUGI_ERROR_INVALID_ARGUMENT;
    HV p{position[0], position[1], position[2]}, l{lookat[0], lookat[1], lookat[2]}, u{up[0], up[1], up[2]};
    HV W = hnorm(hsub(l, p));
    HV U = hnorm(hcross(W, u));
    HV V = hnorm(hcross(U, W));
    const float aspect = (float)width / (float)height;
    const float f = std::tan(yFovDegrees / 2.0f * (3.14159265358979f / 180.0f));
    U = {U.x * f * aspect, U.y * f * aspect, U.z * f * aspect};
    V = {V.x * f, V.y * f, V.z * f};
    float lu = std::sqrt(hdot(U, U)), lv = std::sqrt(hdot(V, V));
    const float v[12] = {U.x, U.y, U.z, V.x, V.y, V.z, W.x, W.y, W.z, p.x, p.y, p.z};
    std::memcpy(out->U, v, 3 * sizeof(float));
    std::memcpy(out->V, v + 3, 3 * sizeof(float));
    std::memcpy(out->W, v + 6, 3 * sizeof(float));
    std::memcpy(out->position, v + 9, 3 * sizeof(float));
    out->pixelArea = lu * lv * 4.0f / (float)(width * height);
    return GPUGI_OK;
}

gpugi_status gpugi_scene_add_point_light(gpugi_scene* sc, const float position[3], const float intensity[3]) {
    if (!sc || !position || !intensity) return GPUGI_ERROR_INVALID_ARGUMENT;
    PointLight p;
    std::memcpy(p.position, position, sizeof p.position);
    std::memcpy(p.intensity, intensity, sizeof p.intensity);
    sc->pointLights.push_back(p);
    point_light_table(sc);
    return GPUGI_OK;
}

gpugi_status gpugi_scene_add_directional_light(gpugi_scene* sc, const float towardsLight[3],
                                               const float irradiance[3]) {
    if (!sc || !towardsLight || !irradiance) return GPUGI_ERROR_INVALID_ARGUMENT;
    HV d = hnorm(HV{towardsLight[0], towardsLight[1], towardsLight[2]});
    if (!(std::isfinite(d.x) && std::isfinite(d.y) && std::isfinite(d.z))) return GPUGI_ERROR_INVALID_ARGUMENT;
    DirLight l;
    l.dir[0] = d.x;
    l.dir[1] = d.y;
    l.dir[2] = d.z;
    std::memcpy(l.irradiance, irradiance, sizeof l.irradiance);
    sc->dirLights.push_back(l);
    return GPUGI_OK;
}

gpugi_status gpugi_generate_light_samples(const gpugi_scene* scene, uint64_t* rngState, uint32_t numSamples,
                                          float* out) {
    if (!scene || !rngState || !out || numSamples == 0) return GPUGI_ERROR_INVALID_ARGUMENT;
    generate_light_samples(const_cast<gpugi_scene*>(scene), *rngState, numSamples, out);
    return GPUGI_OK;
}

}  // extern "C"
