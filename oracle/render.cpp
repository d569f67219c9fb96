// ORACLE — test infrastructure only (see glsl.hpp for the parity status).
//
// CPU restatement of gpugi's rendering passes, one shader invocation per
// pixel or light particle, run on std::threads:
//   random.glsl:1-87, helper.glsl:22-47       RNG, samplers, ONB, normal packing
//   scenedata.glsl:94-105                     GetTriangleHitInfo
//   materials.glsl:19-436                     BSDF sampling / evaluation
//   lightsource.glsl:3-93                     EstimateDirectLight (NEE)
//   pathtracer.comp:16-110                    PT pass
//   lighttracer.comp:48-193 +
//   screenreproject.glsl:19-227 +
//   showlightcaches.comp:9-65                 LT pass
//   bidirpathtracer/*                         BPT light-cache + eye pass
//   whittedraytracer.comp:14-115              Whitted ray tracer (STOP_ON_DIFFUSE_BOUNCE)
//   photonmapper/photondistribution.comp,
//   photonmapper/gather.comp, maps/grid.glsl   photon mapper (lossless hash grid)
// Two documented additions that the reference lacks: a constant sky radiance
// returned on a miss (the reference samples a cube map, black by default) and
// directional light samples (normalThetaCos == 3) for a sun.
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "oracle.hpp"

using namespace glsl;

namespace oracle {

static const float PI = 3.14159265358979f;
static const float PI_2 = 6.28318530717958f;
static const float DIVISOR_EPSILON = 1e-5f;
static const float RAY_HIT_EPSILON = 0.0001f;
static const float RAY_MAX = 3.402823466e+38f;

// ---------------------------------------------------------------- random.glsl
static uint wanghash(uint x) {
    x = (x ^ 61u) ^ (x >> 16);
    x *= 9u;
    x = x ^ (x >> 4);
    x *= 0x27d4eb2du;
    x = x ^ (x >> 15);
    return x;
}
// Random streams. Reference mode: random.glsl as written (wanghash seeds,
// xorshift32 draws, float(u) / 4294967297.0). PCG mode (the default of the
// CUDA passes, an addition): PCG-RXS-M-XS-32 (O'Neill, "PCG: A Family of
// Simple Fast Space-Efficient Statistically Good Algorithms for Random Number
// Generation", 2014, section 6.3.4) with multiplier 747796405 and increment
// 2891336453; one step doubles as the seed hash; draws as float(u >> 8) / 2^24.
struct Rng {
    uint s;
    uint pcg;
};
static uint PcgOutput(uint state) {
    uint w = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (w >> 22u) ^ w;
}
static uint PcgHash(uint x) { return PcgOutput(x * 747796405u + 2891336453u); }
static uint SeedHash(uint pcg, uint x) { return pcg ? PcgHash(x) : wanghash(x); }
static uint XorShift32(uint& seed) {
    seed ^= (seed << 13);
    seed ^= (seed >> 17);
    seed ^= (seed << 5);
    return seed;
}
static uint RandomUInt(Rng& r) {
    if (r.pcg) {
        r.s = r.s * 747796405u + 2891336453u;
        return PcgOutput(r.s);
    }
    return XorShift32(r.s);
}
// InitRandomSeed(frameSeed, invocationID) = hash(frameSeed + invocationID).
static Rng InitRandomSeed(uint pcg, uint frameSeed, uint invocationID) {
    return Rng{SeedHash(pcg, frameSeed + invocationID), pcg};
}
// float(RandomUInt) / 4294967297.0: the float literal rounds to 2^32.
static float Random(Rng& r) {
    uint u = RandomUInt(r);
    return r.pcg ? float(u >> 8) / 16777216.0f : float(u) / 4294967297.0f;
}
static vec2 Random2(Rng& seed) {
    float a = Random(seed);
    float b = Random(seed);
    return vec2(a, b);
}
// Mode of the next oracle call (the rendering entry points copy it into
// their Params; the oracle serves one caller at a time).
static uint g_rngPcg = 1;
static vec3 SampleDirection(vec2 r) {
    float cosTheta = r.x * 2.0f - 1.0f;
    float sinTheta = sqrt((1.0f - cosTheta) * (1.0f + cosTheta));
    float phi = r.y * PI_2;
    return normalize(vec3(sinTheta * std::sin(phi), sinTheta * std::cos(phi), cosTheta));
}
static vec3 SampleHemisphereCosine(vec2 r, vec3 U, vec3 V, vec3 W) {
    float phi = PI_2 * r.x;
    float sinTheta = sqrt(r.y);
    float x = sinTheta * std::cos(phi);
    float y = sinTheta * std::sin(phi);
    float z = sqrt(1.0f - r.y);
    return x * U + y * V + z * W;
}
static vec3 SamplePhongLobe(vec2 r, float exponent, vec3 U, vec3 V, vec3 W) {
    float phi = PI_2 * r.x;
    float power = std::pow(r.y, 1.0f / (exponent + 1.0f));
    float scale = sqrt(1.0f - power * power);
    float x = std::cos(phi) * scale;
    float y = std::sin(phi) * scale;
    float z = power;
    return x * U + y * V + z * W;
}

// ---------------------------------------------------------------- helper.glsl
static void CreateONB(vec3 n, vec3& U, vec3& V) {
    U = cross(n, vec3(0.0f, 1.0f, 0.0f));
    vec3 a = abs(U);
    if (a.x < 0.0001f && a.y < 0.0001f && a.z < 0.0001f) U = cross(n, vec3(1.0f, 0.0f, 0.0f));
    U = normalize(U);
    V = cross(n, U);
}
static float GetLuminance(vec3 rgb) { return dot(rgb, vec3(0.212671f, 0.715160f, 0.072169f)); }
static vec3 UnpackNormal(vec2 p) {
    float sinPhi = sqrt(saturate((1.0f - p.y) * (1.0f + p.y)));
    return vec3(std::cos(p.x) * sinPhi, std::sin(p.x) * sinPhi, p.y);
}
static vec3 UnpackNormal2(float p0, float p1) {
    float sinPhi = sqrt(1.0f - p1 * p1);
    return vec3(std::cos(p0) * sinPhi, std::sin(p0) * sinPhi, p1);
}
static vec2 PackNormal(vec3 n) {
    return vec2(n.x == 0.0f ? sign(n.y) * PI / 2 : std::atan2(n.y, n.x), n.z);
}

// ------------------------------------------------------------ materials.glsl
struct MaterialData {
    vec4 Reflectiveness;
    vec3 Opacity, Diffuse, Emissivity, Fresnel0;
    float RefractionIndexAvg;
    vec3 Fresnel1;
};

struct RenderScene {
    Scene geo;
    const float* materials = nullptr;  // 24 floats per material
    uint32_t numMaterials = 0;
};

// Material textures of the scene (oracle_set_textures; the oracle serves one
// caller at a time): RGBA32F texels, per texture {first texel, width,
// height}, per material the texture of {reflectiveness, opacity, diffuse,
// emissivity} or -1.
static const float* g_texels = nullptr;
static const uint32_t* g_texInfo = nullptr;
static const int32_t* g_matTex = nullptr;
static uint32_t g_numTexMaterials = 0;

// textureLod(sampler2D, tc, 0.0) with the reference's sampler (scene.cpp:15-20:
// magnified level 0 -> LINEAR, wrap REPEAT): bilinear per OpenGL 4.5 8.14.2,
// u = s w - 1/2, weights from the fractional parts, float arithmetic in the
// library's fixed order.
static vec4 SampleTexture(int tex, vec2 tc) {
    const uint32_t* info = g_texInfo + 4 * (size_t)tex;
    const float w = (float)info[1], h = (float)info[2];
    float u = tc.x * w - 0.5f, v = tc.y * h - 0.5f;
    if (!std::isfinite(u)) u = 0.0f;
    if (!std::isfinite(v)) v = 0.0f;
    const float fu = std::floor(u), fv = std::floor(v);
    const float a = u - fu, b = v - fv;
    float i0 = std::fmod(fu, w), j0 = std::fmod(fv, h);
    if (i0 < 0.0f) i0 = i0 + w;
    if (j0 < 0.0f) j0 = j0 + h;
    const uint32_t x0 = (uint32_t)i0 < info[1] ? (uint32_t)i0 : 0u, y0 = (uint32_t)j0 < info[2] ? (uint32_t)j0 : 0u;
    const uint32_t x1 = x0 + 1 == info[1] ? 0u : x0 + 1, y1 = y0 + 1 == info[2] ? 0u : y0 + 1;
    const float* t = g_texels + 4 * (size_t)info[0];
    auto T = [&](uint32_t x, uint32_t y, int c) { return t[4 * ((size_t)y * info[1] + x) + c]; };
    const float na = 1.0f - a, nb = 1.0f - b;
    const float w00 = na * nb, w10 = a * nb, w01 = na * b, w11 = a * b;
    float r[4];
    for (int c = 0; c < 4; ++c)
        r[c] = ((w00 * T(x0, y0, c) + w10 * T(x1, y0, c)) + w01 * T(x0, y1, c)) + w11 * T(x1, y1, c);
    return vec4(r[0], r[1], r[2], r[3]);
}

static MaterialData SampleMaterialDataConst(const RenderScene& s, int id);

// SampleMaterialData (materials.glsl:19-30): the textured maps at tc.
static MaterialData SampleMaterialData(const RenderScene& s, int id, vec2 tc) {
    MaterialData d = SampleMaterialDataConst(s, id);
    if (g_matTex && (uint32_t)id < g_numTexMaterials) {
        const int32_t* tx = g_matTex + 4 * (size_t)id;
        if (tx[0] >= 0) d.Reflectiveness = SampleTexture(tx[0], tc);
        if (tx[1] >= 0) d.Opacity = SampleTexture(tx[1], tc).xyz();
        if (tx[2] >= 0) d.Diffuse = SampleTexture(tx[2], tc).xyz();
        if (tx[3] >= 0) d.Emissivity = SampleTexture(tx[3], tc).xyz();
    }
    return d;
}

// The material record's constant values.
static MaterialData SampleMaterialDataConst(const RenderScene& s, int id) {
    const float* m = s.materials + 24 * (size_t)id;
    MaterialData d;
    d.Diffuse = vec3(m[0], m[1], m[2]);
    d.RefractionIndexAvg = m[3];
    d.Opacity = vec3(m[4], m[5], m[6]);
    d.Reflectiveness = vec4(m[8], m[9], m[10], m[11]);
    d.Emissivity = vec3(m[12], m[13], m[14]);
    d.Fresnel0 = vec3(m[16], m[17], m[18]);
    d.Fresnel1 = vec3(m[20], m[21], m[22]);
    return d;
}

static float AvgProbability(vec3 c) { return (c.x + c.y + c.z + DIVISOR_EPSILON) / (3.0f + DIVISOR_EPSILON); }
static float Avg(vec3 c) { return (c.x + c.y + c.z) / 3.0f; }

// USE_CONSTANT_REFLECTION is the active branch (materials.glsl:3-4,52-55).
static void GetBSDFDecisionPropabilities(const MaterialData& m, float, vec3& preflect, vec3& prefract,
                                         vec3& pdiffuse) {
    preflect = m.Fresnel0;
    prefract = vec3(1.0f) - saturate(preflect);
    pdiffuse = prefract * m.Opacity;
    prefract = prefract - pdiffuse;
}
static vec3 GetDiffuseProbability(const MaterialData& m, float) {
    vec3 preflect = m.Fresnel0;
    return (vec3(1.0f) - saturate(preflect)) * m.Opacity;
}

// materials.glsl:118-277
static vec3 SampleBSDFImpl(vec3 incidentDirection, const MaterialData& m, Rng& seed, vec3 N, vec3& pathThroughput,
                           bool adjoint, float& pdf, bool* isReflectedDiffuse, bool stopOnDiffuse = false) {
    float cosTheta = dot(N, incidentDirection);
    float cosThetaAbs = saturate(abs(cosTheta));
    vec3 reflectRefractDir = incidentDirection - (2.0f * cosTheta) * N;
    vec2 randomSamples = Random2(seed);
    vec3 preflect, prefract, pdiffuse;
    GetBSDFDecisionPropabilities(m, cosThetaAbs, preflect, prefract, pdiffuse);
    float avgPReflect = AvgProbability(preflect);
    float avgPRefract = AvgProbability(prefract);
    float avgPDiffuse = Avg(pdiffuse);
    vec3 pphong = preflect;
    float avgPPhong = avgPReflect;
    float pathDecisionVar = Random(seed);
    if (avgPDiffuse > pathDecisionVar) {
        if (isReflectedDiffuse) *isReflectedDiffuse = true;
        if (stopOnDiffuse) {  // STOP_ON_DIFFUSE_BOUNCE (materials.glsl:164-167)
            pathThroughput = vec3(-1.0f, 0.0f, 0.0f);
            return vec3(0.0f);
        }
        pathThroughput *= (m.Diffuse * pdiffuse) / avgPDiffuse;
        if (cosTheta > 0.0f) N = -N;
        vec3 U, V;
        CreateONB(N, U, V);
        vec3 outDir = SampleHemisphereCosine(randomSamples, U, V, N);
        float cosThetaOut = dot(N, outDir);
        pdf = saturate(cosThetaOut) / PI;
        return outDir;
    } else if (avgPDiffuse + avgPRefract > pathDecisionVar) {
        pphong = prefract;
        avgPPhong = avgPRefract;
        float eta = cosTheta < 0.0f ? 1.0f / m.RefractionIndexAvg : m.RefractionIndexAvg;
        float etaSq = eta * eta;
        float sinTheta2Sq = etaSq * (1.0f - cosTheta * cosTheta);
        if (sinTheta2Sq < 1.0f) {
            reflectRefractDir = eta * incidentDirection +
                                (sign(cosTheta) * (sqrt(saturate(1.0f - sinTheta2Sq)) - eta * cosThetaAbs)) * N;
            if (!adjoint) pathThroughput /= etaSq;
        }
    }
    reflectRefractDir = normalize(reflectRefractDir);
    vec3 RU, RV;
    CreateONB(reflectRefractDir, RU, RV);
    // The rejection loop is disabled in the reference (plausible = true), so
    // exactly one lobe sample is taken and counter == 1.
    vec3 outDir = SamplePhongLobe(randomSamples, m.Reflectiveness.w, RU, RV, reflectRefractDir);
    if (!adjoint) pathThroughput *= abs(dot(N, outDir)) / abs(dot(N, reflectRefractDir));
    float cosThetaOutAbs = abs(dot(outDir, reflectRefractDir));
    pdf = (m.Reflectiveness.w + 1.0f) / PI_2 * std::pow(cosThetaOutAbs, m.Reflectiveness.w);
    pdf *= 1.0f;
    pathThroughput *= pphong / avgPPhong;
    if (isReflectedDiffuse) *isReflectedDiffuse = false;
    return outDir;
}

// materials.glsl:306-391
static vec3 BSDFImpl(vec3 incidentDirection, vec3 excidentDirection, const MaterialData& m, vec3 N, float& pdf,
                     bool adjoint, bool specularOnly, bool stopOnDiffuse = false) {
    vec3 bsdf(0.0f);
    float cosTheta = dot(N, incidentDirection);
    float cosThetaAbs = saturate(abs(cosTheta));
    float cosThetaOut = dot(N, excidentDirection);
    vec3 preflect, prefract, pdiffuse;
    GetBSDFDecisionPropabilities(m, cosThetaAbs, preflect, prefract, pdiffuse);
    float phongFactor_brdf = (m.Reflectiveness.w + 1.0f) / (2 * PI_2 * abs(cosThetaOut) + DIVISOR_EPSILON);
    float phongNormalization_pdf = (m.Reflectiveness.w + 1.0f) / PI_2;
    vec3 reflectRefractDir = normalize(incidentDirection - (2.0f * cosTheta) * N);
    float reflectionDotExcident_powN = std::pow(saturate(dot(reflectRefractDir, excidentDirection)), m.Reflectiveness.w);
    float reflrefrBRDFFactor = phongFactor_brdf * reflectionDotExcident_powN;
    float reflrefrPDFFactor = phongNormalization_pdf * reflectionDotExcident_powN;
    bsdf = preflect * reflrefrBRDFFactor;
    bsdf *= abs(cosThetaOut) / cosThetaAbs;
    pdf = AvgProbability(preflect) * reflrefrPDFFactor;
    if (!specularOnly && cosTheta * cosThetaOut < 0.0f) {
        bsdf += pdiffuse * m.Diffuse / PI;
        pdf += Avg(pdiffuse) * saturate(cosThetaOut) / PI;
    }
    if (stopOnDiffuse) return bsdf;  // STOP_ON_DIFFUSE_BOUNCE: no refractive NEE (materials.glsl:355-358)
    float eta = cosTheta < 0.0f ? 1.0f / m.RefractionIndexAvg : m.RefractionIndexAvg;
    float etaSq = eta * eta;
    float sinTheta2Sq = etaSq * (1.0f - cosTheta * cosTheta);
    if (sinTheta2Sq < 1.0f) {
        reflectRefractDir = normalize(eta * incidentDirection +
                                      (sign(cosTheta) * (sqrt(saturate(1.0f - sinTheta2Sq)) - eta * cosThetaAbs)) * N);
        float refractionDotExcident_powN = std::pow(saturate(dot(reflectRefractDir, excidentDirection)), m.Reflectiveness.w);
        reflrefrBRDFFactor = phongFactor_brdf * refractionDotExcident_powN;
        reflrefrPDFFactor = phongNormalization_pdf * refractionDotExcident_powN;
        if (!adjoint) reflrefrBRDFFactor /= etaSq;
        reflrefrBRDFFactor *= abs(dot(N, excidentDirection)) / abs(dot(N, reflectRefractDir));
    }
    bsdf += prefract * reflrefrBRDFFactor;
    pdf += AvgProbability(prefract) * reflrefrPDFFactor;
    return bsdf;
}
static vec3 BSDF(vec3 i, vec3 e, const MaterialData& m, vec3 N, float& pdf) { return BSDFImpl(i, e, m, N, pdf, false, false); }
static vec3 AdjointBSDF(vec3 i, vec3 e, const MaterialData& m, vec3 N, float& pdf) {
    return BSDFImpl(-e, -i, m, N, pdf, true, false);
}
// materials.glsl:415-436
static float AdjointBSDFShadingNormalCorrectedOutDotN(vec3 incomingLight, vec3 toCamera, vec3 gN, vec3 sN) {
    if (dot(incomingLight, gN) * dot(incomingLight, sN) < 0 || dot(toCamera, gN) * dot(toCamera, sN) < 0) return 0.0f;
    return saturate(abs(dot(incomingLight, sN) * dot(toCamera, gN)) / max(abs(dot(incomingLight, gN)), DIVISOR_EPSILON));
}
static float AdjointBSDFShadingNormalCorrection(vec3 inDir, vec3 outDir, vec3 gN, vec3 sN) {
    if (dot(inDir, gN) * dot(inDir, sN) < 0 || dot(outDir, gN) * dot(outDir, sN) < 0) return 0.0f;
    return saturate(abs(dot(inDir, sN) * dot(outDir, gN)) / max(abs(dot(inDir, gN) * dot(outDir, sN)), DIVISOR_EPSILON));
}

// ------------------------------------------------------------ scenedata.glsl
static void GetTriangleHitInfo(const Scene& s, ivec4 tri, vec3 bc, vec3& normal, vec2& texcoord) {
    vec4 v0 = s.vertexInfo[tri.x], v1 = s.vertexInfo[tri.y], v2 = s.vertexInfo[tri.z];
    normal = normalize(UnpackNormal(vec2(v0.x, v0.y)) * bc.x + UnpackNormal(vec2(v1.x, v1.y)) * bc.y +
                       UnpackNormal(vec2(v2.x, v2.y)) * bc.z);
    texcoord = vec2(v0.z, v0.w) * bc.x + vec2(v1.z, v1.w) * bc.y + vec2(v2.z, v2.w) * bc.z;
}

// ------------------------------------------------------------ render params
struct Params {
    int width, height;
    int maxPathLength;
    int rrStartDepth;         // Russian roulette from this bounce on (0 = reference)
    vec3 camU, camV, camW, camPos;
    float pixelArea;
    uint frameSeed;
    uint rng = g_rngPcg;       // 1 PCG streams, 0 the reference's
    int numLightSamples;
    const vec4* lightSamples;  // 2 texels per sample
    vec3 sky;                  // constant radiance on a miss (addition)
    int numRaysPerLightSample; // LT / BPT
    bool stopOnDiffuse = false;  // Whitted: BSDF without its refractive part in NEE
};

struct Image {
    float* rgba;  // width*height*4, accumulated
    int width, height;
    std::mutex* locks;  // one per row, for LT splats
};

static void Splat(Image& img, int x, int y, vec3 c) {
    if (x < 0 || y < 0 || x >= img.width || y >= img.height) return;  // GLSL image atomics ignore OOB
    std::lock_guard<std::mutex> g(img.locks[y]);
    float* p = img.rgba + 4 * ((size_t)y * img.width + x);
    p[0] += c.x;
    p[1] += c.y;
    p[2] += c.z;
}

// ------------------------------------------------------------ lightsource.glsl
// Returns the NEE radiance; directional samples (normalThetaCos == 3, the
// position texel holding the direction towards the light) are the sun addition.
static vec3 EstimateDirectLight(const RenderScene& s, const Params& P, vec3 pos, vec3 normal, int idx, vec3 viewDir,
                                const MaterialData& m, bool sampleAreaLights) {
    vec4 pn0 = P.lightSamples[2 * idx];
    vec4 in1 = P.lightSamples[2 * idx + 1];
    Ray lightRay;
    if (in1.w > 2.5f) {  // directional (addition)
        lightRay.Direction = pn0.xyz();
        float surfaceCos = saturate(dot(lightRay.Direction, normal));
        if (surfaceCos <= 0.0f) return vec3(0.0f);
        lightRay.Origin = RAY_HIT_EPSILON * lightRay.Direction + pos;
        if (!TraceRayAnyHit(s.geo, lightRay, RAY_MAX, nullptr)) {
            float pdf;
            vec3 bsdf = BSDFImpl(viewDir, lightRay.Direction, m, normal, pdf, false, false, P.stopOnDiffuse);
            return (surfaceCos * in1.xyz()) * bsdf;
        }
        return vec3(0.0f);
    }
    lightRay.Direction = pn0.xyz() - pos;
    float lightDistSq = dot(lightRay.Direction, lightRay.Direction) + DIVISOR_EPSILON;
    float lightDist = sqrt(lightDistSq);
    lightRay.Direction /= lightDist;
    float surfaceCos = saturate(dot(lightRay.Direction, normal));
    if (surfaceCos <= 0.0f) return vec3(0.0f);
    if (in1.w > 1.5f) {
        lightRay.Origin = RAY_HIT_EPSILON * lightRay.Direction + pos;
        if (!TraceRayAnyHit(s.geo, lightRay, lightDist - RAY_HIT_EPSILON * 2, nullptr)) {
            vec3 irradiance = (surfaceCos / lightDistSq) * in1.xyz();
            float pdf;
            vec3 bsdf = BSDFImpl(viewDir, lightRay.Direction, m, normal, pdf, false, false, P.stopOnDiffuse);
            return irradiance * bsdf;
        }
    } else if (sampleAreaLights) {
        vec3 lightNormal = UnpackNormal(vec2(pn0.w, in1.w));
        float f = saturate(dot(lightNormal, -lightRay.Direction));
        if (f > 0.0f) {
            lightRay.Origin = RAY_HIT_EPSILON * lightRay.Direction + pos;
            if (!TraceRayAnyHit(s.geo, lightRay, lightDist - RAY_HIT_EPSILON * 2, nullptr)) {
                float pdf;
                vec3 intensity = in1.xyz() * f;
                vec3 bsdf = BSDFImpl(viewDir, lightRay.Direction, m, normal, pdf, false, false, P.stopOnDiffuse);
                vec3 irradiance = (surfaceCos / lightDistSq) * intensity;
                return irradiance * bsdf;
            }
        }
    }
    return vec3(0.0f);
}

static Ray PrimaryRay(const Params& P, Rng& seed, int x, int y) {
    vec2 sub = Random2(seed) - 0.5f;
    vec2 screen = (sub + vec2((float)x, (float)y)) / vec2((float)P.width, (float)P.height) * 2.0f - 1.0f;
    Ray r;
    r.Origin = P.camPos;
    r.Direction = normalize(screen.x * P.camU + screen.y * P.camV + P.camW);
    return r;
}

// ------------------------------------------------------------ pathtracer.comp
static vec3 PathtracePixel(const RenderScene& s, const Params& P, int x, int y) {
    const float lightSampleWeight = float(P.numLightSamples) / 1;
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, (uint)(x + y * P.width));
    vec3 color(0.0f), pathThroughput(1.0f);
    bool didNEE = false;
    Ray ray = PrimaryRay(P, seed, x, y);
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) {
            color += pathThroughput * P.sky;
            break;
        }
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 hitNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, hitNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        if (!didNEE) color += pathThroughput * m.Emissivity;
        didNEE = m.Reflectiveness.w < 500.0f;
        int sampleIndex = int(RandomUInt(seed) % (uint)P.numLightSamples);
        vec3 radiance = EstimateDirectLight(s, P, ray.Origin, hitNormal, sampleIndex, ray.Direction, m, didNEE);
        color += radiance * pathThroughput * lightSampleWeight;
        vec3 throughput(1.0f);
        float pdf;
        ray.Direction = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, false, pdf, nullptr);
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
        pathThroughput *= throughput;
        if (i >= P.rrStartDepth) {
            float p = saturate(GetLuminance(throughput));
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
    }
    return color;
}

// ------------------------------------------------------ whittedraytracer.comp
// One pixel: InitCoherentRandomSeed (random.glsl:23-28) gives every pixel of a
// frame the same RNG stream; specular/glossy decisions continue the path with
// a colour-shift throughput, the first diffuse decision ends it with
// NUM_LIGHT_SAMPLES = 2 NEE samples. The miss sky is the documented addition.
static vec3 WhittedPixel(const RenderScene& s, const Params& P, int x, int y) {
    const float lightSampleWeight = float(P.numLightSamples) / 2.0f;
    Rng seed{SeedHash(P.rng, P.frameSeed), P.rng};  // InitCoherentRandomSeed
    vec2 screen = (Random2(seed) + vec2((float)x, (float)y)) / vec2((float)P.width, (float)P.height) * 2.0f - 1.0f;
    Ray ray;
    ray.Origin = P.camPos;
    ray.Direction = normalize(screen.x * P.camU + screen.y * P.camV + P.camW);
    vec3 color(0.0f), pathThroughput(1.0f);
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) {
            color += pathThroughput * P.sky;
            break;
        }
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 hitNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, hitNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        color += pathThroughput * m.Emissivity;
        vec3 pdiffuse = GetDiffuseProbability(m, abs(dot(hitNormal, ray.Direction)));
        float pdiffuseAvg = GetLuminance(pdiffuse);
        vec3 throughput(1.0f);
        float pdf;
        vec3 sampleDirection = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, false, pdf, nullptr, true);
        if (throughput.x == -1.0f) {
            for (int l = 0; l < 2; ++l) {
                int sampleIndex = int(RandomUInt(seed) % (uint)P.numLightSamples);
                vec3 radiance = EstimateDirectLight(s, P, ray.Origin, hitNormal, sampleIndex, ray.Direction, m, true);
                color += radiance * pathThroughput * (lightSampleWeight / (pdiffuseAvg + DIVISOR_EPSILON));
            }
            break;
        }
        ray.Direction = sampleDirection;
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
        pathThroughput *= throughput / (GetLuminance(throughput) + DIVISOR_EPSILON);
    }
    return color;
}

// --------------------------------------------------------- photonmapper/*
// PackNormal32 / UnpackNormal(uint) (helper.glsl:67-76): packSnorm2x16 of
// (phi / pi, z), rounded to nearest even.
static uint PackNormal32(vec3 n) {
    float px = n.x == 0.0f ? sign(n.y) / 2.0f : std::atan2(n.y, n.x) / PI;
    auto q = [](float v) { return (uint)(uint16_t)(int16_t)std::nearbyint(clamp(v, -1.0f, 1.0f) * 32767.0f); };
    return q(px) | (q(n.z) << 16);
}
static vec3 UnpackNormal32(uint p) {
    auto u = [](uint bits) { return clamp((float)(int16_t)(uint16_t)bits / 32767.0f, -1.0f, 1.0f); };
    vec2 v(u(p & 0xFFFFu), u(p >> 16));
    v.x *= PI;
    return UnpackNormal(v);
}
struct Photon {
    vec3 flux, pos;
    uint dir;
};
// worldPosToGrid (maps/grid.glsl): ceil(pos / HashGridSpacing)
struct CellKey {
    int x, y, z;
    bool operator==(const CellKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct CellHash {
    size_t operator()(const CellKey& k) const {
        return (size_t)(uint32_t)k.x * 73856093u ^ (size_t)(uint32_t)k.y * 19349663u ^ (size_t)(uint32_t)k.z * 83492791u;
    }
};
// The reference's lossless hash map keeps a linked list per cell; a gather
// sums over every photon of the queried cells, so a map from cell to photon
// list gives the same sets (aliased cells are far outside the query radius).
struct PhotonGrid {
    float spacing = 0.0f, radiusSq = 0.0f;
    std::unordered_map<CellKey, std::vector<uint32_t>, CellHash> cells;
    std::vector<Photon> photons;
};

// photondistribution.comp:10-106, one photon path.
static void PhotonThread(const RenderScene& s, const Params& P, uint gid, int photonsPerSample,
                         std::vector<Photon>& out) {
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, gid);
    int lightSampleIndex = int(gid / (uint)photonsPerSample);
    vec4 pn0 = P.lightSamples[2 * lightSampleIndex];
    vec4 in1 = P.lightSamples[2 * lightSampleIndex + 1];
    vec3 pathThroughput = in1.xyz() * (PI / (float)photonsPerSample);
    Ray ray;
    ray.Origin = pn0.xyz();
    if (in1.w > 1.0f) {
        ray.Direction = SampleDirection(Random2(seed));
        pathThroughput *= 4.0f;
    } else {
        vec3 normal = UnpackNormal(vec2(pn0.w, in1.w));
        vec3 U, V;
        CreateONB(normal, U, V);
        ray.Direction = SampleHemisphereCosine(Random2(seed), U, V, normal);
    }
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) break;
        vec3 geometryNormal = hit.normal;
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 shadingNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, shadingNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        vec3 throughput(1.0f);
        float samplePDF;
        bool diffuse = false;
        vec3 newDirection = SampleBSDFImpl(ray.Direction, m, seed, shadingNormal, throughput, true, samplePDF, &diffuse);
        if (diffuse) out.push_back(Photon{pathThroughput, ray.Origin, PackNormal32(ray.Direction)});
        throughput *= AdjointBSDFShadingNormalCorrection(ray.Direction, newDirection, geometryNormal, shadingNormal);
        pathThroughput *= throughput;
        if (i >= P.rrStartDepth) {  // RUSSIAN_ROULETTE with the photon mapper's +0.02
            float p = saturate(GetLuminance(throughput) + 0.02f);
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
        ray.Direction = newDirection;
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
    }
}

// gather.comp:11-36
static vec3 IrradianceEstimate(const Photon& ph, const Ray& ray, const MaterialData& m, vec3 shadingNormal,
                               float radiusSq) {
    vec3 toPhoton = ph.pos - ray.Origin;
    float rsq = dot(toPhoton, toPhoton);
    if (rsq <= radiusSq && abs(dot(toPhoton, shadingNormal)) < 0.01f) {
        vec3 photonDir = UnpackNormal32(ph.dir);
        if (dot(ray.Direction, shadingNormal) * dot(photonDir, shadingNormal) < 0.0f) return vec3(0.0f);
        float cosAbs = abs(dot(ray.Direction, shadingNormal));
        vec3 fr = GetDiffuseProbability(m, cosAbs) * m.Diffuse / PI;
        float kernel = 1.0f / (PI * radiusSq);
        fr /= Avg(GetDiffuseProbability(m, cosAbs));
        return fr * ph.flux * (1.0f * kernel);
    }
    return vec3(0.0f);
}

// gather.comp:38-133, one pixel: eye path to the first diffuse decision,
// then the photons of the 2x2x2 cells from round(pos / spacing).
static vec3 GatherPixel(const RenderScene& s, const Params& P, const PhotonGrid& grid, int x, int y) {
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, (uint)(x + y * P.width));
    vec2 screen = (Random2(seed) + vec2((float)x, (float)y)) / vec2((float)P.width, (float)P.height) * 2.0f - 1.0f;
    Ray ray;
    ray.Origin = P.camPos;
    ray.Direction = normalize(screen.x * P.camU + screen.y * P.camV + P.camW);
    vec3 color(0.0f), pathThroughput(1.0f);
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) {
            color += pathThroughput * P.sky;  // addition: the reference adds nothing (its cube map lookup is commented out)
            break;
        }
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 hitNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, hitNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        color += pathThroughput * m.Emissivity;
        vec3 throughput(1.0f);
        float pdf;
        bool diffuse = false;
        vec3 newDirection = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, false, pdf, &diffuse);
        if (diffuse) {
            vec3 irradiance(0.0f);
            const int bx = (int)std::nearbyint(ray.Origin.x / grid.spacing);
            const int by = (int)std::nearbyint(ray.Origin.y / grid.spacing);
            const int bz = (int)std::nearbyint(ray.Origin.z / grid.spacing);
            for (int c = 0; c < 8; ++c) {
                auto it = grid.cells.find(CellKey{bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1)});
                if (it == grid.cells.end()) continue;
                // the cell's linked list, newest photon first (insertToHashGrid
                // prepends with atomicExchange, maps/hashmap.glsl)
                for (auto k = it->second.rbegin(); k != it->second.rend(); ++k)
                    irradiance += IrradianceEstimate(grid.photons[*k], ray, m, hitNormal, grid.radiusSq);
            }
            color += irradiance * pathThroughput;
            break;
        }
        ray.Direction = newDirection;
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
        pathThroughput *= throughput;
        if (i >= P.rrStartDepth) {
            float p = saturate(GetLuminance(throughput) + 0.02f);
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
    }
    return color;
}

// ----------------------------------------------------------- pixelmaplt/*
// PackHDR64 / UnpackHDR64 (helper.glsl:116-156): YCgCo, Y as a float, Cg and
// Co as 12-bit mantissas over a shared exponent ceil(log2(max |Cg|, |Co|)),
// clamped to [-126, 127]; log2 and exp2 taken exactly from the binary exponent.
static int Hdr64Exponent(float maxValue) {
    if (!(maxValue > 0.0f)) return -126;
    if (std::isinf(maxValue)) return 127;
    int e;
    float m = std::frexp(maxValue, &e);
    if (m == 0.5f) --e;
    return std::min(std::max(e, -126), 127);
}
static vec2 PackHDR64(vec3 c) {
    float y = c.x * 0.25f + c.y * 0.5f + c.z * 0.25f;
    float cg = c.x * -0.25f + c.y * 0.5f + c.z * -0.25f;
    float co = c.x * 0.5f + c.z * -0.5f;
    int e = Hdr64Exponent(max(abs(cg), abs(co)));
    float range = std::ldexp(1.0f, e);
    float mx = clamp(cg * 2048.0f / range + 2048.0f, 0.0f, 4095.0f);
    float my = clamp(co * 2048.0f / range + 2048.0f, 0.0f, 4095.0f);
    return vec2(y, uintBitsToFloat(((uint)mx << 20) | ((uint)my << 8) | (uint)(e + 126)));
}
static vec3 UnpackHDR64(vec2 h) {
    uint p = floatBitsToUint(h.y);
    float scale = std::ldexp(1.0f, (int)(p & 0xFFu) - 126) / 2048.0f;
    float cg = ((float)(p >> 20) - 2048.0f) * scale;
    float co = ((float)((p >> 8) & 0xFFFu) - 2048.0f) * scale;
    float tmp = h.x - cg;
    return vec3(tmp + co, h.x + cg, tmp - co);
}

struct Importon {
    vec2 throughput;  // PackHDR64
    uint dir;         // PackNormal32 of the incident direction
    vec3 pos;
    int x, y;
};
// G-buffer of the first eye hits: position, packed geometry normal (the
// reference keeps .x in the output image's alpha and the rest in a texture).
struct GBufferTexel {
    float px, py, pz, n1, n0;
};

// importondistribution.comp:19-120 with DEPTH_BUFFER_OCCLUSION_TEST and the
// lossless hash map: one eye path; returns its emission and, at a diffuse
// decision after the first vertex, the importon.
static vec3 ImportonPixel(const RenderScene& s, const Params& P, int x, int y, GBufferTexel& gb, Importon& imp,
                          bool& stored) {
    stored = false;
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, (uint)(x + y * P.width));
    Ray ray = PrimaryRay(P, seed, x, y);
    vec3 color(0.0f), pathThroughput(1.0f);
    gb.n0 = 0.0f;  // color_a.w of a path that misses
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) {
            color += pathThroughput * P.sky;  // addition: the reference's cube-map lookup is commented out
            break;
        }
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 hitNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, hitNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        if (i == 0) {
            vec3 gN = normalize(hit.normal);
            vec2 packed = PackNormal(dot(gN, ray.Direction) > 0.0f ? -gN : gN);
            gb = GBufferTexel{ray.Origin.x, ray.Origin.y, ray.Origin.z, packed.y, packed.x};
        }
        color += pathThroughput * m.Emissivity;
        vec3 throughput(1.0f);
        float pdf;
        bool diffuse = false;
        vec3 newDirection = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, false, pdf, &diffuse);
        vec3 pDiffuse = GetDiffuseProbability(m, saturate(abs(dot(hitNormal, ray.Direction))));
        if (diffuse) {
            if (i > 0) {
                pathThroughput *= pDiffuse / max(Avg(pDiffuse), DIVISOR_EPSILON);
                imp = Importon{PackHDR64(pathThroughput), PackNormal32(ray.Direction), ray.Origin, x, y};
                stored = true;
            }
            break;
        }
        ray.Direction = newDirection;
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
        pathThroughput *= throughput;
        if (i >= P.rrStartDepth) {
            float p = saturate(GetLuminance(throughput) + 0.02f);
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
    }
    return color;
}

struct ImportonGrid {
    float spacing = 0.0f, radiusSq = 0.0f;
    std::unordered_map<CellKey, std::vector<uint32_t>, CellHash> cells;
    std::vector<Importon> importons;
};

// ProjectToScreen (screenreproject.glsl:55-227) under DEPTH_BUFFER_OCCLUSION_TEST:
// the G-buffer plane test of the pixel replaces the visibility ray.
static void ProjectToScreenGBuffer(const Params& P, Image& img, const GBufferTexel* gbuf, const Ray& ray,
                                   vec3 geometryNormal, vec3 shadingNormal, const MaterialData& m,
                                   vec3 pathThroughput, bool computeFullBSDF) {
    Ray cameraRay;
    cameraRay.Direction = P.camPos - ray.Origin;
    float camViewDotRay = -dot(P.camW, cameraRay.Direction);
    if (!(camViewDotRay > 0.0f)) return;
    vec3 proj(-dot(P.camU, cameraRay.Direction), -dot(P.camV, cameraRay.Direction), camViewDotRay);
    vec2 screen(proj.x / proj.z, proj.y / proj.z);
    screen.x /= dot(P.camU, P.camU);
    screen.y /= dot(P.camV, P.camV);
    if (!(screen.x >= -1.0f && screen.x < 1.0f && screen.y > -1.0f && screen.y <= 1.0f)) return;
    float cameraDistSq = dot(cameraRay.Direction, cameraRay.Direction);
    float cameraDist = sqrt(cameraDistSq);
    cameraRay.Direction /= cameraDist;
    cameraRay.Origin = cameraRay.Direction * RAY_HIT_EPSILON + ray.Origin;
    vec2 pixelPos = (screen * 0.5f + vec2(0.5f)) * vec2((float)P.width, (float)P.height);
    int px = (int)std::nearbyint(pixelPos.x), py = (int)std::nearbyint(pixelPos.y);
    if (px < 0 || py < 0 || px >= P.width || py >= P.height) return;
    const GBufferTexel& g = gbuf[(size_t)py * P.width + px];
    vec3 occluderNormal = UnpackNormal(vec2(g.n0, g.n1));
    vec3 occluderPos = vec3(g.px, g.py, g.pz) - (4.0f * RAY_HIT_EPSILON) * occluderNormal;
    float planeDist = dot(cameraRay.Origin - occluderPos, occluderNormal) / cameraDist;
    if (!(planeDist >= -5e-4f && planeDist < 5e-3f)) return;
    float cosAtCamera = saturate(camViewDotRay / cameraDist);
    float fluxToIrradiance = AdjointBSDFShadingNormalCorrectedOutDotN(ray.Direction, cameraRay.Direction,
                                                                      geometryNormal, shadingNormal) /
                             (cosAtCamera * cosAtCamera * cosAtCamera * P.pixelArea * cameraDistSq);
    vec3 bsdf(1.0f);
    if (computeFullBSDF) {
        float pdf;
        bsdf = AdjointBSDF(ray.Direction, cameraRay.Direction, m, shadingNormal, pdf);
    } else if (dot(ray.Direction, shadingNormal) * dot(cameraRay.Direction, shadingNormal) < 0.0f) {
        vec3 pDiffuse = GetDiffuseProbability(m, abs(dot(ray.Direction, shadingNormal)));
        bsdf = pDiffuse * m.Diffuse * Avg(pDiffuse) / PI;
    } else {
        bsdf = vec3(0.0f);
    }
    Splat(img, px, py, pathThroughput * fluxToIrradiance * bsdf);
}

// photontracing.comp:38-136 (REPROJECT, USE_PIXEL_CACHE, lossless hash map),
// one photon path.
static void ImportonPhotonThread(const RenderScene& s, const Params& P, Image& img, const GBufferTexel* gbuf,
                                 const ImportonGrid& grid, uint gid, int photonsPerSample) {
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, gid);
    int lightSampleIndex = int(gid / (uint)photonsPerSample);
    vec4 pn0 = P.lightSamples[2 * lightSampleIndex];
    vec4 in1 = P.lightSamples[2 * lightSampleIndex + 1];
    vec3 pathThroughput = in1.xyz() * (PI / (float)photonsPerSample);
    bool specularPath = false;
    Ray ray;
    ray.Origin = pn0.xyz();
    if (in1.w > 1.5f) {
        ray.Direction = SampleDirection(Random2(seed));
        pathThroughput *= 4.0f;
        specularPath = true;
    } else {
        vec3 normal = UnpackNormal(vec2(pn0.w, in1.w));
        vec3 U, V;
        CreateONB(normal, U, V);
        ray.Direction = SampleHemisphereCosine(Random2(seed), U, V, normal);
    }
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) break;
        vec3 geometryNormal = hit.normal;
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 shadingNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, shadingNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        float cosThetaAbs = saturate(abs(dot(shadingNormal, ray.Direction)));
        vec3 bsdf = GetDiffuseProbability(m, cosThetaAbs) * m.Diffuse / PI;
        const int bx = (int)std::nearbyint(ray.Origin.x / grid.spacing);
        const int by = (int)std::nearbyint(ray.Origin.y / grid.spacing);
        const int bz = (int)std::nearbyint(ray.Origin.z / grid.spacing);
        for (int c = 0; c < 8; ++c) {
            auto it = grid.cells.find(CellKey{bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1)});
            if (it == grid.cells.end()) continue;
            // radianceEstimate (photontracing.comp:15-36) over the cell's list, newest first
            for (auto kk = it->second.rbegin(); kk != it->second.rend(); ++kk) {
                const Importon& im = grid.importons[*kk];
                vec3 toImporton = im.pos - ray.Origin;
                vec3 incidentDirection = UnpackNormal32(im.dir);
                if (dot(toImporton, toImporton) <= grid.radiusSq && abs(dot(toImporton, shadingNormal)) < 0.01f &&
                    dot(ray.Direction, shadingNormal) * dot(shadingNormal, incidentDirection) > 0.0f) {
                    vec3 viewPathThroughput = UnpackHDR64(im.throughput);
                    Splat(img, im.x, im.y, viewPathThroughput * (bsdf * pathThroughput) / (PI * grid.radiusSq));
                }
            }
        }
        if (Avg(pathThroughput) > 1e-10f)
            ProjectToScreenGBuffer(P, img, gbuf, ray, geometryNormal, shadingNormal, m, pathThroughput, specularPath);
        vec3 throughput(1.0f);
        float samplePDF;
        bool diffuse = false;
        vec3 newDirection = SampleBSDFImpl(ray.Direction, m, seed, shadingNormal, throughput, true, samplePDF, &diffuse);
        throughput *= AdjointBSDFShadingNormalCorrection(ray.Direction, newDirection, geometryNormal, shadingNormal);
        pathThroughput *= throughput;
        specularPath = specularPath && !diffuse;
        if (i >= P.rrStartDepth) {
            float p = saturate(GetLuminance(throughput) + 0.02f);
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
        ray.Direction = newDirection;
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
    }
}

// ------------------------------------------------------------ lightcache.glsl
struct LightCacheEntry {
    vec3 Flux;
    int MaterialIndex;
    vec3 Position;
    float Normal0;
    vec2 Texcoord;
    float Normal1;
    int PathLength;
    vec2 IncidentDirectionPacked;
    float ChainedN, ChainedT;
};
static_assert(sizeof(LightCacheEntry) == 64, "LightCacheEntry is 64 bytes");
static float MISHeuristic(float p) { return min(1e18f, p); }
static float InitialMIS() { return 1.0f; }
static float DistanceMISHeuristic(float d, float) { return MISHeuristic(d * d); }

struct LightCache {
    LightCacheEntry* entries;
    uint32_t capacity;
    std::atomic<uint32_t> count;
};

// ------------------------------------------------------ screenreproject.glsl
static void ProjectToScreen(const RenderScene& s, const Params& P, Image& img, const Ray& ray, vec3 geometryNormal,
                            vec3 shadingNormal, const MaterialData& m, vec3 pathThroughput, bool computeMIS) {
    Ray cameraRay;
    cameraRay.Direction = P.camPos - ray.Origin;
    float camViewDotRay = -dot(P.camW, cameraRay.Direction);
    if (!(camViewDotRay > 0.0f)) return;
    vec3 proj(-dot(P.camU, cameraRay.Direction), -dot(P.camV, cameraRay.Direction), camViewDotRay);
    vec2 screen(proj.x / proj.z, proj.y / proj.z);
    screen.x /= dot(P.camU, P.camU);
    screen.y /= dot(P.camV, P.camV);
    if (!(screen.x >= -1.0f && screen.x < 1.0f && screen.y > -1.0f && screen.y <= 1.0f)) return;
    float cameraDistSq = dot(cameraRay.Direction, cameraRay.Direction);
    float cameraDist = sqrt(cameraDistSq);
    cameraRay.Direction /= cameraDist;
    cameraRay.Origin = cameraRay.Direction * RAY_HIT_EPSILON + ray.Origin;
    vec2 pixelPos = (screen * 0.5f + vec2(0.5f)) * vec2((float)P.width, (float)P.height);
    int px = (int)std::nearbyint(pixelPos.x), py = (int)std::nearbyint(pixelPos.y);
    if (TraceRayAnyHit(s.geo, cameraRay, cameraDist, nullptr)) return;
    float cosAtCamera = saturate(camViewDotRay / cameraDist);
    float fluxToIrradiance = AdjointBSDFShadingNormalCorrectedOutDotN(ray.Direction, cameraRay.Direction,
                                                                      geometryNormal, shadingNormal) /
                             (cosAtCamera * cosAtCamera * cosAtCamera * P.pixelArea * cameraDistSq);
    float pdf;
    vec3 bsdf = AdjointBSDF(ray.Direction, cameraRay.Direction, m, shadingNormal, pdf);
    if (computeMIS) {
        float e2l = InitialMIS();
        float l2e = MISHeuristic(pdf);
        float mis = e2l / max(l2e + e2l, DIVISOR_EPSILON);
        bsdf *= mis;
    }
    Splat(img, px, py, pathThroughput * fluxToIrradiance * bsdf);
}

// ------------------------------------------------------------ lighttracer.comp
static void LighttraceThread(const RenderScene& s, const Params& P, Image& img, uint gid, LightCache* cache) {
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, gid);
    int lightSampleIndex = int(gid / (uint)P.numRaysPerLightSample);
    vec4 pn0 = P.lightSamples[2 * lightSampleIndex];
    vec4 in1 = P.lightSamples[2 * lightSampleIndex + 1];
    if (cache) {
        LightCacheEntry& e = cache->entries[gid];
        e.Flux = in1.xyz() / PI_2 / (float)P.numRaysPerLightSample;
        e.MaterialIndex = -1;
        e.Position = pn0.xyz();
        e.Normal0 = pn0.w;
        e.Normal1 = in1.w;
        e.Texcoord = vec2(0.0f);
        e.IncidentDirectionPacked = PackNormal(vec3(0.0f));
        e.PathLength = 0;
        e.ChainedN = e.ChainedT = 0.0f;
    }
    vec3 pathThroughput = in1.xyz() * (PI / (float)P.numRaysPerLightSample);
    Ray ray;
    ray.Origin = pn0.xyz();
    if (in1.w > 1.5f) {
        ray.Direction = SampleDirection(Random2(seed));
        pathThroughput *= 4.0f;
    } else {
        vec3 normal = UnpackNormal(vec2(pn0.w, in1.w));
        vec3 U, V;
        CreateONB(normal, U, V);
        ray.Direction = SampleHemisphereCosine(Random2(seed), U, V, normal);
    }
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) break;
        vec3 geometryNormal = hit.normal;  // not normalised (lighttracer.comp:105)
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 shadingNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, shadingNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        if (cache && m.Reflectiveness.w < 100.0f) {
            uint32_t k = cache->count.fetch_add(1);
            if (k < cache->capacity) {
                LightCacheEntry& e = cache->entries[k];
                e.Flux = pathThroughput;
                e.MaterialIndex = hit.triangle.w;
                e.Position = ray.Origin;
                vec2 pn = PackNormal(shadingNormal);
                e.Normal0 = pn.x;
                e.Normal1 = pn.y;
                e.Texcoord = tc;
                e.IncidentDirectionPacked = PackNormal(ray.Direction);
                e.PathLength = i + 1;
                e.ChainedN = e.ChainedT = 0.0f;
            }
        }
        ProjectToScreen(s, P, img, ray, geometryNormal, shadingNormal, m, pathThroughput, cache != nullptr);
        vec3 throughput(1.0f);
        float samplePDF;
        bool diffuse;
        vec3 newDirection = SampleBSDFImpl(ray.Direction, m, seed, shadingNormal, throughput, true, samplePDF, &diffuse);
        throughput *= AdjointBSDFShadingNormalCorrection(ray.Direction, newDirection, geometryNormal, shadingNormal);
        pathThroughput *= throughput;
        if (i >= P.rrStartDepth) {
            float p = saturate(GetLuminance(throughput));
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
        ray.Direction = newDirection;
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
    }
}

// showlightcaches.comp:9-65: the light samples seen directly by the camera
// (LightPathtracer::Draw runs it after the light trace, lightpathtracer.cpp:48).
static void ShowLightSample(const RenderScene& s, const Params& P, Image& img, int idx) {
    vec4 pn0 = P.lightSamples[2 * idx];
    vec4 in1 = P.lightSamples[2 * idx + 1];
    Ray cameraRay;
    cameraRay.Direction = P.camPos - pn0.xyz();
    float camViewDotRay = -dot(P.camW, cameraRay.Direction);
    if (!(camViewDotRay > 0.0f)) return;
    vec3 proj(-dot(P.camU, cameraRay.Direction), -dot(P.camV, cameraRay.Direction), camViewDotRay);
    vec2 screen(proj.x / proj.z, proj.y / proj.z);
    screen.x /= dot(P.camU, P.camU);
    screen.y /= dot(P.camV, P.camV);
    if (!(screen.x >= -1.0f && screen.x < 1.0f && screen.y > -1.0f && screen.y <= 1.0f)) return;
    float cameraDistSq = dot(cameraRay.Direction, cameraRay.Direction);
    float cameraDist = sqrt(cameraDistSq);
    cameraRay.Direction /= cameraDist;
    cameraRay.Origin = cameraRay.Direction * RAY_HIT_EPSILON + pn0.xyz();
    if (TraceRayAnyHit(s.geo, cameraRay, cameraDist, nullptr)) return;
    vec3 normal = UnpackNormal(vec2(pn0.w, in1.w));
    float cosTheta = dot(normal, cameraRay.Direction);
    float cosAtCamera = saturate(camViewDotRay / cameraDist);
    float intensityToRadiance = cosTheta / (PI_2 * cosAtCamera * cosAtCamera * cosAtCamera * P.pixelArea * cameraDistSq);
    vec3 color = in1.xyz() * intensityToRadiance;
    vec2 pix = (screen * 0.5f + vec2(0.5f)) * vec2((float)P.width, (float)P.height);
    Splat(img, (int)pix.x, (int)pix.y, color);  // ivec2() truncates
}

// ----------------------------------------------- pathtracer_bidir.comp
static vec3 BidirPixel(const RenderScene& s, const Params& P, const LightCache& cache, uint32_t numEntries, int x,
                       int y) {
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, (uint)(x + y * P.width));
    Ray ray = PrimaryRay(P, seed, x, y);
    vec3 color(0.0f), pathThroughput(1.0f);
    const uint actual = numEntries;
    const float lightSampleWeight = float(actual);
    float lastConnectionProbability = InitialMIS();
    float lastCosAbs = 1.0f;
    float mis = 0.0f;
    for (int i = 0; i < P.maxPathLength; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        if (rayHit == RAY_MAX) {
            color += pathThroughput * P.sky;  // addition: the reference's eye pass adds nothing on a miss
            break;
        }
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 hitNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, hitNormal, tc);
        MaterialData m = SampleMaterialData(s, hit.triangle.w, tc);
        float incidentSurfaceCosSat = saturate(-dot(hitNormal, ray.Direction));
        float connectionLightToEyePath = DistanceMISHeuristic(rayHit, lastCosAbs) * MISHeuristic(incidentSurfaceCosSat / PI);
        mis = (i == 0) ? 1.0f : (lastConnectionProbability / max(lastConnectionProbability + connectionLightToEyePath, DIVISOR_EPSILON));
        color += mis * pathThroughput * m.Emissivity;
        if (actual > 0) {
            uint li = RandomUInt(seed) % actual;
            const LightCacheEntry& e = cache.entries[li];
            int pathLength = e.PathLength + i + 1;
            if (pathLength <= P.maxPathLength) {
                Ray lightRay;
                lightRay.Direction = e.Position - ray.Origin;
                float lightDistSq = dot(lightRay.Direction, lightRay.Direction);
                float lightDist = sqrt(lightDistSq);
                lightRay.Direction /= max(lightDist, DIVISOR_EPSILON);
                lightRay.Origin = RAY_HIT_EPSILON * lightRay.Direction + ray.Origin;
                if (!TraceRayAnyHit(s.geo, lightRay, lightDist - RAY_HIT_EPSILON * 2, nullptr)) {
                    vec3 lightSampleHitNormal(0.0f, 1.0f, 0.0f);
                    float connectionLightPathToEyePath;
                    float cosLight = 0.0f;
                    vec3 lightSampleIntensity;
                    float cosCamera = abs(dot(lightRay.Direction, hitNormal));
                    if (e.Normal1 < 1.5f) {
                        lightSampleHitNormal = UnpackNormal2(e.Normal0, e.Normal1);
                        cosLight = abs(dot(lightRay.Direction, lightSampleHitNormal));
                    }
                    float pdf;
                    vec3 bsdf = BSDF(ray.Direction, lightRay.Direction, m, hitNormal, pdf);
                    float connectionEyePathToLightPath = MISHeuristic(pdf);
                    if (i > 0) {
                        float distMIS = DistanceMISHeuristic(rayHit, lastCosAbs);
                        connectionEyePathToLightPath *= distMIS;
                        mis = lastConnectionProbability / max(lastConnectionProbability + connectionEyePathToLightPath, DIVISOR_EPSILON);
                        if (m.Reflectiveness.w >= 100.0f) mis = 1.0f;
                    } else {
                        mis = connectionEyePathToLightPath / max(lastConnectionProbability + connectionEyePathToLightPath, DIVISOR_EPSILON);
                    }
                    float misLight = 1.0f;
                    if (e.Normal1 < 1.5f) {
                        if (e.MaterialIndex != -1) {
                            MaterialData lm = SampleMaterialData(s, e.MaterialIndex, e.Texcoord);
                            vec3 incidentDir = UnpackNormal(e.IncidentDirectionPacked);
                            vec3 lightBSDF = AdjointBSDF(lightRay.Direction, -incidentDir, lm, lightSampleHitNormal, pdf);
                            lightSampleIntensity = e.Flux * lightBSDF * cosLight;
                            connectionLightPathToEyePath = MISHeuristic(pdf) * DistanceMISHeuristic(lightDist, cosCamera);
                        } else {
                            lightSampleIntensity = e.Flux * (cosLight * PI_2);
                            connectionLightPathToEyePath = MISHeuristic(cosLight / PI) * DistanceMISHeuristic(lightDist, cosCamera);
                        }
                        misLight = connectionLightPathToEyePath / max(connectionLightPathToEyePath + connectionEyePathToLightPath, DIVISOR_EPSILON);
                    } else {
                        lightSampleIntensity = e.Flux * PI_2;
                        misLight = 1.0f;
                    }
                    mis *= misLight;
                    vec3 irradiance = (mis * lightSampleWeight * cosCamera / lightDistSq) * lightSampleIntensity;
                    color += irradiance * pathThroughput * bsdf;
                }
            }
        }
        float samplePDF;
        vec3 throughput(1.0f);
        ray.Direction = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, false, samplePDF, nullptr);
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
        pathThroughput *= throughput;
        if (i >= P.rrStartDepth) {
            float p = saturate(GetLuminance(throughput));
            if (Random(seed) >= p) break;
            pathThroughput /= p;
        }
        float reverseConnectionProbability = MISHeuristic(samplePDF);
        if (i == 0) {
            mis = reverseConnectionProbability / max(reverseConnectionProbability + lastConnectionProbability, DIVISOR_EPSILON);
        } else {
            float distMIS = DistanceMISHeuristic(rayHit, lastCosAbs);
            reverseConnectionProbability *= distMIS;
            mis = lastConnectionProbability / max(lastConnectionProbability + distMIS * reverseConnectionProbability, DIVISOR_EPSILON);
            if (m.Reflectiveness.w >= 100.0f) mis = 1.0f;
        }
        pathThroughput *= mis;
        lastConnectionProbability = reverseConnectionProbability;
        lastCosAbs = abs(dot(ray.Direction, hitNormal));
    }
    return color;
}

}  // namespace oracle

using namespace oracle;

namespace oracle {

// ------------------------------------------------- hierarchy importance
// HierarchyImportance (gpugi/renderer/hierarchyimportance.cpp:83-160) on AABB
// hierarchies: importance acquisition (hierarchy/acquisition2.comp with
// hierarchy/counthits.glsl), propagation (hierarchy/hierarchypropagation_
// init.comp and _nodes.comp), node materials (hierarchy/sampleleafmaterials
// .comp, pullmaterials.comp), node NDFs (hierarchy/sggx.glsl) and the path
// tracer that stops at well-approximated nodes (hierarchy/hierarchypathtracer
// .comp with traceray.glsl's TRACERAY_IMPORTANCE_BREAK). The importance
// buffer holds {x, y} per node, then {x, y} per leaf slot.

static const float kNotificationBias = 1.19e-07f;  // hierarchypropagation_init.comp:18

// IEEE binary16 conversions with round-to-nearest-even (packHalf2x16 /
// unpackHalf2x16; GLSL leaves the rounding of packHalf2x16 open).
static uint16_t FloatToHalf(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u, a = x & 0x7FFFFFFFu;
    if (a >= 0x7F800000u) return (uint16_t)(sign | (a > 0x7F800000u ? 0x7E00u : 0x7C00u));
    if (a >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // >= 65520 rounds to infinity
    const int e = (int)(a >> 23) - 127;
    if (e >= -14) {
        const uint32_t mant = a & 0x7FFFFFu, rem = mant & 0x1FFFu;
        uint32_t h = ((uint32_t)(e + 15) << 10) | (mant >> 13);
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    if (e < -25) return (uint16_t)sign;
    const uint32_t mant = (a & 0x7FFFFFu) | 0x800000u;
    const int shift = -e - 1;  // 14..24
    uint32_t h = mant >> shift;
    const uint32_t rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}
static float HalfToFloat(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    uint32_t x;
    if (e == 0) {
        const float v = (float)m * 5.9604644775390625e-8f;  // m * 2^-24, exact
        std::memcpy(&x, &v, 4);
        x |= sign;
    } else if (e == 31) {
        x = sign | 0x7F800000u | (m << 13);
    } else {
        x = sign | ((e + 112u) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}
static uint packHalf2x16(vec2 v) { return (uint)FloatToHalf(v.x) | ((uint)FloatToHalf(v.y) << 16); }
static vec2 unpackHalf2x16(uint p) { return vec2(HalfToFloat((uint16_t)(p & 0xFFFFu)), HalfToFloat((uint16_t)(p >> 16))); }

static inline uint NodeChild(const Scene& s, int i) { return floatBitsToUint(s.hierarchy[2 * i].w); }
static inline int NodeEscape(const Scene& s, int i) { return floatBitsToInt(s.hierarchy[2 * i + 1].w); }

// TraceRayCountHits (hierarchy/counthits.glsl:1-71): every node entered and
// every triangle hit up to rayLength gains the path importance.
static void TraceRayCountHits(const Scene& s, const Ray& ray, float rayLength, float pathImportance, float* imp) {
    const int TRIANGLES_PER_LEAF = (int)s.leafSize;
    int currentNodeIndex = 0, currentLeafIndex = 0;
    vec3 invRayDir = 1.0f / ray.Direction;
    bool nextIsLeafNode = false;
    uint64_t guard = (uint64_t)s.numNodes + (uint64_t)s.numSlots + 2;
    do {
        if (guard-- == 0) return;
        if (!nextIsLeafNode) {
            float newHit, exitDist, nodeSizeSq;
            uint childCode;
            int escape;
            if (FetchIntersectBoxNode(s, ray.Origin, invRayDir, currentNodeIndex, newHit, exitDist, childCode, escape,
                                      nodeSizeSq) && newHit <= rayLength) {
                imp[2 * currentNodeIndex] += pathImportance;
                currentNodeIndex = int(childCode & 0x7FFFFFFFu);
                nextIsLeafNode = (uint)currentNodeIndex != childCode;
                if (nextIsLeafNode) {
                    currentLeafIndex = TRIANGLES_PER_LEAF * currentNodeIndex;
                    currentNodeIndex = escape;
                }
            } else {
                currentNodeIndex = escape;
            }
        }
        if (nextIsLeafNode) {
            ivec4 triangle = s.triangles[currentLeafIndex];
            if (triangle.x == triangle.y) {
                nextIsLeafNode = false;
            } else {
                float newHit;
                vec3 bary;
                if (IntersectSlot(s, ray, currentLeafIndex, newHit, bary, triangle) && newHit <= rayLength)
                    imp[2 * ((int64_t)s.numNodes + currentLeafIndex)] += pathImportance;
                ++currentLeafIndex;
                nextIsLeafNode = (currentLeafIndex % TRIANGLES_PER_LEAF) != 0;
            }
        }
    } while (currentNodeIndex != 0 || nextIsLeafNode);
}

// acquisition2.comp:26-112 (NEXT_EVENT_IMPORTANCE, one light sample, path
// length 8, no Russian roulette) for one pixel of iteration `iteration`.
static void AcquirePixel(const RenderScene& s, const Params& P, int iteration, int x, int y, float* imp) {
    Rng seed = InitRandomSeed(0u, wanghash((uint)iteration), (uint)(x + y * P.width));  // reference streams
    vec2 screen = (Random2(seed) + vec2((float)x, (float)y)) / vec2((float)P.width, (float)P.height) * 2.0f - 1.0f;
    float pathImportance = 1.0f;
    Ray ray;
    ray.Origin = P.camPos;
    ray.Direction = normalize(screen.x * P.camU + screen.y * P.camV + P.camW);
    for (int i = 0; i < 8; ++i) {
        HitRecord hit;
        float rayHit = RAY_MAX;
        TraceRay(s.geo, ray, rayHit, hit, nullptr);
        TraceRayCountHits(s.geo, ray, rayHit * 1.000001f, pathImportance, imp);
        if (rayHit == RAY_MAX) break;
        vec3 hitNormal;
        vec2 tc;
        GetTriangleHitInfo(s.geo, hit.triangle, hit.bary, hitNormal, tc);
        MaterialData m = SampleMaterialDataConst(s, hit.triangle.w);  // hierarchy acquisition: constants
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        pathImportance *= 0.5f;
        int sampleIndex = int(RandomUInt(seed) % (uint)P.numLightSamples);
        vec4 pn0 = P.lightSamples[2 * sampleIndex], in1 = P.lightSamples[2 * sampleIndex + 1];
        Ray lightRay;
        lightRay.Direction = pn0.xyz() - ray.Origin;
        float lightDistSq = dot(lightRay.Direction, lightRay.Direction);
        float lightDist = sqrt(lightDistSq);
        lightRay.Direction /= lightDist;
        vec3 lightSampleDir = UnpackNormal(vec2(pn0.w, in1.w));
        float f = saturate(dot(lightSampleDir, -lightRay.Direction));
        if (f > 0.0f) {
            lightRay.Origin = ray.Origin;
            HitRecord lh;
            float lr = lightDist;
            TraceRay(s.geo, lightRay, lr, lh, nullptr);
            if (lr < lightDist) TraceRayCountHits(s.geo, lightRay, lr * 1.000001f, pathImportance, imp);
        }
        vec3 throughput(1.0f);
        float pdf;
        ray.Direction = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, false, pdf, nullptr);
        ray.Origin += ray.Direction * RAY_HIT_EPSILON;
    }
}

// hierarchypropagation_init.comp + _nodes.comp, run to convergence: the
// nodes pass fills a node once all its children are filled, so one pass
// over the nodes children-first (reverse preorder) gives the same values.
// The init shader reads the node's minimum corner from an undeclared
// `hierarchy0` (init.comp:59; the shader does not compile for AABB
// hierarchies); it is the node's first texel, as in the nodes shader.
static float NodeAvgArea(const Scene& s, int i) {
    vec3 sides = s.hierarchy[2 * i + 1].xyz() - s.hierarchy[2 * i].xyz();
    return (sides.x * sides.y + sides.x * sides.z + sides.y * sides.z) * 2.0f / 6.0f;
}
static void PropagateImportance(const Scene& s, int iterations, float* imp, float* subtree) {
    const int n = (int)s.numNodes;
    for (int i = 0; i < n; ++i) {
        imp[2 * i] /= (float)iterations;
        imp[2 * i + 1] = 0.0f;
        subtree[i] = 0.0f;
    }
    for (int i = n - 1; i >= 0; --i) {
        const uint childCode = NodeChild(s, i);
        float childrenImportance = 0.0f;
        if (childCode & 0x80000000u) {
            int t = (int)s.leafSize * (int)(childCode & 0x7FFFFFFFu);
            for (int k = 0; k < (int)s.leafSize; ++k, ++t) childrenImportance += imp[2 * ((int64_t)n + t)];
            childrenImportance /= (float)iterations;
            subtree[i] = max(childrenImportance, kNotificationBias);
        } else {
            int c = (int)childCode;
            while (true) {
                childrenImportance += subtree[c];
                c = NodeEscape(s, c);
                if (c == 0) break;
                // continue while i is the child's parent: the next sibling of
                // a binary node's first child is its second child
                if (c != NodeEscape(s, (int)childCode)) break;
            }
            subtree[i] = childrenImportance;
        }
        float approximation = imp[2 * i] / childrenImportance;
        imp[2 * i + 1] = approximation * approximation * NodeAvgArea(s, i);
    }
}

// sampleleafmaterials.comp / pullmaterials.comp: area-weighted node
// materials as 6 uvec2 of packed halves per node; area in Opacity.y's upper half.
static void StoreHierMaterial(uint* o, const MaterialData& m, float area) {
    o[0] = packHalf2x16(vec2(m.Reflectiveness.x, m.Reflectiveness.y));
    o[1] = packHalf2x16(vec2(m.Reflectiveness.z, m.Reflectiveness.w));
    o[2] = packHalf2x16(vec2(m.Opacity.x, m.Opacity.y));
    o[3] = packHalf2x16(vec2(m.Opacity.z, area));
    o[4] = packHalf2x16(vec2(m.Diffuse.x, m.Diffuse.y));
    o[5] = packHalf2x16(vec2(m.Diffuse.z, 0.0f));
    o[6] = packHalf2x16(vec2(m.Emissivity.x, m.Emissivity.y));
    o[7] = packHalf2x16(vec2(m.Emissivity.z, 0.0f));
    o[8] = packHalf2x16(vec2(m.Fresnel0.x, m.Fresnel0.y));
    o[9] = packHalf2x16(vec2(m.Fresnel0.z, m.RefractionIndexAvg));
    o[10] = packHalf2x16(vec2(m.Fresnel1.x, m.Fresnel1.y));
    o[11] = packHalf2x16(vec2(m.Fresnel1.z, 0.0f));
}
static MaterialData LoadHierMaterial(const uint* o) {
    MaterialData m;
    vec2 a = unpackHalf2x16(o[0]), b = unpackHalf2x16(o[1]);
    m.Reflectiveness = vec4(a.x, a.y, b.x, b.y);
    a = unpackHalf2x16(o[2]);
    b = unpackHalf2x16(o[3]);
    m.Opacity = vec3(a.x, a.y, b.x);
    a = unpackHalf2x16(o[4]);
    m.Diffuse = vec3(a.x, a.y, unpackHalf2x16(o[5]).x);
    a = unpackHalf2x16(o[6]);
    m.Emissivity = vec3(a.x, a.y, unpackHalf2x16(o[7]).x);
    a = unpackHalf2x16(o[8]);
    b = unpackHalf2x16(o[9]);
    m.Fresnel0 = vec3(a.x, a.y, b.x);
    m.RefractionIndexAvg = b.y;
    a = unpackHalf2x16(o[10]);
    m.Fresnel1 = vec3(a.x, a.y, unpackHalf2x16(o[11]).x);
    return m;
}
static void HierarchyMaterials(const RenderScene& rs, uint* out) {
    const Scene& s = rs.geo;
    for (int i = (int)s.numNodes - 1; i >= 0; --i) {
        const uint childCode = NodeChild(s, i);
        MaterialData mat;
        mat.Reflectiveness = vec4(0.0f, 0.0f, 0.0f, 0.0f);
        mat.Opacity = mat.Diffuse = mat.Emissivity = mat.Fresnel0 = mat.Fresnel1 = vec3(0.0f);
        mat.RefractionIndexAvg = 0.0f;
        float area = 0.0f;
        if (childCode & 0x80000000u) {
            const int base = (int)s.leafSize * (int)(childCode & 0x7FFFFFFFu);
            for (int k = 0; k < (int)s.leafSize; ++k) {
                ivec4 t = s.triangles[base + k];
                if (t.x == t.y) break;
                vec3 p0 = vec3(s.positions[3 * t.x], s.positions[3 * t.x + 1], s.positions[3 * t.x + 2]);
                vec3 p1 = vec3(s.positions[3 * t.y], s.positions[3 * t.y + 1], s.positions[3 * t.y + 2]);
                vec3 p2 = vec3(s.positions[3 * t.z], s.positions[3 * t.z + 1], s.positions[3 * t.z + 2]);
                vec3 c = cross(p1 - p0, p2 - p0);
                float triangleArea = sqrt(dot(c, c)) / 2.0f;
                area += triangleArea;
                MaterialData m = SampleMaterialDataConst(rs, t.w);  // hierarchy: constants
                mat.Reflectiveness = mat.Reflectiveness + m.Reflectiveness * triangleArea;
                mat.Opacity += m.Opacity * triangleArea;
                mat.Diffuse += m.Diffuse * triangleArea;
                mat.Emissivity += m.Emissivity * triangleArea;
                mat.Fresnel0 += m.Fresnel0 * triangleArea;
                mat.Fresnel1 += m.Fresnel1 * triangleArea;
                mat.RefractionIndexAvg += m.RefractionIndexAvg * triangleArea;
            }
        } else {
            const int second = NodeEscape(s, (int)childCode);
            for (int c : {(int)childCode, second}) {
                const uint* o = out + 12 * (size_t)c;
                float childArea = unpackHalf2x16(o[3]).y;
                area += childArea;
                vec2 r0 = unpackHalf2x16(o[0]) * childArea, r1 = unpackHalf2x16(o[1]) * childArea;
                mat.Reflectiveness = mat.Reflectiveness + vec4(r0.x, r0.y, r1.x, r1.y);
                vec2 v = unpackHalf2x16(o[2]) * childArea;
                mat.Opacity = mat.Opacity + vec3(v.x, v.y, unpackHalf2x16(o[3]).x * childArea);
                v = unpackHalf2x16(o[4]) * childArea;
                mat.Diffuse = mat.Diffuse + vec3(v.x, v.y, unpackHalf2x16(o[5]).x * childArea);
                v = unpackHalf2x16(o[6]) * childArea;
                mat.Emissivity = mat.Emissivity + vec3(v.x, v.y, unpackHalf2x16(o[7]).x * childArea);
                v = unpackHalf2x16(o[8]) * childArea;
                mat.Fresnel0 = mat.Fresnel0 + vec3(v.x, v.y, unpackHalf2x16(o[9]).x * childArea);
                mat.RefractionIndexAvg += unpackHalf2x16(o[9]).y * childArea;
                v = unpackHalf2x16(o[10]) * childArea;
                mat.Fresnel1 = mat.Fresnel1 + vec3(v.x, v.y, unpackHalf2x16(o[11]).x * childArea);
            }
        }
        mat.Reflectiveness = mat.Reflectiveness / area;
        mat.Opacity /= area;
        mat.Diffuse /= area;
        mat.Emissivity /= area;
        mat.Fresnel0 /= area;
        mat.Fresnel1 /= area;
        mat.RefractionIndexAvg /= area;
        StoreHierMaterial(out + 12 * (size_t)i, mat, area);
    }
}

// loadSGGX (sggx.glsl:1-14): RG16 unorm texels {sigma.x, sigma.y},
// {sigma.z, r.x}, {r.y, r.z}; S[col][row].
struct Mat3 {
    vec3 c[3];
};
static Mat3 LoadSGGX(const uint16_t* n) {
    vec3 sigma(n[0] / 65535.0f, n[1] / 65535.0f, n[2] / 65535.0f);
    vec3 r = vec3(n[3] / 65535.0f, n[4] / 65535.0f, n[5] / 65535.0f) * 2.0f - 1.0f;
    Mat3 m;
    m.c[0].x = saturate(sigma.x * sigma.x);
    m.c[1].y = saturate(sigma.y * sigma.y);
    m.c[2].z = saturate(sigma.z * sigma.z);
    m.c[0].y = m.c[1].x = clamp(r.x * sigma.x * sigma.y, -1.0f, 1.0f);
    m.c[0].z = m.c[2].x = clamp(r.y * sigma.x * sigma.z, -1.0f, 1.0f);
    m.c[1].z = m.c[2].y = clamp(r.z * sigma.y * sigma.z, -1.0f, 1.0f);
    return m;
}
static vec3 MulMV(const Mat3& m, vec3 v) {  // column combination, left to right
    return (m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z;
}

// sampleNormal (sggx.glsl:16-56): a visible normal of the node's NDF.
static vec3 SampleSGGXNormal(vec3 incident, const Mat3& S, Rng& seed) {
    Mat3 local;
    local.c[2] = -incident;
    CreateONB(incident, local.c[0], local.c[1]);
    float Sxx = dot(local.c[0], MulMV(S, local.c[0]));
    float Sxy = dot(local.c[0], MulMV(S, local.c[1]));
    float Sxz = dot(local.c[0], MulMV(S, local.c[2]));
    float Syy = dot(local.c[1], MulMV(S, local.c[1]));
    float Syz = dot(local.c[1], MulMV(S, local.c[2]));
    float Szz = dot(local.c[2], MulMV(S, local.c[2]));
    vec3 m_i, m_j, m_k;
    float det = max(0.0f, Sxx * Syy * Szz + Sxy * Syz * Sxz * 2.0f - Sxz * Sxz * Syy - Sxy * Sxy * Szz -
                              Syz * Syz * Sxx - DIVISOR_EPSILON);
    float tmp = Syy * Szz - Syz * Syz + DIVISOR_EPSILON;
    m_i = tmp != 0.0f ? vec3(sqrt(det / tmp), 0.0f, 0.0f) : vec3(0.0f);
    tmp = sqrt(tmp);
    m_j = (tmp != 0.0f && Szz != 0.0f) ? vec3((Sxy * Szz - Sxz * Syz) / tmp, tmp, 0.0f) / sqrt(Szz) : vec3(0.0f);
    m_k = Szz != 0.0f ? vec3(Sxz, Syz, Szz) / sqrt(Szz) : vec3(0.0f);
    float chi0 = Random(seed);
    float w = sqrt(1.0f - chi0);
    chi0 = sqrt(chi0);
    float chi1 = Random(seed) * 6.283185307f;
    float u = chi0 * std::cos(chi1);
    float v = chi0 * std::sin(chi1);
    vec3 normal = (u * m_i + v * m_j) + w * m_k;
    return normalize(MulMV(local, normal));
}

// TraceRay / TraceRayAnyHit with TRACERAY_IMPORTANCE_BREAK and HIT_INDEX_OUTPUT
// (traceray.glsl:25-180) at IMPORTANCE_THRESHOLD 0: a node whose importance y
// is at most threshold x entry distance ends the descent. Closest hit: the
// node becomes a hit at a hashed point between entry and exit (rayLength
// shrinks to it) and the walk continues at its escape; any hit: it occludes
// when it ends within rayLength, else it is skipped.
struct ImportanceHit {
    int node = -1, slot = -1;  // _hitIndex: slot -1 = the node itself
    float nodeImportance = 0.0f, nodeSizeSq = 0.0f;
    vec3 bary;
    ivec4 triangle{0, 0, 0, 0};
};
template <bool ANY_HIT>
static bool TraceImportance(const Scene& s, const float* imp, const Ray& ray, float& rayLength, float threshold,
                            ImportanceHit* out) {
    const int TRIANGLES_PER_LEAF = (int)s.leafSize;
    int currentNodeIndex = 0, currentLeafIndex = 0, lastNodeIndex = 0;
    float lastNodeImportance = 0.0f, lastNodeSizeSq = 0.0f;
    vec3 invRayDir = 1.0f / ray.Direction;
    bool nextIsLeafNode = false;
    uint64_t guard = (uint64_t)s.numNodes + (uint64_t)s.numSlots + 2;
    do {
        if (guard-- == 0) return false;
        if (!nextIsLeafNode) {
            float newHit, exitDist, nodeSizeSq;
            uint childCode;
            int escape;
            if (FetchIntersectBoxNode(s, ray.Origin, invRayDir, currentNodeIndex, newHit, exitDist, childCode, escape,
                                      nodeSizeSq) && newHit <= rayLength) {
                lastNodeIndex = currentNodeIndex;
                const float ix = imp[2 * currentNodeIndex], iy = imp[2 * currentNodeIndex + 1];
                lastNodeImportance = ix;
                lastNodeSizeSq = nodeSizeSq;
                if ((ix < 0.0f && newHit > 0.0f) || iy <= threshold * newHit) {
                    if (ANY_HIT) {
                        if (exitDist <= rayLength) return true;
                    } else {
                        out->nodeImportance = ix;
                        out->nodeSizeSq = lastNodeSizeSq;
                        out->node = currentNodeIndex;
                        // grouped as the shader: newHit + ((exitDist - newHit) * h) / 8388593
                        rayLength = newHit + (exitDist - newHit) *
                                                 (float)(wanghash(floatBitsToUint(exitDist)) % 8388593u) / 8388593.0f;
                        out->slot = -1;
                    }
                    currentNodeIndex = escape;
                } else {
                    currentNodeIndex = int(childCode & 0x7FFFFFFFu);
                    nextIsLeafNode = (uint)currentNodeIndex != childCode;
                    if (nextIsLeafNode) {
                        currentLeafIndex = TRIANGLES_PER_LEAF * currentNodeIndex;
                        currentNodeIndex = escape;
                    }
                }
            } else {
                currentNodeIndex = escape;
            }
        }
        if (nextIsLeafNode) {
            ivec4 triangle = s.triangles[currentLeafIndex];
            if (triangle.x == triangle.y) {
                nextIsLeafNode = false;
            } else {
                float newHit;
                vec3 bary;
                if (IntersectSlot(s, ray, currentLeafIndex, newHit, bary, triangle) && newHit < rayLength) {
                    if (ANY_HIT) return true;
                    rayLength = newHit;
                    out->triangle = triangle;
                    out->bary = bary;
                    out->node = lastNodeIndex;
                    out->slot = currentLeafIndex;
                    out->nodeImportance = lastNodeImportance;
                    out->nodeSizeSq = lastNodeSizeSq;
                }
                ++currentLeafIndex;
                nextIsLeafNode = (currentLeafIndex % TRIANGLES_PER_LEAF) != 0;
            }
        }
    } while (currentNodeIndex != 0 || nextIsLeafNode);
    return false;
}

// EstimateDirectLight with TRACERAY_IMPORTANCE_BREAK (lightsource.glsl:3-93);
// directional samples are the sun addition, offset like point lights.
static vec3 EstimateDirectLightImportance(const RenderScene& s, const Params& P, const float* imp, vec3 pos,
                                          vec3 normal, int idx, vec3 viewDir, const MaterialData& m,
                                          bool sampleAreaLights, float threshold, float distEpsilon) {
    vec4 pn0 = P.lightSamples[2 * idx];
    vec4 in1 = P.lightSamples[2 * idx + 1];
    Ray lightRay;
    if (in1.w > 2.5f) {
        lightRay.Direction = pn0.xyz();
        float surfaceCos = saturate(dot(lightRay.Direction, normal));
        if (surfaceCos <= 0.0f) return vec3(0.0f);
        lightRay.Origin = distEpsilon * lightRay.Direction + pos;
        float len = RAY_MAX;
        if (!TraceImportance<true>(s.geo, imp, lightRay, len, threshold, nullptr)) {
            float pdf;
            vec3 bsdf = BSDFImpl(viewDir, lightRay.Direction, m, normal, pdf, false, false);
            return (surfaceCos * in1.xyz()) * bsdf;
        }
        return vec3(0.0f);
    }
    lightRay.Direction = pn0.xyz() - pos;
    float lightDistSq = dot(lightRay.Direction, lightRay.Direction) + DIVISOR_EPSILON;
    float lightDist = sqrt(lightDistSq);
    lightRay.Direction /= lightDist;
    float surfaceCos = saturate(dot(lightRay.Direction, normal));
    if (surfaceCos <= 0.0f) return vec3(0.0f);
    if (in1.w > 1.5f) {
        lightRay.Origin = distEpsilon * lightRay.Direction + pos;
        float len = lightDist - RAY_HIT_EPSILON - distEpsilon;
        if (!TraceImportance<true>(s.geo, imp, lightRay, len, threshold, nullptr)) {
            vec3 irradiance = (surfaceCos / lightDistSq) * in1.xyz();
            float pdf;
            vec3 bsdf = BSDFImpl(viewDir, lightRay.Direction, m, normal, pdf, false, false);
            return irradiance * bsdf;
        }
    } else if (sampleAreaLights) {
        vec3 lightNormal = UnpackNormal(vec2(pn0.w, in1.w));
        float f = saturate(dot(lightNormal, -lightRay.Direction));
        if (f > 0.0f) {
            lightRay.Origin = RAY_HIT_EPSILON * lightRay.Direction + pos;
            float len = lightDist - RAY_HIT_EPSILON * 2;
            if (!TraceImportance<true>(s.geo, imp, lightRay, len, threshold, nullptr)) {
                float pdf;
                vec3 intensity = in1.xyz() * f;
                vec3 bsdf = BSDFImpl(viewDir, lightRay.Direction, m, normal, pdf, false, false);
                vec3 irradiance = (surfaceCos / lightDistSq) * intensity;
                return irradiance * bsdf;
            }
        }
    }
    return vec3(0.0f);
}

// hierarchypathtracer.comp:20-149 (one light sample; maxPathLength is the
// shader's MAX_PATHLENGTH, 4 in the reference): the jittered primary ray
// without the -0.5 offset, node hits shaded with the node material and a
// normal sampled from the node NDF, the adjoint BSDF sampled, the importance
// threshold x20 per bounce, Russian roulette from the first bounce.
static vec3 HierarchyPixel(const RenderScene& s, const Params& P, const float* imp, const uint* mats,
                           const uint16_t* sggx, int x, int y) {
    const float lightSampleWeight = float(P.numLightSamples) / 1;
    Rng seed = InitRandomSeed(P.rng, P.frameSeed, (uint)(x + y * P.width));
    vec2 screen = (Random2(seed) + vec2((float)x, (float)y)) / vec2((float)P.width, (float)P.height) * 2.0f - 1.0f;
    Ray ray;
    ray.Origin = P.camPos;
    ray.Direction = normalize(screen.x * P.camU + screen.y * P.camV + P.camW);
    vec3 color(0.0f), pathThroughput(1.0f);
    float pathImportanceThreshold = 0.000430915f;
    bool didNEE = false;
    for (int i = 0; i < P.maxPathLength; ++i) {
        ImportanceHit h;
        float rayHit = RAY_MAX;
        TraceImportance<false>(s.geo, imp, ray, rayHit, pathImportanceThreshold, &h);
        if (rayHit == RAY_MAX) {
            color += pathThroughput * P.sky;
            break;
        }
        ray.Origin = ray.Origin + rayHit * ray.Direction;
        vec3 hitNormal;
        MaterialData m;
        if (h.slot < 0) {
            m = LoadHierMaterial(mats + 12 * (size_t)h.node);
            Mat3 S = LoadSGGX(sggx + 6 * (size_t)h.node);
            hitNormal = SampleSGGXNormal(ray.Direction, S, seed);
        } else {
            vec2 tc;
            GetTriangleHitInfo(s.geo, h.triangle, h.bary, hitNormal, tc);
            m = SampleMaterialDataConst(s, h.triangle.w);  // hierarchy: constants
        }
        float nextThreshold = pathImportanceThreshold * 20.0f;
        float epsilon = RAY_HIT_EPSILON;
        if (h.slot < 0) epsilon = sqrt(h.nodeSizeSq) * 0.1f;
        if (!didNEE) color += pathThroughput * m.Emissivity;
        didNEE = m.Reflectiveness.w < 500.0f;
        int sampleIndex = int(RandomUInt(seed) % (uint)P.numLightSamples);
        vec3 radiance = EstimateDirectLightImportance(s, P, imp, ray.Origin, hitNormal, sampleIndex, ray.Direction, m,
                                                      didNEE, pathImportanceThreshold, epsilon);
        color += radiance * pathThroughput * lightSampleWeight;
        vec3 throughput(1.0f);
        float pdf;
        bool isReflectedDiffuse;
        ray.Direction = SampleBSDFImpl(ray.Direction, m, seed, hitNormal, throughput, true, pdf, &isReflectedDiffuse);
        ray.Origin = ray.Origin + ray.Direction * epsilon;
        pathThroughput *= throughput;
        pathImportanceThreshold = nextThreshold;
        float p = saturate(GetLuminance(throughput));
        if (Random(seed) >= p) break;
        pathThroughput /= p;
    }
    return color;
}

static RenderScene MakeRenderScene(const float* hierarchy, uint32_t numNodes, const int32_t* slots, uint32_t numSlots,
                                   uint32_t leafSize, const float* positions, const float* vertexInfo,
                                   uint32_t numVertices, const float* materials, uint32_t numMaterials) {
    RenderScene s;
    s.geo.hierarchy = reinterpret_cast<const vec4*>(hierarchy);
    s.geo.numNodes = numNodes;
    s.geo.boundsKind = BOUNDS_AABB;
    s.geo.triangles = reinterpret_cast<const ivec4*>(slots);
    s.geo.numSlots = numSlots;
    s.geo.leafSize = leafSize;
    s.geo.positions = positions;
    s.geo.numVertices = numVertices;
    s.geo.vertexInfo = reinterpret_cast<const vec4*>(vertexInfo);
    s.materials = materials;
    s.numMaterials = numMaterials;
    return s;
}
static Params MakeCameraParams(int width, int height, const float* cam, const float* lightSamples,
                               int numLightSamples) {
    Params P;
    P.width = width;
    P.height = height;
    P.maxPathLength = 0;
    P.rrStartDepth = 0;
    P.camU = vec3(cam[0], cam[1], cam[2]);
    P.camV = vec3(cam[3], cam[4], cam[5]);
    P.camW = vec3(cam[6], cam[7], cam[8]);
    P.camPos = vec3(cam[9], cam[10], cam[11]);
    P.pixelArea = cam[12];
    P.frameSeed = 0;
    P.numLightSamples = numLightSamples;
    P.lightSamples = reinterpret_cast<const vec4*>(lightSamples);
    P.sky = vec3(0.0f);
    P.numRaysPerLightSample = 0;
    return P;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

// Photon mapper iteration (PhotonMapper::Draw, gpugi/renderer/photonmapper.cpp:
// 79-114): photonsPerLightSample photons per light sample build the grid
// (spacing 2.01 x queryRadius), then the gather pass; rgba as oracle_render.
int oracle_render_pm(const float* hierarchy, uint32_t numNodes, uint32_t boundsKind, const int32_t* slots,
                     uint32_t numSlots, uint32_t leafSize, const float* positions, const float* vertexInfo,
                     uint32_t numVertices, const float* materials, uint32_t numMaterials, int width, int height,
                     int maxPathLength, int rrStartDepth, const float* cam, uint32_t frameSeed,
                     const float* lightSamples, int numLightSamples, const float* sky, int photonsPerLightSample,
                     float queryRadius, float* rgba, int numThreads) {
    RenderScene s;
    s.geo.hierarchy = reinterpret_cast<const vec4*>(hierarchy);
    s.geo.numNodes = numNodes;
    s.geo.boundsKind = boundsKind;
    s.geo.triangles = reinterpret_cast<const ivec4*>(slots);
    s.geo.numSlots = numSlots;
    s.geo.leafSize = leafSize;
    s.geo.positions = positions;
    s.geo.numVertices = numVertices;
    s.geo.vertexInfo = reinterpret_cast<const vec4*>(vertexInfo);
    s.materials = materials;
    s.numMaterials = numMaterials;
    Params P;
    P.width = width;
    P.height = height;
    P.maxPathLength = maxPathLength;
    P.rrStartDepth = rrStartDepth;
    P.camU = vec3(cam[0], cam[1], cam[2]);
    P.camV = vec3(cam[3], cam[4], cam[5]);
    P.camW = vec3(cam[6], cam[7], cam[8]);
    P.camPos = vec3(cam[9], cam[10], cam[11]);
    P.pixelArea = cam[12];
    P.frameSeed = frameSeed;
    P.numLightSamples = numLightSamples;
    P.lightSamples = reinterpret_cast<const vec4*>(lightSamples);
    P.sky = sky ? vec3(sky[0], sky[1], sky[2]) : vec3(0.0f);
    P.numRaysPerLightSample = 0;
    if (photonsPerLightSample <= 0 || !(queryRadius > 0.0f)) return -1;
    const uint64_t nPhotons = (uint64_t)numLightSamples * (uint64_t)photonsPerLightSample;
    // photons traced in parallel, stored in photon order
    const int nt = numThreads > 0 ? numThreads : (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::vector<Photon>> parts(nt);
    const uint64_t per = (nPhotons + nt - 1) / nt;
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t]() {
            for (uint64_t g = t * per; g < std::min<uint64_t>(nPhotons, (t + 1) * per); ++g)
                PhotonThread(s, P, (uint)g, photonsPerLightSample, parts[t]);
        });
    for (auto& th : pool) th.join();
    PhotonGrid grid;
    grid.spacing = queryRadius * 2.01f;
    grid.radiusSq = queryRadius * queryRadius;
    for (auto& part : parts)
        for (const Photon& ph : part) {
            const uint32_t k = (uint32_t)grid.photons.size();
            grid.photons.push_back(ph);
            CellKey key{(int)std::ceil(ph.pos.x / grid.spacing), (int)std::ceil(ph.pos.y / grid.spacing),
                        (int)std::ceil(ph.pos.z / grid.spacing)};
            grid.cells[key].push_back(k);
        }
    ParallelFor((uint64_t)width * height, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t p = b; p < e; ++p) {
            int x = (int)(p % width), y = (int)(p / width);
            vec3 c = GatherPixel(s, P, grid, x, y);
            float* o = rgba + 4 * p;
            o[0] += c.x;
            o[1] += c.y;
            o[2] += c.z;
            o[3] += 1.0f;
        }
    });
    return 0;
}

// Importon map light tracer iteration (PixelMapLighttracer::Draw,
// gpugi/renderer/pixelmaplighttracer.cpp:76-116): the eye pass stores the
// importons (one per pixel at most) and the first hits in gbuf (w*h*5 floats,
// carried from iteration to iteration: zeros before the first), then the
// photons splat into the importons' pixels and reproject; rgba as oracle_render.
int oracle_render_im(const float* hierarchy, uint32_t numNodes, uint32_t boundsKind, const int32_t* slots,
                     uint32_t numSlots, uint32_t leafSize, const float* positions, const float* vertexInfo,
                     uint32_t numVertices, const float* materials, uint32_t numMaterials, int width, int height,
                     int maxPathLength, int rrStartDepth, const float* cam, uint32_t frameSeed,
                     const float* lightSamples, int numLightSamples, const float* sky, int photonsPerLightSample,
                     float queryRadius, float* rgba, float* gbuf, int numThreads) {
    RenderScene s;
    s.geo.hierarchy = reinterpret_cast<const vec4*>(hierarchy);
    s.geo.numNodes = numNodes;
    s.geo.boundsKind = boundsKind;
    s.geo.triangles = reinterpret_cast<const ivec4*>(slots);
    s.geo.numSlots = numSlots;
    s.geo.leafSize = leafSize;
    s.geo.positions = positions;
    s.geo.numVertices = numVertices;
    s.geo.vertexInfo = reinterpret_cast<const vec4*>(vertexInfo);
    s.materials = materials;
    s.numMaterials = numMaterials;
    Params P;
    P.width = width;
    P.height = height;
    P.maxPathLength = maxPathLength;
    P.rrStartDepth = rrStartDepth;
    P.camU = vec3(cam[0], cam[1], cam[2]);
    P.camV = vec3(cam[3], cam[4], cam[5]);
    P.camW = vec3(cam[6], cam[7], cam[8]);
    P.camPos = vec3(cam[9], cam[10], cam[11]);
    P.pixelArea = cam[12];
    P.frameSeed = frameSeed;
    P.numLightSamples = numLightSamples;
    P.lightSamples = reinterpret_cast<const vec4*>(lightSamples);
    P.sky = sky ? vec3(sky[0], sky[1], sky[2]) : vec3(0.0f);
    P.numRaysPerLightSample = 0;
    if (photonsPerLightSample <= 0 || !(queryRadius > 0.0f) || !gbuf) return -1;
    const size_t numPixels = (size_t)width * height;
    GBufferTexel* gb = reinterpret_cast<GBufferTexel*>(gbuf);
    std::vector<Importon> imp(numPixels);
    std::vector<char> stored(numPixels, 0);
    ParallelFor((uint64_t)numPixels, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t p = b; p < e; ++p) {
            int x = (int)(p % width), y = (int)(p / width);
            bool st = false;
            vec3 c = ImportonPixel(s, P, x, y, gb[p], imp[p], st);
            stored[p] = st;
            float* o = rgba + 4 * p;
            o[0] += c.x;
            o[1] += c.y;
            o[2] += c.z;
            o[3] += 1.0f;
        }
    });
    ImportonGrid grid;
    grid.spacing = queryRadius * 2.01f;
    grid.radiusSq = queryRadius * queryRadius;
    for (size_t p = 0; p < numPixels; ++p) {
        if (!stored[p]) continue;
        const Importon& im = imp[p];
        const uint32_t k = (uint32_t)grid.importons.size();
        grid.importons.push_back(im);
        CellKey key{(int)std::ceil(im.pos.x / grid.spacing), (int)std::ceil(im.pos.y / grid.spacing),
                    (int)std::ceil(im.pos.z / grid.spacing)};
        grid.cells[key].push_back(k);
    }
    std::vector<std::mutex> locks(height);
    Image img{rgba, width, height, locks.data()};
    const uint64_t nPhotons = (uint64_t)numLightSamples * (uint64_t)photonsPerLightSample;
    ParallelFor(nPhotons, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t g = b; g < e; ++g) ImportonPhotonThread(s, P, img, gb, grid, (uint)g, photonsPerLightSample);
    });
    return 0;
}

// One iteration of a pass, accumulated into rgba (w*h*4 floats).
//   pass: 0 = PT, 1 = LT, 2 = BPT, 3 = Whitted
//   cam: 13 floats {U, V, W, position, pixelArea}
//   lightSamples: 8 floats per sample; sky: 3 floats (may be NULL)
int oracle_render(const float* hierarchy, uint32_t numNodes, uint32_t boundsKind, const int32_t* slots,
                  uint32_t numSlots, uint32_t leafSize, const float* positions, const float* vertexInfo,
                  uint32_t numVertices, const float* materials, uint32_t numMaterials, int pass, int width,
                  int height, int maxPathLength, int rrStartDepth, const float* cam, uint32_t frameSeed,
                  const float* lightSamples, int numLightSamples, const float* sky, float* rgba, int numThreads) {
    RenderScene s;
    s.geo.hierarchy = reinterpret_cast<const vec4*>(hierarchy);
    s.geo.numNodes = numNodes;
    s.geo.boundsKind = boundsKind;
    s.geo.triangles = reinterpret_cast<const ivec4*>(slots);
    s.geo.numSlots = numSlots;
    s.geo.leafSize = leafSize;
    s.geo.positions = positions;
    s.geo.numVertices = numVertices;
    s.geo.vertexInfo = reinterpret_cast<const vec4*>(vertexInfo);
    s.materials = materials;
    s.numMaterials = numMaterials;
    Params P;
    P.width = width;
    P.height = height;
    P.maxPathLength = maxPathLength;
    P.rrStartDepth = rrStartDepth;
    P.camU = vec3(cam[0], cam[1], cam[2]);
    P.camV = vec3(cam[3], cam[4], cam[5]);
    P.camW = vec3(cam[6], cam[7], cam[8]);
    P.camPos = vec3(cam[9], cam[10], cam[11]);
    P.pixelArea = cam[12];
    P.frameSeed = frameSeed;
    P.numLightSamples = numLightSamples;
    P.lightSamples = reinterpret_cast<const vec4*>(lightSamples);
    P.sky = sky ? vec3(sky[0], sky[1], sky[2]) : vec3(0.0f);
    // LightPathtracer::SetScreenSize (lightpathtracer.cpp:34)
    const int numPixels = width * height;
    P.numRaysPerLightSample = std::max(64, (numPixels / numLightSamples / 64) * 64);
    std::vector<std::mutex> locks(height);
    Image img{rgba, width, height, locks.data()};
    P.stopOnDiffuse = pass == 3;  // STOP_ON_DIFFUSE_BOUNCE, a compile-time define of the Whitted shader
    if (pass == 3) {
        ParallelFor((uint64_t)numPixels, numThreads, [&](uint64_t b, uint64_t e) {
            for (uint64_t p = b; p < e; ++p) {
                int x = (int)(p % width), y = (int)(p / width);
                vec3 c = WhittedPixel(s, P, x, y);
                float* o = rgba + 4 * p;
                o[0] += c.x;
                o[1] += c.y;
                o[2] += c.z;
                o[3] += 1.0f;
            }
        });
        return 0;
    }
    if (pass == 0) {
        ParallelFor((uint64_t)numPixels, numThreads, [&](uint64_t b, uint64_t e) {
            for (uint64_t p = b; p < e; ++p) {
                int x = (int)(p % width), y = (int)(p / width);
                vec3 c = PathtracePixel(s, P, x, y);
                float* o = rgba + 4 * p;
                o[0] += c.x;
                o[1] += c.y;
                o[2] += c.z;
            }
        });
        return 0;
    }
    const uint64_t nThreads = (uint64_t)numLightSamples * P.numRaysPerLightSample;
    if (pass == 1) {
        ParallelFor(nThreads, numThreads, [&](uint64_t b, uint64_t e) {
            for (uint64_t g = b; g < e; ++g) LighttraceThread(s, P, img, (uint)g, nullptr);
        });
        for (int i = 0; i < numLightSamples; ++i) ShowLightSample(s, P, img, i);
        return 0;
    }
    if (pass == 2) {
        // Capacity: every thread stores at most 1 + maxPathLength entries, so
        // the worst case never overflows (no warm-up estimate needed).
        std::vector<LightCacheEntry> entries(nThreads * (uint64_t)(maxPathLength + 1));
        LightCache cache;
        cache.entries = entries.data();
        cache.capacity = (uint32_t)entries.size();
        cache.count = (uint32_t)nThreads;  // resetcounter.comp: initial samples occupy the first slots
        ParallelFor(nThreads, numThreads, [&](uint64_t b, uint64_t e) {
            for (uint64_t g = b; g < e; ++g) LighttraceThread(s, P, img, (uint)g, &cache);
        });
        uint32_t n = std::min<uint32_t>(cache.count.load(), cache.capacity);
        ParallelFor((uint64_t)numPixels, numThreads, [&](uint64_t b, uint64_t e) {
            for (uint64_t p = b; p < e; ++p) {
                int x = (int)(p % width), y = (int)(p / width);
                vec3 c = BidirPixel(s, P, cache, n, x, y);
                float* o = rgba + 4 * p;
                o[0] += c.x;
                o[1] += c.y;
                o[2] += c.z;
                o[3] += 1.0f;
            }
        });
        return 0;
    }
    return -1;
}

uint32_t oracle_wanghash(uint32_t x) { return wanghash(x); }
uint32_t oracle_pcg_hash(uint32_t x) { return PcgHash(x); }
// Random streams of the following calls: 1 PCG, 0 the reference's.
void oracle_set_rng(int pcg) { g_rngPcg = pcg ? 1u : 0u; }

// Material textures of the following rendering calls (the arrays must stay
// alive until then); numMaterials 0 removes them.
void oracle_set_textures(const float* texels, const uint32_t* info, const int32_t* materialTextures,
                         uint32_t numMaterials) {
    g_texels = texels;
    g_texInfo = info;
    g_matTex = numMaterials ? materialTextures : nullptr;
    g_numTexMaterials = numMaterials;
}

// The restated random.glsl / helper.glsl functions over arrays, in the
// reference's random streams; `kind` and layouts as ref_eval of the
// reference-text build (oracle/ref_glue.cpp), so the two can be compared.
int oracle_eval(int kind, uint64_t n, const void* in, void* out) {
    const uint32_t* iu = static_cast<const uint32_t*>(in);
    const float* f = static_cast<const float*>(in);
    uint32_t* ou = static_cast<uint32_t*>(out);
    float* of = static_cast<float*>(out);
    for (uint64_t i = 0; i < n; ++i) {
        switch (kind) {
        case 0: ou[i] = wanghash(iu[i]); break;
        case 1: {
            Rng r{iu[i], 0u};
            for (int k = 0; k < 4; ++k) ou[4 * i + k] = RandomUInt(r);
            break;
        }
        case 2: {
            Rng r{iu[i], 0u};
            for (int k = 0; k < 4; ++k) of[4 * i + k] = Random(r);
            break;
        }
        case 3: ou[i] = InitRandomSeed(0u, iu[2 * i], iu[2 * i + 1]).s; break;
        case 4: {
            vec3 d = SampleDirection(vec2(f[2 * i], f[2 * i + 1]));
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 5: {
            const float* q = f + 5 * i;
            vec3 N(q[2], q[3], q[4]), U, V;
            CreateONB(N, U, V);
            vec3 d = SampleHemisphereCosine(vec2(q[0], q[1]), U, V, N);
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 6: {
            const float* q = f + 6 * i;
            vec3 N(q[3], q[4], q[5]), U, V;
            CreateONB(N, U, V);
            vec3 d = SamplePhongLobe(vec2(q[0], q[1]), q[2], U, V, N);
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 7: {
            vec3 N(f[3 * i], f[3 * i + 1], f[3 * i + 2]), U, V;
            CreateONB(N, U, V);
            of[6 * i] = U.x, of[6 * i + 1] = U.y, of[6 * i + 2] = U.z;
            of[6 * i + 3] = V.x, of[6 * i + 4] = V.y, of[6 * i + 5] = V.z;
            break;
        }
        case 8: {
            vec3 d = UnpackNormal(vec2(f[2 * i], f[2 * i + 1]));
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 9: {
            vec2 q = PackNormal(vec3(f[3 * i], f[3 * i + 1], f[3 * i + 2]));
            of[2 * i] = q.x, of[2 * i + 1] = q.y;
            break;
        }
        case 10: of[i] = GetLuminance(vec3(f[3 * i], f[3 * i + 1], f[3 * i + 2])); break;
        case 11: {  // SampleTexture(texture f[0], tc f[1], f[2]) of the textures set by oracle_set_textures
            vec4 r = SampleTexture((int)f[3 * i], vec2(f[3 * i + 1], f[3 * i + 2]));
            of[4 * i] = r.x, of[4 * i + 1] = r.y, of[4 * i + 2] = r.z, of[4 * i + 3] = r.w;
            break;
        }
        default: return 1;
        }
    }
    return 0;
}

// HierarchyImportance::Draw's importance pass on an AABB hierarchy
// (hierarchyimportance.cpp:83-109): `iterations` acquisition passes of
// width x height paths (numbered 1..iterations), then the propagation.
// imp: 2 * (numNodes + numSlots) floats {x, y}; subtree: numNodes floats.
int oracle_hier_importance(const float* hierarchy, uint32_t numNodes, const int32_t* slots, uint32_t numSlots,
                           uint32_t leafSize, const float* positions, const float* vertexInfo, uint32_t numVertices,
                           const float* materials, uint32_t numMaterials, int width, int height, const float* cam,
                           const float* lightSamples, int numLightSamples, int iterations, float* imp, float* subtree,
                           int numThreads) {
    if (iterations < 1 || numLightSamples < 1) return -1;
    RenderScene s = MakeRenderScene(hierarchy, numNodes, slots, numSlots, leafSize, positions, vertexInfo, numVertices,
                                    materials, numMaterials);
    Params P = MakeCameraParams(width, height, cam, lightSamples, numLightSamples);
    const size_t n = 2 * ((size_t)numNodes + numSlots);
    const uint64_t pixels = (uint64_t)width * height;
    int nt = numThreads > 0 ? numThreads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = (int)std::min<uint64_t>((uint64_t)nt, std::max<uint64_t>(1, pixels));
    std::vector<std::vector<float>> part(nt, std::vector<float>(n, 0.0f));
    std::vector<std::thread> pool;
    const uint64_t per = (pixels + nt - 1) / nt;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t]() {
            for (int it = 1; it <= iterations; ++it)
                for (uint64_t p = t * per; p < std::min<uint64_t>(pixels, (t + 1) * per); ++p)
                    AcquirePixel(s, P, it, (int)(p % width), (int)(p / width), part[t].data());
        });
    for (auto& th : pool) th.join();
    for (size_t k = 0; k < n; ++k) {
        float acc = 0.0f;
        for (int t = 0; t < nt; ++t) acc += part[t][k];
        imp[k] = acc;
    }
    PropagateImportance(s.geo, iterations, imp, subtree);
    return 0;
}

// The propagation alone on accumulated importance x (imp: 2 per node and slot).
int oracle_hier_propagate(const float* hierarchy, uint32_t numNodes, const int32_t* slots, uint32_t numSlots,
                          uint32_t leafSize, int iterations, float* imp, float* subtree) {
    RenderScene s = MakeRenderScene(hierarchy, numNodes, slots, numSlots, leafSize, nullptr, nullptr, 0, nullptr, 0);
    PropagateImportance(s.geo, iterations, imp, subtree);
    return 0;
}

// ComputeHierarchyMaterials (hierarchyimportance.cpp:136-160): 12 uint32 per node.
int oracle_hier_materials(const float* hierarchy, uint32_t numNodes, const int32_t* slots, uint32_t numSlots,
                          uint32_t leafSize, const float* positions, const float* vertexInfo, uint32_t numVertices,
                          const float* materials, uint32_t numMaterials, uint32_t* out) {
    RenderScene s = MakeRenderScene(hierarchy, numNodes, slots, numSlots, leafSize, positions, vertexInfo, numVertices,
                                    materials, numMaterials);
    HierarchyMaterials(s, out);
    return 0;
}

// One iteration of the hierarchy path tracer into rgba (alpha counts iterations).
int oracle_render_hier(const float* hierarchy, uint32_t numNodes, const int32_t* slots, uint32_t numSlots,
                       uint32_t leafSize, const float* positions, const float* vertexInfo, uint32_t numVertices,
                       const float* materials, uint32_t numMaterials, int width, int height, int maxPathLength,
                       const float* cam, uint32_t frameSeed, const float* lightSamples, int numLightSamples,
                       const float* sky, const float* imp, const uint32_t* hierMaterials, const uint16_t* sggx,
                       float* rgba, int numThreads) {
    RenderScene s = MakeRenderScene(hierarchy, numNodes, slots, numSlots, leafSize, positions, vertexInfo, numVertices,
                                    materials, numMaterials);
    Params P = MakeCameraParams(width, height, cam, lightSamples, numLightSamples);
    P.maxPathLength = maxPathLength;
    P.frameSeed = frameSeed;
    P.sky = sky ? vec3(sky[0], sky[1], sky[2]) : vec3(0.0f);
    ParallelFor((uint64_t)width * height, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t p = b; p < e; ++p) {
            vec3 c = HierarchyPixel(s, P, imp, hierMaterials, sggx, (int)(p % width), (int)(p / width));
            float* o = rgba + 4 * p;
            o[0] += c.x;
            o[1] += c.y;
            o[2] += c.z;
            o[3] += 1.0f;
        }
    });
    return 0;
}

// packHalf2x16 / unpackHalf2x16 of n values (tests of the conversion).
void oracle_float_to_half(const float* in, uint16_t* out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) out[i] = FloatToHalf(in[i]);
}
void oracle_half_to_float(const uint16_t* in, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) out[i] = HalfToFloat(in[i]);
}

}  // extern "C"
