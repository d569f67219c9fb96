// Device shading library: gpugi's RNG, samplers, BSDF and light-transport
// helpers as CUDA device functions.
//
//   RNG / samplers        gpugi/shader/random.glsl:1-87 (+ PCG, see Rng)
//   ONB / normal packing  gpugi/shader/helper.glsl:22-76
//   hit attributes        gpugi/shader/scenedata.glsl:94-105
//   BSDF                  gpugi/shader/materials.glsl:33-436 (USE_CONSTANT_REFLECTION)
//   MIS helpers           gpugi/shader/bidirpathtracer/lightcache.glsl:59-89
//
// Shading math is ordinary float code (FMA contraction allowed): only the
// traversal is held to bit-exactness; images are judged by RMSE.
#pragma once
#include "common.cuh"
#include "scene.cuh"

namespace gpugi {

constexpr float kPI = 3.14159265358979f;
constexpr float kPI_2 = 6.28318530717958f;
constexpr float kDIVISOR_EPSILON = 1e-5f;
constexpr float kRAY_HIT_EPSILON = 0.0001f;
constexpr float kRAY_MAX = 3.402823466e+38f;

GPUGI_HD uint32_t wanghash(uint32_t x) {
    x = (x ^ 61u) ^ (x >> 16);
    x *= 9u;
    x = x ^ (x >> 4);
    x *= 0x27d4eb2du;
    x = x ^ (x >> 15);
    return x;
}

// Random streams of the passes. Two generators share the 32-bit state of a
// path (the wavefront stores one uint32 per path):
//  * reference (parity mode): gpugi/shader/random.glsl:1-43. Path seed
//    InitRandomSeed(FrameSeed, index) = wanghash(FrameSeed + index) with
//    FrameSeed = WangHash(iteration), draws by xorshift32, and
//    Random = float(u) / 4294967297.0;
//  * PCG (the default): PCG-RXS-M-XS-32, the 32-bit-state member of
//    O'Neill's PCG family (M. E. O'Neill, "PCG: A Family of Simple Fast
//    Space-Efficient Statistically Good Algorithms for Random Number
//    Generation", HMC-CS-2014-0905, section 6.3.4): an LCG step
//    s = s * 747796405 + 2891336453 followed by the RXS-M-XS output
//    permutation. One step from a given state doubles as the hash that seeds
//    a path per pixel (Jarzynski and Olano, "Hash Functions for GPU
//    Rendering", JCGT 9(3), 2020): seed = pcg(pcg(iteration) + index).
//    Random = float(u >> 8) * 2^-24, in [0, 1).
// `pcg` is uniform across a launch (a field of the call's constants), so the
// selection costs no divergence.
struct Rng {
    uint32_t s;
    uint32_t pcg;
};
GPUGI_HD uint32_t pcg_output(uint32_t state) {
    const uint32_t w = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (w >> 22u) ^ w;
}
GPUGI_HD uint32_t pcg_hash(uint32_t x) { return pcg_output(x * 747796405u + 2891336453u); }
GPUGI_HD uint32_t rng_hash(uint32_t pcg, uint32_t x) { return pcg ? pcg_hash(x) : wanghash(x); }
// InitRandomSeed(FrameSeed(frame), index) of the selected generator.
GPUGI_HD Rng rng_init(uint32_t pcg, uint32_t frame, uint32_t index) {
    return Rng{rng_hash(pcg, rng_hash(pcg, frame) + index), pcg};
}
// InitCoherentRandomSeed(FrameSeed(frame)): one stream for every pixel.
GPUGI_HD Rng rng_init_coherent(uint32_t pcg, uint32_t frame) { return Rng{rng_hash(pcg, rng_hash(pcg, frame)), pcg}; }
// RandomUInt (random.glsl:11-19), also the reference's grid-cell hash.
GPUGI_HD uint32_t xorshift32(uint32_t& s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
GPUGI_D uint32_t random_uint(Rng& r) {
    if (r.pcg) {
        r.s = r.s * 747796405u + 2891336453u;
        return pcg_output(r.s);
    }
    return xorshift32(r.s);
}
// Reference: float(u) / 4294967297.0 in GLSL float arithmetic; the literal
// rounds to 2^32, and a division by a power of two is exact, so this is
// float(u) * 2^-32 (1.0 for u >= 2^32 - 128, as in the shader).
GPUGI_D float random01(Rng& r) {
    const uint32_t u = random_uint(r);
    return r.pcg ? __uint2float_rn(u >> 8) * 5.9604644775390625e-8f : __uint2float_rn(u) * 2.3283064365386963e-10f;
}
GPUGI_D float2 random2(Rng& r) {
    float a = random01(r);
    float b = random01(r);
    return make_float2(a, b);
}

GPUGI_D float3 sample_direction(float2 r) {
    float cosTheta = r.x * 2.0f - 1.0f;
    float sinTheta = sqrtf((1.0f - cosTheta) * (1.0f + cosTheta));
    float phi = r.y * kPI_2;
    float s, c;
    sincosf(phi, &s, &c);
    return normalize(f3(sinTheta * s, sinTheta * c, cosTheta));
}
GPUGI_D float3 sample_hemisphere_cosine(float2 r, float3 U, float3 V, float3 W) {
    float phi = kPI_2 * r.x;
    float sinTheta = sqrtf(r.y);
    float s, c;
    sincosf(phi, &s, &c);
    float z = sqrtf(1.0f - r.y);
    return (sinTheta * c) * U + (sinTheta * s) * V + z * W;
}
GPUGI_D float3 sample_phong_lobe(float2 r, float exponent, float3 U, float3 V, float3 W) {
    float phi = kPI_2 * r.x;
    float power = powf(r.y, 1.0f / (exponent + 1.0f));
    float scale = sqrtf(1.0f - power * power);
    float s, c;
    sincosf(phi, &s, &c);
    return (c * scale) * U + (s * scale) * V + power * W;
}
GPUGI_D void create_onb(float3 n, float3& U, float3& V) {
    U = cross(n, f3(0.0f, 1.0f, 0.0f));
    if (fabsf(U.x) < 0.0001f && fabsf(U.y) < 0.0001f && fabsf(U.z) < 0.0001f) U = cross(n, f3(1.0f, 0.0f, 0.0f));
    U = normalize(U);
    V = cross(n, U);
}
GPUGI_D float luminance(float3 c) { return dot(c, f3(0.212671f, 0.715160f, 0.072169f)); }
GPUGI_D float3 unpack_normal(float phi, float z) {  // UnpackNormal(vec2), helper.glsl:38-42
    float sinPhi = sqrtf(saturate((1.0f - z) * (1.0f + z)));
    float s, c;
    sincosf(phi, &s, &c);
    return f3(c * sinPhi, s * sinPhi, z);
}
GPUGI_D float3 unpack_normal_raw(float phi, float z) {  // UnpackNormal(float, float), helper.glsl:43-47
    float sinPhi = sqrtf(1.0f - z * z);
    float s, c;
    sincosf(phi, &s, &c);
    return f3(c * sinPhi, s * sinPhi, z);
}
GPUGI_D float2 pack_normal(float3 n) {
    return make_float2(n.x == 0.0f ? signf(n.y) * kPI / 2 : atan2f(n.y, n.x), n.z);
}

// GetTriangleHitInfo (scenedata.glsl:94-105): interpolated shading normal.
GPUGI_D float3 hit_normal(const DevScene& s, int4 tri, float u, float v, float2* texcoord) {
    if (kChecked && ((uint32_t)tri.x >= s.numVertices || (uint32_t)tri.y >= s.numVertices ||
                     (uint32_t)tri.z >= s.numVertices)) {
        raise_error(s.err, DEVERR_BOUNDS);
        if (texcoord) *texcoord = make_float2(0.0f, 0.0f);
        return make_float3(0.0f, 0.0f, 1.0f);
    }
    float4 a = __ldg(s.vinfo + tri.x), b = __ldg(s.vinfo + tri.y), c = __ldg(s.vinfo + tri.z);
    float w = 1.0f - (v + u);
    float3 n = unpack_normal(a.x, a.y) * w + unpack_normal(b.x, b.y) * u + unpack_normal(c.x, c.y) * v;
    if (texcoord) *texcoord = make_float2(a.z * w + b.z * u + c.z * v, a.w * w + b.w * u + c.w * v);
    return normalize(n);
}

GPUGI_D float avg_probability(float3 c) { return (c.x + c.y + c.z + kDIVISOR_EPSILON) / (3.0f + kDIVISOR_EPSILON); }
GPUGI_D float avg3(float3 c) { return (c.x + c.y + c.z) / 3.0f; }

GPUGI_D void decision_probabilities(const MaterialData& m, float3& preflect, float3& prefract, float3& pdiffuse) {
    preflect = m.Fresnel0;
    prefract = f3(1.0f) - saturate(preflect);
    pdiffuse = prefract * m.Opacity;
    prefract = prefract - pdiffuse;
}

// __SampleBSDF (materials.glsl:118-277). The reference's rejection loop is
// disabled (plausible = true), so exactly one lobe sample is drawn. With
// stopOnDiffuse (the Whitted shader's STOP_ON_DIFFUSE_BOUNCE) a diffuse
// decision sets throughput = (-1, 0, 0) and returns no direction.
GPUGI_D float3 sample_bsdf(float3 incident, const MaterialData& m, Rng& seed, float3 N, float3& throughput,
                           bool adjoint, float& pdf, bool stopOnDiffuse = false, bool* reflectedDiffuse = nullptr) {
    float cosTheta = dot(N, incident);
    float cosThetaAbs = saturate(fabsf(cosTheta));
    float3 rrDir = incident - (2.0f * cosTheta) * N;
    float2 rs = random2(seed);
    float3 preflect, prefract, pdiffuse;
    decision_probabilities(m, preflect, prefract, pdiffuse);
    float avgPReflect = avg_probability(preflect);
    float avgPRefract = avg_probability(prefract);
    float avgPDiffuse = avg3(pdiffuse);
    float3 pphong = preflect;
    float avgPPhong = avgPReflect;
    float decision = random01(seed);
    if (reflectedDiffuse) *reflectedDiffuse = avgPDiffuse > decision;  // SAMPLING_DECISION_OUTPUT
    if (avgPDiffuse > decision) {
        if (stopOnDiffuse) {
            throughput = f3(-1.0f, 0.0f, 0.0f);
            return f3(0.0f);
        }
        throughput *= (m.Diffuse * pdiffuse) / avgPDiffuse;
        if (cosTheta > 0.0f) N = -N;
        float3 U, V;
        create_onb(N, U, V);
        float3 outDir = sample_hemisphere_cosine(rs, U, V, N);
        pdf = saturate(dot(N, outDir)) / kPI;
        return outDir;
    } else if (avgPDiffuse + avgPRefract > decision) {
        pphong = prefract;
        avgPPhong = avgPRefract;
        float eta = cosTheta < 0.0f ? 1.0f / m.RefractionIndexAvg : m.RefractionIndexAvg;
        float etaSq = eta * eta;
        float sin2 = etaSq * (1.0f - cosTheta * cosTheta);
        if (sin2 < 1.0f) {
            rrDir = eta * incident + (signf(cosTheta) * (sqrtf(saturate(1.0f - sin2)) - eta * cosThetaAbs)) * N;
            if (!adjoint) throughput /= etaSq;
        }
    }
    rrDir = normalize(rrDir);
    float3 RU, RV;
    create_onb(rrDir, RU, RV);
    float3 outDir = sample_phong_lobe(rs, m.Reflectiveness.w, RU, RV, rrDir);
    if (!adjoint) throughput *= fabsf(dot(N, outDir)) / fabsf(dot(N, rrDir));
    float cosOut = fabsf(dot(outDir, rrDir));
    pdf = (m.Reflectiveness.w + 1.0f) / kPI_2 * powf(cosOut, m.Reflectiveness.w);
    throughput *= pphong / avgPPhong;
    return outDir;
}

// __BSDF (materials.glsl:306-391); stopOnDiffuse drops the refractive part
// (STOP_ON_DIFFUSE_BOUNCE, materials.glsl:355-358).
GPUGI_D float3 eval_bsdf(float3 incident, float3 excident, const MaterialData& m, float3 N, float& pdf, bool adjoint,
                         bool stopOnDiffuse = false) {
    float cosTheta = dot(N, incident);
    float cosThetaAbs = saturate(fabsf(cosTheta));
    float cosThetaOut = dot(N, excident);
    float3 preflect, prefract, pdiffuse;
    decision_probabilities(m, preflect, prefract, pdiffuse);
    const float exponent = m.Reflectiveness.w;
    float phongBrdf = (exponent + 1.0f) / (2 * kPI_2 * fabsf(cosThetaOut) + kDIVISOR_EPSILON);
    float phongPdf = (exponent + 1.0f) / kPI_2;
    float3 rrDir = normalize(incident - (2.0f * cosTheta) * N);
    float powN = powf(saturate(dot(rrDir, excident)), exponent);
    float brdfF = phongBrdf * powN;
    float pdfF = phongPdf * powN;
    float3 bsdf = preflect * brdfF;
    bsdf *= fabsf(cosThetaOut) / cosThetaAbs;
    pdf = avg_probability(preflect) * pdfF;
    if (cosTheta * cosThetaOut < 0.0f) {
        bsdf += pdiffuse * m.Diffuse / kPI;
        pdf += avg3(pdiffuse) * saturate(cosThetaOut) / kPI;
    }
    if (stopOnDiffuse) return bsdf;
    float eta = cosTheta < 0.0f ? 1.0f / m.RefractionIndexAvg : m.RefractionIndexAvg;
    float etaSq = eta * eta;
    float sin2 = etaSq * (1.0f - cosTheta * cosTheta);
    if (sin2 < 1.0f) {
        rrDir = normalize(eta * incident + (signf(cosTheta) * (sqrtf(saturate(1.0f - sin2)) - eta * cosThetaAbs)) * N);
        float powR = powf(saturate(dot(rrDir, excident)), exponent);
        brdfF = phongBrdf * powR;
        pdfF = phongPdf * powR;
        if (!adjoint) brdfF /= etaSq;
        brdfF *= fabsf(dot(N, excident)) / fabsf(dot(N, rrDir));
    }
    bsdf += prefract * brdfF;
    pdf += avg_probability(prefract) * pdfF;
    return bsdf;
}
GPUGI_D float3 adjoint_bsdf(float3 incident, float3 excident, const MaterialData& m, float3 N, float& pdf) {
    return eval_bsdf(-excident, -incident, m, N, pdf, true);
}
GPUGI_D float shading_corrected_out_dot_n(float3 inL, float3 toCam, float3 gN, float3 sN) {
    if (dot(inL, gN) * dot(inL, sN) < 0.0f || dot(toCam, gN) * dot(toCam, sN) < 0.0f) return 0.0f;
    return saturate(fabsf(dot(inL, sN) * dot(toCam, gN)) / fmaxf(fabsf(dot(inL, gN)), kDIVISOR_EPSILON));
}
GPUGI_D float shading_correction(float3 inDir, float3 outDir, float3 gN, float3 sN) {
    if (dot(inDir, gN) * dot(inDir, sN) < 0.0f || dot(outDir, gN) * dot(outDir, sN) < 0.0f) return 0.0f;
    return saturate(fabsf(dot(inDir, sN) * dot(outDir, gN)) /
                    fmaxf(fabsf(dot(inDir, gN) * dot(outDir, sN)), kDIVISOR_EPSILON));
}

GPUGI_D float mis_heuristic(float p) { return fminf(1e18f, p); }
GPUGI_D float distance_mis(float d) { return mis_heuristic(d * d); }

// Warp-aggregated append: one atomic per warp. Must be called by all 32 lanes.
GPUGI_D uint32_t warp_append(uint32_t* counter, bool want, uint32_t& slot) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned ballot = __ballot_sync(0xffffffffu, want);
    uint32_t base = 0;
    if (lane == 0 && ballot) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, 0);
    slot = base + (uint32_t)__popc(ballot & ((1u << lane) - 1u));
    return ballot;
}

}  // namespace gpugi
