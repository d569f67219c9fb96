// Wavefront renderers: PT, LT and BPT on the traversal kernels.
//
// The reference runs one megakernel invocation per pixel (pathtracer.comp,
// pathtracer_bidir.comp) or light particle (lighttracer.comp), with the path
// loop inside. Here every path's state lives in structure-of-arrays queues
// in HBM and each bounce is a sequence of kernels:
//
//   generate -> [ extend (closest hit) -> shade -> shadow (any hit) ] x depth
//
//  * extend/shadow are persistent walks that refill finished lanes (same
//    tests per ray as TraceRay/TraceRayAnyHit);
//  * shade evaluates the hit (emission, NEE or camera/light-cache connection,
//    BSDF sampling, Russian roulette) and appends the surviving paths and the
//    connection rays to the next queues with warp-ballot compaction (one
//    atomic per warp);
//  * contributions are added to the RGBA32F image with 16-byte vector float
//    atomics (red.global.add.v4.f32), optionally also in FP64;
//  * all kernels take their element counts from device memory, so a whole
//    render is a fixed launch sequence with no host round trip (graph-capturable).
//
// Per-path RNG streams, the order of RNG draws and all shading formulas are
// those of the shaders, so each estimator is the reference's.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "shade.cuh"
#include "trace.cuh"

// The passes' walkers walk a queue with 8-lane groups while it holds fewer
// rays than this many times the resident lanes, and a ray per lane otherwise.
#ifndef GPUGI_GROUP_BELOW_LANES
#define GPUGI_GROUP_BELOW_LANES 2u
#endif

namespace gpugi {

constexpr int kMaxDepth = 64;

struct PathSoA {
    float *ox, *oy, *oz, *dx, *dy, *dz, *tx, *ty, *tz, *lastP;
    uint32_t *seed, *pixel, *info;  // info: bit 0 = didNEE, bits 8..31 = sample (iteration) index
    uint32_t* job;                  // batched render: index of the path's job; BPT with the radiance
                                    // cache: float bits of the product of the path's MIS factors
};
struct HitSoA {
    int32_t* slot;
    float *t, *u, *v;
};
struct ShadowSoA {
    float *ox, *oy, *oz, *dx, *dy, *dz, *tmax, *cr, *cg, *cb;
    uint32_t* pixel;
    uint32_t* train;  // radiance-cache training vertex that also receives the contribution, or kNoTrain
    uint32_t* job;    // batched render: index of the ray's job
};
constexpr uint32_t kNoTrain = 0xFFFFFFFFu;
constexpr uint32_t kNoPixel = 0xFFFFFFFFu;  // a path that only trains the radiance cache: no splat

// Light-cache entry (bidirpathtracer/lightcache.glsl:1-16), 64 bytes.
struct CacheEntry {
    float4 fluxMat;    // flux.xyz, material index (int bits; -1 = light sample)
    float4 posN0;      // position.xyz, normal0 (packed phi)
    float4 tcN1Len;    // texcoord.xy, normal1 (cos theta; > 1.5 marks a point light), path length (int bits)
    float4 incident;   // incident direction packed (phi, z), unused, unused
};

struct Counters {
    uint32_t path[kMaxDepth + 2];
    uint32_t shadow[kMaxDepth + 2];
    unsigned long long extendWork[kMaxDepth + 2];
    unsigned long long shadowWork[kMaxDepth + 2];
    unsigned long long rays[2];  // closest-hit, any-hit rays traced
};

struct RenderConst {
    DevScene s;
    float3 camU, camV, camW, camPos;
    float pixelArea;
    int width, height, numPixels;
    int maxPathLength, rrStartDepth;
    uint32_t iteration, samples, sampleBase;  // sample s of this chunk = iteration sampleBase + s
    uint32_t pass;               // gpugi_pass (the batched wavefront shades each path by its job's pass)
    uint32_t rng;                // 1: PCG streams (default), 0: the reference's wanghash + xorshift32
    uint32_t numLightSamples;
    const float4* lightSamples;  // [samples][numLightSamples][2]
    float3 sky;
    int numRaysPerLightSample;
    uint32_t lightThreads;       // numLightSamples * numRaysPerLightSample
    float4* image;
    double* image64;
    CacheEntry* cache;
    uint32_t* cacheCount;        // [samples]
    uint32_t cacheCap;           // entries per sample
    Counters* cnt;
    uint32_t* err;
    // radiance cache (PT with NRC); unused by the other passes
    int nrcTerminateDepth;       // render paths query the cache at this vertex
    uint32_t nrcTrainThreshold;  // pixel hash below this: a training path
    int nrcTrainLength;          // self-training: training paths query the cache at this vertex (0: off)
    uint32_t nrcUnbiasedThreshold;  // training-path hash below this: never stops at the cache
    float nrcSpread;             // > 0: render paths stop once the path spread exceeds this x a0
    float* tvRec;                // training vertices: 16 floats {pos, dir, normal, albedo, T, pad}
    float* tvC;                  // training vertices: 3 floats, radiance accumulated after the vertex
    uint32_t* tvCount;           // vertices recorded per training path
    uint32_t* trainPaths;        // counter of training paths
    uint32_t trainCap;           // training paths the buffers hold
    float* queries;              // 12 floats per cache query
    float* qT;                   // 3 floats: throughput at the query
    uint32_t* qPixel;
    uint32_t* queryCount;
    uint32_t queryCap;
    // photon mapper; unused by the other passes
    uint32_t* pmMap;             // HashMap: {cell hash key, list head} per entry
    uint32_t pmMapSize;          // prime
    float4* pmPhotons;           // 2 x float4 per photon: {next, flux}, {position, packed direction}
    uint32_t* pmCount;
    uint32_t pmCap;
    float pmSpacing, pmRadiusSq; // HashGridSpacing, PhotonQueryRadiusSq
    int photonsPerSample;        // NumPhotonsPerLightSample
    // importon map light tracer: G-buffer of the first eye hits {position, packed normal .y}, packed normal .x
    float4* imGbuf;
    float* imGbufN0;
};

// ------------------------------------------------------------ accumulation
GPUGI_D void splat(const RenderConst& rc, uint32_t pixel, float3 c, float w = 0.0f) {
    if (!(c.x != 0.0f || c.y != 0.0f || c.z != 0.0f || w != 0.0f) || pixel == kNoPixel) return;
    atomicAdd(rc.image + pixel, make_float4(c.x, c.y, c.z, w));
    if (rc.image64) {
        atomicAdd(rc.image64 + 3 * (size_t)pixel, (double)c.x);
        atomicAdd(rc.image64 + 3 * (size_t)pixel + 1, (double)c.y);
        atomicAdd(rc.image64 + 3 * (size_t)pixel + 2, (double)c.z);
    }
}

GPUGI_D void store_path(const PathSoA& P, uint32_t i, float3 o, float3 d, float3 tp, Rng seed, uint32_t pixel,
                        uint32_t info, float lastP) {
    P.ox[i] = o.x; P.oy[i] = o.y; P.oz[i] = o.z;
    P.dx[i] = d.x; P.dy[i] = d.y; P.dz[i] = d.z;
    P.tx[i] = tp.x; P.ty[i] = tp.y; P.tz[i] = tp.z;
    P.seed[i] = seed.s; P.pixel[i] = pixel; P.info[i] = info; P.lastP[i] = lastP;
}
GPUGI_D void store_shadow(const ShadowSoA& Q, uint32_t i, float3 o, float3 d, float tmax, float3 c, uint32_t pixel,
                          uint32_t train = kNoTrain) {
    Q.train[i] = train;
    Q.ox[i] = o.x; Q.oy[i] = o.y; Q.oz[i] = o.z;
    Q.dx[i] = d.x; Q.dy[i] = d.y; Q.dz[i] = d.z;
    Q.tmax[i] = tmax; Q.cr[i] = c.x; Q.cg[i] = c.y; Q.cb[i] = c.z; Q.pixel[i] = pixel;
}

// Persistent refill loop shared by the extend and shadow kernels.
template <bool ANY_HIT, int BOUNDS, typename Load, typename Finish>
GPUGI_D void persistent_walks(const DevScene& s, uint32_t n, unsigned long long* work, uint32_t* err, Load load,
                              Finish finish, uint32_t stage) {
    extern __shared__ float4 s_top[];
    stage_top_nodes(s, s_top, stage);
    const unsigned lane = threadIdx.x & 31u;
    WalkState w;
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    while (true) {
        const bool need = !active && !exhausted;
        const unsigned needMask = __ballot_sync(0xffffffffu, need);
        if (needMask) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(work, (unsigned long long)__popc(needMask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need) {
                const unsigned long long my = base + (unsigned long long)__popc(needMask & ((1u << lane) - 1u));
                if (my < n) {
                    ray = (uint32_t)my;
                    float3 o, d;
                    float tmax;
                    load(ray, o, d, tmax);
                    walk_begin(w, s, o, d, tmax);
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active && walk_step<ANY_HIT, BOUNDS>(w, s, err, s_top, stage)) {
            finish(ray, w);
            active = false;
        }
    }
}

// Closest hits of the path queue. Queues shorter than groupBelow rays are
// walked by 8-lane groups (group_walks: a short queue leaves lanes idle, and
// groups shorten the longest walks); longer ones with one lane per ray (more
// rays in flight; top nodes staged in shared memory). The choice depends on
// the device-side count, so it costs no host round trip.
template <int BOUNDS>
__global__ void __launch_bounds__(128) k_extend(RenderConst rc, PathSoA A, HitSoA H, int depth, uint32_t stage,
                                                uint32_t groupBelow) {
    const uint32_t n = rc.cnt->path[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&rc.cnt->rays[0], (unsigned long long)n);
    auto load = [&](auto i, float3& o, float3& d, float& tmax) {
        o = make_float3(A.ox[i], A.oy[i], A.oz[i]);
        d = make_float3(A.dx[i], A.dy[i], A.dz[i]);
        tmax = kRAY_MAX;
    };
    if (n < groupBelow) {
        group_walks<false, BOUNDS, 8>(rc.s, n, &rc.cnt->extendWork[depth], rc.err, load,
                                      [&](uint64_t i, const GroupWalk& g) {
                                          H.slot[i] = g.slot;
                                          H.t[i] = g.len;
                                          H.u[i] = g.u;
                                          H.v[i] = g.v;
                                      });
    } else {
        persistent_walks<false, BOUNDS>(
            rc.s, n, &rc.cnt->extendWork[depth], rc.err, load,
            [&](uint32_t i, const WalkState& w) {
                H.slot[i] = w.slot;
                H.t[i] = w.len;
                H.u[i] = w.u;
                H.v[i] = w.v;
            },
            stage);
    }
}

// Shadow rays: unoccluded contributions are splatted (and added to their
// radiance-cache training vertex).
GPUGI_D void shadow_unoccluded(const RenderConst& rc, const ShadowSoA& Q, uint32_t i) {
    const float3 c = make_float3(Q.cr[i], Q.cg[i], Q.cb[i]);
    splat(rc, Q.pixel[i], c);
    const uint32_t tr = Q.train[i];
    if (tr != kNoTrain) {
        atomicAdd(rc.tvC + 3 * (size_t)tr, c.x);
        atomicAdd(rc.tvC + 3 * (size_t)tr + 1, c.y);
        atomicAdd(rc.tvC + 3 * (size_t)tr + 2, c.z);
    }
}

template <int BOUNDS>
__global__ void __launch_bounds__(128) k_shadow(RenderConst rc, ShadowSoA Q, int depth, uint32_t stage,
                                                uint32_t groupBelow) {
    const uint32_t n = rc.cnt->shadow[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&rc.cnt->rays[1], (unsigned long long)n);
    auto load = [&](auto i, float3& o, float3& d, float& tmax) {
        o = make_float3(Q.ox[i], Q.oy[i], Q.oz[i]);
        d = make_float3(Q.dx[i], Q.dy[i], Q.dz[i]);
        tmax = Q.tmax[i];
    };
    if (n < groupBelow) {
        group_walks<true, BOUNDS, 8>(rc.s, n, &rc.cnt->shadowWork[depth], rc.err, load,
                                     [&](uint64_t i, const GroupWalk& g) {
                                         if (g.slot < 0) shadow_unoccluded(rc, Q, (uint32_t)i);
                                     });
    } else {
        persistent_walks<true, BOUNDS>(
            rc.s, n, &rc.cnt->shadowWork[depth], rc.err, load,
            [&](uint32_t i, const WalkState& w) {
                if (w.slot < 0) shadow_unoccluded(rc, Q, i);
            },
            stage);
    }
}

// Launch shapes and launches of the walkers for a scene: group walks when the
// context's trace mode is 3 or 4, else lane walks with staged top nodes.
struct Walkers {
    int bounds = 0;  // node kind: 0 box, 1 ellipsoid, 2 oriented box
    uint32_t groupBelowE = 0, groupBelowS = 0;  // queue lengths below which groups walk
    WalkerLaunch LE, LS;
};

// ------------------------------------------------------------ generation
// Primary ray (pathtracer.comp:132-139) in exact IEEE operations, so camera
// rays, and with them the first hits, are bit-identical to the oracle's.
GPUGI_D float3 primary_direction(const RenderConst& rc, Rng& seed, int x, int y) {
    float2 r = random2(seed);
    const float sx = X::sub(X::mul(X::div(X::add(X::sub(r.x, 0.5f), (float)x), (float)rc.width), 2.0f), 1.0f);
    const float sy = X::sub(X::mul(X::div(X::add(X::sub(r.y, 0.5f), (float)y), (float)rc.height), 2.0f), 1.0f);
    return X::normalize(X::add3(X::add3(X::scale(sx, rc.camU), X::scale(sy, rc.camV)), rc.camW));
}

// pathtracer.comp:16-46 / pathtracer_bidir.comp:16-24: one camera path per
// pixel and iteration. BPT also counts the iteration in the alpha channel.
// The eye path of pixel pix in sample s at queue slot p (pathtracer.comp:37-46,
// pathtracer_bidir.comp:36-52; the bidirectional tracer counts the sample in
// alpha).
GPUGI_D void camera_path_start(const RenderConst& rc, const PathSoA& A, uint32_t p, uint32_t s, uint32_t pix,
                               bool bidir) {
    const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
    Rng seed = rng_init(rc.rng, rc.iteration + rc.sampleBase + s, pix);
    const float3 d = primary_direction(rc, seed, x, y);
    store_path(A, p, rc.camPos, d, f3(1.0f), seed, pix, s << 8, 1.0f);
    if (bidir) splat(rc, pix, f3(0.0f), 1.0f);
}

__global__ void k_camera_generate(RenderConst rc, PathSoA A, bool bidir) {
    const uint32_t total = rc.samples * (uint32_t)rc.numPixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x)
        camera_path_start(rc, A, p, p / (uint32_t)rc.numPixels, p % (uint32_t)rc.numPixels, bidir);
}

GPUGI_D void write_cache(const RenderConst& rc, uint32_t s, uint32_t k, float3 flux, int mat, float3 pos, float n0,
                         float n1, float2 tc, float2 incident, int pathLength) {
    CacheEntry e;
    e.fluxMat = make_float4(flux.x, flux.y, flux.z, __int_as_float(mat));
    e.posN0 = make_float4(pos.x, pos.y, pos.z, n0);
    e.tcN1Len = make_float4(tc.x, tc.y, n1, __int_as_float(pathLength));
    e.incident = make_float4(incident.x, incident.y, 0.0f, 0.0f);
    rc.cache[(size_t)s * rc.cacheCap + k] = e;
}

// lighttracer.comp:49-93: one particle per thread, numRaysPerLightSample
// particles per initial light sample. With a light cache (BPT) each thread
// first stores its own light sample (lighttracer.comp:56-61).
GPUGI_D void light_path_start(const RenderConst& rc, const PathSoA& A, uint32_t p, uint32_t s, uint32_t gid,
                              bool withCache) {
    Rng seed = rng_init(rc.rng, rc.iteration + rc.sampleBase + s, gid);
    const uint32_t li = gid / (uint32_t)rc.numRaysPerLightSample;
    const float4* ls = rc.lightSamples + 2 * ((size_t)s * rc.numLightSamples + li);
    const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
    if (withCache) {
        if (gid == 0) rc.cacheCount[s] = rc.lightThreads;  // resetcounter.comp
        write_cache(rc, s, gid, xyz(in1) / kPI_2 / (float)rc.numRaysPerLightSample, -1, xyz(pn0), pn0.w, in1.w,
                    make_float2(0.0f, 0.0f), pack_normal(f3(0.0f)), 0);
    }
    float3 tp = xyz(in1) * (kPI / (float)rc.numRaysPerLightSample);
    float3 d;
    if (in1.w > 1.5f) {
        d = sample_direction(random2(seed));
        tp *= 4.0f;
    } else {
        float3 n = unpack_normal(pn0.w, in1.w), U, V;
        create_onb(n, U, V);
        d = sample_hemisphere_cosine(random2(seed), U, V, n);
    }
    store_path(A, p, xyz(pn0), d, tp, seed, gid, s << 8, 1.0f);
}

__global__ void k_light_generate(RenderConst rc, PathSoA A, bool withCache) {
    const uint32_t total = rc.samples * rc.lightThreads;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x)
        light_path_start(rc, A, g, g / rc.lightThreads, g % rc.lightThreads, withCache);
}

// ------------------------------------------------------------ shading
struct Hit {
    bool valid;
    float3 pos, N;
    float2 tc;  // texture coordinate (GetTriangleHitInfo)
    int4 tri;
    MaterialData m;
    float t;
};

GPUGI_D Hit load_hit(const RenderConst& rc, const HitSoA& H, uint32_t k, float3 o, float3 d) {
    Hit h;
    const int32_t slot = H.slot[k];
    h.valid = slot >= 0;
    if (!h.valid) return h;
    h.t = H.t[k];
    h.pos = X::add3(o, X::scale(h.t, d));  // ray.Origin + rayHit * ray.Direction, uncontracted
    h.tri = __ldg(rc.s.slots + slot);
    h.N = hit_normal(rc.s, h.tri, H.u[k], H.v[k], &h.tc);
    h.m = load_material(rc.s, h.tri.w, h.tc);
    return h;
}

// EstimateDirectLight (lightsource.glsl:3-93), split: returns the radiance
// assuming visibility and the shadow ray that decides it.
GPUGI_D bool direct_light(const RenderConst& rc, uint32_t s, float3 pos, float3 N, uint32_t idx, float3 viewDir,
                          const MaterialData& m, bool sampleAreaLights, float3& radiance, float3& ro, float3& rd,
                          float& rlen, bool stopOnDiffuse = false) {
    const float4* ls = rc.lightSamples + 2 * ((size_t)s * rc.numLightSamples + idx);
    const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
    float pdf;
    if (in1.w > 2.5f) {  // directional light (addition)
        rd = xyz(pn0);
        float cosS = saturate(dot(rd, N));
        if (cosS <= 0.0f) return false;
        radiance = (cosS * xyz(in1)) * eval_bsdf(viewDir, rd, m, N, pdf, false, stopOnDiffuse);
        ro = kRAY_HIT_EPSILON * rd + pos;
        rlen = kRAY_MAX;
        return true;
    }
    float3 L = xyz(pn0) - pos;
    const float distSq = dot(L, L) + kDIVISOR_EPSILON;
    const float dist = sqrtf(distSq);
    L /= dist;
    const float cosS = saturate(dot(L, N));
    if (cosS <= 0.0f) return false;
    if (in1.w > 1.5f) {
        radiance = ((cosS / distSq) * xyz(in1)) * eval_bsdf(viewDir, L, m, N, pdf, false, stopOnDiffuse);
    } else if (sampleAreaLights) {
        const float f = saturate(dot(unpack_normal(pn0.w, in1.w), -L));
        if (!(f > 0.0f)) return false;
        radiance = ((cosS / distSq) * (xyz(in1) * f)) * eval_bsdf(viewDir, L, m, N, pdf, false, stopOnDiffuse);
    } else {
        return false;
    }
    ro = kRAY_HIT_EPSILON * L + pos;
    rd = L;
    rlen = dist - kRAY_HIT_EPSILON * 2;
    return true;
}

// Russian roulette (pathtracer.comp:99-104); rrStartDepth > 0 delays it.
GPUGI_D bool roulette(const RenderConst& rc, int depth, float3 throughput, float3& tp, Rng& seed) {
    if (depth < rc.rrStartDepth) return true;
    const float p = saturate(luminance(throughput));
    if (random01(seed) >= p) return false;
    tp /= p;
    return true;
}

// Warp-uniform grid-stride loop over a device count: every lane of a warp
// runs the body together so ballots see all 32 lanes.
#define WARP_LOOP(n, k, valid)                                                                                   \
    for (uint32_t base_ = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u, k = base_ + (threadIdx.x & 31u);     \
         base_ < (n); base_ += gridDim.x * blockDim.x, k = base_ + (threadIdx.x & 31u))                         \
        for (bool valid = k < (n), once_ = true; once_; once_ = false)

// pathtracer.comp:48-105, one bounce of one path: the per-lane part of the
// PT shade kernels (the queue appends are warp-wide and follow).
struct PtLane {
    bool survive = false, shadow = false;
    float3 o, d, tp, sro, srd, contrib;
    float srl = 0.0f;
    Rng seed{0, 0};
    uint32_t pixel = 0, info = 0;
};

GPUGI_D void pt_shade_lane(const RenderConst& rc, const PathSoA& A, const HitSoA& H, uint32_t k, int depth,
                           PtLane& L) {
    const float lightSampleWeight = (float)rc.numLightSamples;
    L.o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
    L.d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
    L.tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
    L.seed = Rng{A.seed[k], rc.rng};
    L.pixel = A.pixel[k];
    L.info = A.info[k];
    Hit h = load_hit(rc, H, k, L.o, L.d);
    if (!h.valid) {
        splat(rc, L.pixel, L.tp * rc.sky);
        return;
    }
    L.o = h.pos;
    if (!(L.info & 1u)) splat(rc, L.pixel, L.tp * h.m.Emissivity);
    const bool didNEE = h.m.Reflectiveness.w < 500.0f;
    L.info = (L.info & ~1u) | (didNEE ? 1u : 0u);
    const uint32_t li = random_uint(L.seed) % rc.numLightSamples;
    float3 rad;
    if (direct_light(rc, L.info >> 8, L.o, h.N, li, L.d, h.m, didNEE, rad, L.sro, L.srd, L.srl)) {
        L.contrib = rad * L.tp * lightSampleWeight;
        L.shadow = L.contrib.x != 0.0f || L.contrib.y != 0.0f || L.contrib.z != 0.0f;
    }
    float3 thr = f3(1.0f);
    float pdf;
    L.d = sample_bsdf(L.d, h.m, L.seed, h.N, thr, false, pdf);
    L.o = L.o + L.d * kRAY_HIT_EPSILON;
    L.tp *= thr;
    L.survive = roulette(rc, depth, thr, L.tp, L.seed) && depth + 1 < rc.maxPathLength;
}

__global__ void __launch_bounds__(128) k_pt_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                  int depth) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        PtLane L;
        if (valid) pt_shade_lane(rc, A, H, k, depth, L);
        uint32_t qs, qb;
        warp_append(&rc.cnt->shadow[depth], L.shadow, qs);
        if (L.shadow) store_shadow(Q, qs, L.sro, L.srd, L.srl, L.contrib, L.pixel);
        warp_append(&rc.cnt->path[depth + 1], L.survive, qb);
        if (L.survive) store_path(B, qb, L.o, L.d, L.tp, L.seed, L.pixel, L.info, 1.0f);
    }
}

// ProjectToScreen (screenreproject.glsl:248-420) with the box filter: the
// splat and the camera visibility ray, or false when the point does not
// project onto the image.
GPUGI_D bool project_to_screen(const RenderConst& rc, float3 pos, float3 inDir, float3 gN, float3 sN,
                               const MaterialData& m, float3 tp, bool computeMIS, float3& ro, float3& rd, float& rl,
                               float3& color, uint32_t& pixel) {
    float3 cd = rc.camPos - pos;
    const float camViewDotRay = -dot(rc.camW, cd);
    if (!(camViewDotRay > 0.0f)) return false;
    float sx = -dot(rc.camU, cd) / camViewDotRay, sy = -dot(rc.camV, cd) / camViewDotRay;
    sx /= dot(rc.camU, rc.camU);
    sy /= dot(rc.camV, rc.camV);
    if (!(sx >= -1.0f && sx < 1.0f && sy > -1.0f && sy <= 1.0f)) return false;
    const float distSq = dot(cd, cd);
    const float dist = sqrtf(distSq);
    cd /= dist;
    const int px = (int)rintf((sx * 0.5f + 0.5f) * (float)rc.width);
    const int py = (int)rintf((sy * 0.5f + 0.5f) * (float)rc.height);
    if (px < 0 || py < 0 || px >= rc.width || py >= rc.height) return false;  // image atomics drop OOB
    const float cosAtCamera = saturate(camViewDotRay / dist);
    const float fluxToIrradiance = shading_corrected_out_dot_n(inDir, cd, gN, sN) /
                                   (cosAtCamera * cosAtCamera * cosAtCamera * rc.pixelArea * distSq);
    float pdf;
    float3 bsdf = adjoint_bsdf(inDir, cd, m, sN, pdf);
    if (computeMIS) {
        const float e2l = 1.0f;  // InitialMIS
        bsdf *= e2l / fmaxf(mis_heuristic(pdf) + e2l, kDIVISOR_EPSILON);
    }
    color = tp * fluxToIrradiance * bsdf;
    if (!(color.x != 0.0f || color.y != 0.0f || color.z != 0.0f)) return false;
    ro = cd * kRAY_HIT_EPSILON + pos;
    rd = cd;
    rl = dist;
    pixel = (uint32_t)(py * rc.width + px);
    return true;
}

// lighttracer.comp:95-192, one bounce of one particle (with SAVE_LIGHT_CACHE
// when withCache): the per-lane part of the light-shade kernels. The camera
// connection goes to pixel; the particle keeps gid.
struct LightLane {
    bool survive = false, shadow = false;
    float3 o, d, tp, sro, srd, color;
    float srl = 0.0f;
    Rng seed{0, 0};
    uint32_t pixel = 0, info = 0, gid = 0;
};

GPUGI_D void light_shade_lane(const RenderConst& rc, const PathSoA& A, const HitSoA& H, uint32_t k, int depth,
                              bool withCache, LightLane& L) {
    L.o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
    L.d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
    L.tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
    L.seed = Rng{A.seed[k], rc.rng};
    L.gid = A.pixel[k];
    L.info = A.info[k];
    const int32_t slot = H.slot[k];
    if (slot < 0) return;
    const float t = H.t[k];
    const float4 rec = __ldg(rc.s.tris + 3 * (size_t)slot + 2);
    const float3 gN = make_float3(rec.y, rec.z, rec.w);  // cross(e1, e0), not normalised
    L.o = L.o + t * L.d;
    const int4 tri = __ldg(rc.s.slots + slot);
    float2 tc;
    const float3 sN = hit_normal(rc.s, tri, H.u[k], H.v[k], &tc);
    const MaterialData m = load_material(rc.s, tri.w, tc);
    const uint32_t s = L.info >> 8;
    if (withCache && m.Reflectiveness.w < 100.0f) {
        const uint32_t e = atomicAdd(rc.cacheCount + s, 1u);
        if (e < rc.cacheCap) {
            float2 pn = pack_normal(sN);
            write_cache(rc, s, e, L.tp, tri.w, L.o, pn.x, pn.y, tc, pack_normal(L.d), depth + 1);
        } else {
            raise_error(rc.err, DEVERR_QUEUE_OVERFLOW);
        }
    }
    L.shadow = project_to_screen(rc, L.o, L.d, gN, sN, m, L.tp, withCache, L.sro, L.srd, L.srl, L.color, L.pixel);
    float3 thr = f3(1.0f);
    float pdf;
    const float3 nd = sample_bsdf(L.d, m, L.seed, sN, thr, true, pdf);
    thr *= shading_correction(L.d, nd, gN, sN);
    L.tp *= thr;
    L.survive = roulette(rc, depth, thr, L.tp, L.seed) && depth + 1 < rc.maxPathLength;
    L.d = nd;
    L.o = L.o + L.d * kRAY_HIT_EPSILON;
}

__global__ void __launch_bounds__(128) k_light_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                     int depth, bool withCache) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        LightLane L;
        if (valid) light_shade_lane(rc, A, H, k, depth, withCache, L);
        uint32_t qs, qb;
        warp_append(&rc.cnt->shadow[depth], L.shadow, qs);
        if (L.shadow) store_shadow(Q, qs, L.sro, L.srd, L.srl, L.color, L.pixel);
        warp_append(&rc.cnt->path[depth + 1], L.survive, qb);
        if (L.survive) store_path(B, qb, L.o, L.d, L.tp, L.seed, L.gid, L.info, 1.0f);
    }
}

// showlightcaches.comp:9-65 without its visibility test: the camera
// connection of light sample i (sample-major), or false when the sample has
// no position or does not project onto the image. The caller splats color at
// pixel when the segment ro + [0, rl] rd is unoccluded.
GPUGI_D bool light_sample_view(const RenderConst& rc, uint32_t i, float3& ro, float3& rd, float& rl, float3& color,
                               uint32_t& pixel) {
    const float4* ls = rc.lightSamples + 2 * (size_t)i;
    const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
    if (in1.w > 2.5f) return false;  // directional samples have no position
    float3 cd = rc.camPos - xyz(pn0);
    const float camViewDotRay = -dot(rc.camW, cd);
    if (!(camViewDotRay > 0.0f)) return false;
    float sx = -dot(rc.camU, cd) / camViewDotRay, sy = -dot(rc.camV, cd) / camViewDotRay;
    sx /= dot(rc.camU, rc.camU);
    sy /= dot(rc.camV, rc.camV);
    if (!(sx >= -1.0f && sx < 1.0f && sy > -1.0f && sy <= 1.0f)) return false;
    const int px = (int)((sx * 0.5f + 0.5f) * (float)rc.width), py = (int)((sy * 0.5f + 0.5f) * (float)rc.height);
    if (px < 0 || py < 0 || px >= rc.width || py >= rc.height) return false;
    const float distSq = dot(cd, cd);
    const float dist = sqrtf(distSq);
    cd /= dist;
    const float3 n = unpack_normal(pn0.w, in1.w);
    const float cosTheta = dot(n, cd);
    const float cosAtCamera = saturate(camViewDotRay / dist);
    const float i2r = cosTheta / (kPI_2 * cosAtCamera * cosAtCamera * cosAtCamera * rc.pixelArea * distSq);
    ro = cd * kRAY_HIT_EPSILON + xyz(pn0);
    rd = cd;
    rl = dist;
    color = xyz(in1) * i2r;
    pixel = (uint32_t)(py * rc.width + px);
    return true;
}

// showlightcaches.comp:9-65: light samples seen directly by the camera.
template <int BOUNDS>
__global__ void k_show_light_samples(RenderConst rc) {
    const uint32_t total = rc.samples * rc.numLightSamples;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        float3 ro, rd, color;
        float rl;
        uint32_t pixel;
        if (!light_sample_view(rc, i, ro, rd, rl, color, pixel)) continue;
        TraceResult r = trace_ray<true, BOUNDS>(rc.s, ro, rd, rl, rc.err);
        if (r.slot < 0) splat(rc, pixel, color);
    }
}

// pathtracer_bidir.comp:54-245, one bounce of one eye path: the per-lane
// part of the BPT shade kernels. connectCap bounds the length of the paths
// formed by light-cache connections (maxPathLength in the reference). With
// the radiance cache (terminateDepth >= 0) the path stops at vertex
// terminateDepth after its emission term and queries the cache there with
// its throughput divided by the product of the MIS factors applied so far
// (kept in the job column as float bits).
struct BptLane {
    bool survive = false, shadow = false, query = false;
    float3 o, d, tp, sro, srd, contrib, qN, qAlbedo, qT;
    float srl = 0.0f, lastP = 1.0f, misProd = 1.0f;
    Rng seed{0, 0};
    uint32_t pixel = 0, info = 0;
};

GPUGI_D void bpt_shade_lane(const RenderConst& rc, const PathSoA& A, const HitSoA& H, uint32_t k, int depth,
                            int connectCap, int terminateDepth, BptLane& L) {
    L.o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
    L.d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
    L.tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
    L.seed = Rng{A.seed[k], rc.rng};
    L.pixel = A.pixel[k];
    L.info = A.info[k];
    L.lastP = A.lastP[k];
    if (terminateDepth >= 0) L.misProd = __uint_as_float(A.job[k]);
    float3& o = L.o;
    float3& d = L.d;
    float3& tp = L.tp;
    Rng& seed = L.seed;
    const float lastP = L.lastP;
    Hit h = load_hit(rc, H, k, o, d);
    if (!h.valid) {
        splat(rc, L.pixel, tp * rc.sky);
        return;
    }
    const uint32_t s = L.info >> 8;
    o = h.pos;
    const float rayHit = h.t;
    const float incCos = saturate(-dot(h.N, d));
    const float cLE = distance_mis(rayHit) * mis_heuristic(incCos / kPI);
    float mis = depth == 0 ? 1.0f : lastP / fmaxf(lastP + cLE, kDIVISOR_EPSILON);
    splat(rc, L.pixel, mis * tp * h.m.Emissivity);
    if (depth == terminateDepth) {
        L.query = true;
        L.qN = h.N;
        L.qAlbedo = h.m.Diffuse;
        L.qT = L.misProd > 0.0f ? tp / L.misProd : f3(0.0f);
        return;
    }
    const uint32_t actual = min(rc.cacheCount[s], rc.cacheCap);
    if (actual > 0) {
        const uint32_t li = random_uint(seed) % actual;
        const CacheEntry* ep = rc.cache + (size_t)s * rc.cacheCap + li;
        const float4 e0 = ep->fluxMat, e1 = ep->posN0, e2 = ep->tcN1Len, e3 = ep->incident;
        const int pathLength = __float_as_int(e2.w) + depth + 1;
        if (pathLength <= connectCap) {
            float3 Ld = xyz(e1) - o;
            const float lightDistSq = dot(Ld, Ld);
            const float lightDist = sqrtf(lightDistSq);
            Ld /= fmaxf(lightDist, kDIVISOR_EPSILON);
            float3 lN = f3(0.0f, 1.0f, 0.0f);
            float cosLight = 0.0f;
            const float cosCamera = fabsf(dot(Ld, h.N));
            const bool lambertian = e2.z < 1.5f;
            if (lambertian) {
                lN = unpack_normal_raw(e1.w, e2.z);
                cosLight = fabsf(dot(Ld, lN));
            }
            float pdf;
            const float3 bsdf = eval_bsdf(d, Ld, h.m, h.N, pdf, false);
            float cEL = mis_heuristic(pdf);
            if (depth > 0) {
                cEL *= distance_mis(rayHit);
                mis = lastP / fmaxf(lastP + cEL, kDIVISOR_EPSILON);
                if (h.m.Reflectiveness.w >= 100.0f) mis = 1.0f;
            } else {
                mis = cEL / fmaxf(lastP + cEL, kDIVISOR_EPSILON);
            }
            const float3 flux = xyz(e0);
            const int lmat = __float_as_int(e0.w);
            float misLight = 1.0f;
            float3 intensity;
            if (lambertian) {
                float cLtoE;
                if (lmat != -1) {
                    const MaterialData lm = load_material(rc.s, lmat, make_float2(e2.x, e2.y));
                    const float3 inc = unpack_normal(e3.x, e3.y);
                    const float3 lb = adjoint_bsdf(Ld, -inc, lm, lN, pdf);
                    intensity = flux * lb * cosLight;
                    cLtoE = mis_heuristic(pdf) * distance_mis(lightDist);
                } else {
                    intensity = flux * (cosLight * kPI_2);
                    cLtoE = mis_heuristic(cosLight / kPI) * distance_mis(lightDist);
                }
                misLight = cLtoE / fmaxf(cLtoE + cEL, kDIVISOR_EPSILON);
            } else {
                intensity = flux * kPI_2;
            }
            mis *= misLight;
            const float3 irr = (mis * (float)actual * cosCamera / lightDistSq) * intensity;
            L.contrib = irr * tp * bsdf;
            L.shadow = L.contrib.x != 0.0f || L.contrib.y != 0.0f || L.contrib.z != 0.0f;
            L.sro = kRAY_HIT_EPSILON * Ld + o;
            L.srd = Ld;
            L.srl = lightDist - kRAY_HIT_EPSILON * 2;
        }
    }
    float3 thr = f3(1.0f);
    float samplePDF;
    d = sample_bsdf(d, h.m, seed, h.N, thr, false, samplePDF);
    o = o + d * kRAY_HIT_EPSILON;
    tp *= thr;
    L.survive = roulette(rc, depth, thr, tp, seed) && depth + 1 < rc.maxPathLength;
    float rcp = mis_heuristic(samplePDF);
    if (depth == 0) {
        mis = rcp / fmaxf(rcp + lastP, kDIVISOR_EPSILON);
    } else {
        const float dm = distance_mis(rayHit);
        rcp *= dm;
        mis = lastP / fmaxf(lastP + dm * rcp, kDIVISOR_EPSILON);
        if (h.m.Reflectiveness.w >= 100.0f) mis = 1.0f;
    }
    tp *= mis;
    L.misProd *= mis;
    L.lastP = rcp;
}

__global__ void __launch_bounds__(128) k_bpt_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                   int depth) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        BptLane L;
        if (valid) bpt_shade_lane(rc, A, H, k, depth, rc.maxPathLength, -1, L);
        uint32_t qs, qb;
        warp_append(&rc.cnt->shadow[depth], L.shadow, qs);
        if (L.shadow) store_shadow(Q, qs, L.sro, L.srd, L.srl, L.contrib, L.pixel);
        warp_append(&rc.cnt->path[depth + 1], L.survive, qb);
        if (L.survive) store_path(B, qb, L.o, L.d, L.tp, L.seed, L.pixel, L.info, L.lastP);
    }
}

// ------------------------------------------------------------ Whitted
// whittedraytracer.comp:14-30: one path per pixel and iteration. The seed is
// InitCoherentRandomSeed (random.glsl:23-28): the same stream for every
// pixel of a frame; the pixel jitter has no -0.5 offset. The iteration is
// counted in alpha (the shader writes vec4(color, 1)).
__global__ void k_whitted_generate(RenderConst rc, PathSoA A) {
    const uint32_t total = rc.samples * (uint32_t)rc.numPixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        const uint32_t s = p / (uint32_t)rc.numPixels, pix = p % (uint32_t)rc.numPixels;
        const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
        Rng seed = rng_init_coherent(rc.rng, rc.iteration + rc.sampleBase + s);
        const float2 r = random2(seed);
        const float sx = X::sub(X::mul(X::div(X::add(r.x, (float)x), (float)rc.width), 2.0f), 1.0f);
        const float sy = X::sub(X::mul(X::div(X::add(r.y, (float)y), (float)rc.height), 2.0f), 1.0f);
        const float3 d = X::normalize(X::add3(X::add3(X::scale(sx, rc.camU), X::scale(sy, rc.camV)), rc.camW));
        store_path(A, p, rc.camPos, d, f3(1.0f), seed, pix, s << 8, 1.0f);
        splat(rc, pix, f3(0.0f), 1.0f);
    }
}

// whittedraytracer.comp:44-110, one bounce: emission of every hit; a
// specular or glossy decision continues the path with a colour-shift
// throughput; the first diffuse decision ends it with NUM_LIGHT_SAMPLES = 2
// NEE samples (EstimateDirectLight with the BSDF of STOP_ON_DIFFUSE_BOUNCE)
// weighted NumInitialLightSamples / 2 / luminance(pdiffuse).
__global__ void __launch_bounds__(128) k_whitted_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                       int depth) {
    const uint32_t n = rc.cnt->path[depth];
    const float lightSampleWeight = (float)rc.numLightSamples / 2.0f;
    WARP_LOOP(n, k, valid) {
        bool survive = false, shadow[2] = {false, false};
        float3 o, d, tp, sro[2], srd[2], contrib[2];
        float srl[2] = {0.0f, 0.0f};
        Rng seed{0, 0};
    uint32_t pixel = 0, info = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = Rng{A.seed[k], rc.rng};
            pixel = A.pixel[k];
            info = A.info[k];
            Hit h = load_hit(rc, H, k, o, d);
            if (!h.valid) {
                splat(rc, pixel, tp * rc.sky);
            } else {
                o = h.pos;
                splat(rc, pixel, tp * h.m.Emissivity);
                float3 preflect, prefract, pdiffuse;
                decision_probabilities(h.m, preflect, prefract, pdiffuse);
                const float pdiffuseAvg = luminance(pdiffuse);
                float3 thr = f3(1.0f);
                float pdf;
                const float3 nd = sample_bsdf(d, h.m, seed, h.N, thr, false, pdf, true);
                if (thr.x == -1.0f) {
#pragma unroll
                    for (int l = 0; l < 2; ++l) {
                        const uint32_t li = random_uint(seed) % rc.numLightSamples;
                        float3 rad;
                        if (direct_light(rc, info >> 8, o, h.N, li, d, h.m, true, rad, sro[l], srd[l], srl[l], true)) {
                            contrib[l] = rad * tp * (lightSampleWeight / (pdiffuseAvg + kDIVISOR_EPSILON));
                            shadow[l] = contrib[l].x != 0.0f || contrib[l].y != 0.0f || contrib[l].z != 0.0f;
                        }
                    }
                } else {
                    d = nd;
                    o = o + d * kRAY_HIT_EPSILON;
                    tp *= thr / (luminance(thr) + kDIVISOR_EPSILON);
                    survive = depth + 1 < rc.maxPathLength;
                }
            }
        }
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            uint32_t qs;
            warp_append(&rc.cnt->shadow[depth], shadow[l], qs);
            if (shadow[l]) store_shadow(Q, qs, sro[l], srd[l], srl[l], contrib[l], pixel);
        }
        uint32_t qb;
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, pixel, info, 1.0f);
    }
}

// ------------------------------------------------------------ photon mapper
// photonmapper/photondistribution.comp, photonmapper/gather.comp and the
// lossless hash grid of maps/hashmap.glsl + maps/grid.glsl: photons are
// stored at diffuse decisions in a linked list per grid cell (the list
// heads sit in an open-addressed table with quadratic probing), and eye
// paths gather the photons of 2x2x2 cells at their first diffuse decision.

GPUGI_D uint32_t pm_cell_hash(int x, int y, int z) {  // gridCellHash
    uint32_t h = ((uint32_t)x & 0x7FFu) | (((uint32_t)y & 0x3FFu) << 11) | (((uint32_t)z & 0x7FFu) << 21);
    return xorshift32(h);
}
GPUGI_D uint32_t pm_snorm16(float v) {  // packSnorm2x16 component, ties to even
    return (uint32_t)(uint16_t)(int16_t)rintf(fminf(fmaxf(v, -1.0f), 1.0f) * 32767.0f);
}
GPUGI_D uint32_t pack_normal32(float3 n) {  // PackNormal32 (helper.glsl:67-70)
    const float px = n.x == 0.0f ? signf(n.y) / 2.0f : atan2f(n.y, n.x) / kPI;
    return pm_snorm16(px) | (pm_snorm16(n.z) << 16);
}
GPUGI_D float3 unpack_normal32(uint32_t p) {  // UnpackNormal(uint) (helper.glsl:71-76)
    auto u = [](uint32_t b) { return fminf(fmaxf((float)(int16_t)(uint16_t)b / 32767.0f, -1.0f), 1.0f); };
    return unpack_normal(u(p & 0xFFFFu) * kPI, u(p >> 16));
}

// insertToHashGrid (maps/hashmap.glsl:31-59) of a photon at the end of the
// photon array; a full array or table drops the photon and raises the
// queue-overflow bit (the reference writes past its buffer instead).
GPUGI_D void store_photon(const RenderConst& rc, float3 pos, float3 dir, float3 flux) {
    const uint32_t idx = atomicAdd(rc.pmCount, 1u);
    if (idx >= rc.pmCap) {
        raise_error(rc.err, DEVERR_QUEUE_OVERFLOW);
        return;
    }
    const int cx = (int)ceilf(X::div(pos.x, rc.pmSpacing)), cy = (int)ceilf(X::div(pos.y, rc.pmSpacing)),
              cz = (int)ceilf(X::div(pos.z, rc.pmSpacing));
    const uint32_t hash = pm_cell_hash(cx, cy, cz);
    float4* rec = rc.pmPhotons + 2 * (size_t)idx;
    rec[1] = make_float4(pos.x, pos.y, pos.z, __uint_as_float(pack_normal32(dir)));
    uint32_t i = hash % rc.pmMapSize, step = 1;
    for (uint32_t probe = 0; probe < rc.pmMapSize; ++probe) {
        const uint32_t key = atomicCAS(rc.pmMap + 2 * (size_t)i, 0xFFFFFFFFu, hash);
        if (key == hash || key == 0xFFFFFFFFu) {
            const uint32_t next = atomicExch(rc.pmMap + 2 * (size_t)i + 1, idx);
            rec[0] = make_float4(__uint_as_float(next), flux.x, flux.y, flux.z);
            return;
        }
        i = (uint32_t)(((uint64_t)i + step * 2 + 1) % rc.pmMapSize);  // quadratic probing
        ++step;
    }
    raise_error(rc.err, DEVERR_QUEUE_OVERFLOW);
}

// findFirst (maps/hashmap.glsl:61-90): list head of a cell or 0xFFFFFFFF.
GPUGI_D uint32_t pm_find(const RenderConst& rc, uint32_t hash) {
    uint32_t i = hash % rc.pmMapSize, step = 1;
    for (uint32_t probe = 0; probe < rc.pmMapSize; ++probe) {
        const uint2 e = __ldg(reinterpret_cast<const uint2*>(rc.pmMap) + i);
        if (e.x == 0xFFFFFFFFu) return 0xFFFFFFFFu;
        if (e.x == hash) return e.y;
        i = (uint32_t)(((uint64_t)i + step * 2 + 1) % rc.pmMapSize);
        ++step;
    }
    return 0xFFFFFFFFu;
}

// photondistribution.comp:10-32: photonsPerSample photons per light sample.
__global__ void k_photon_generate(RenderConst rc, PathSoA A) {
    const uint32_t total = rc.numLightSamples * (uint32_t)rc.photonsPerSample;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        Rng seed = rng_init(rc.rng, rc.iteration + rc.sampleBase, g);
        const uint32_t li = g / (uint32_t)rc.photonsPerSample;
        const float4* ls = rc.lightSamples + 2 * (size_t)li;
        const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
        float3 tp = xyz(in1) * (kPI / (float)rc.photonsPerSample);
        float3 d;
        if (in1.w > 1.0f) {
            d = sample_direction(random2(seed));
            tp *= 4.0f;
        } else {
            const float3 n = unpack_normal(pn0.w, in1.w);
            float3 U, V;
            create_onb(n, U, V);
            d = sample_hemisphere_cosine(random2(seed), U, V, n);
        }
        store_path(A, g, xyz(pn0), d, tp, seed, g, in1.w > 1.0f ? 1u : 0u, 1.0f);  // bit 0: left a point light
    }
}

// photondistribution.comp:34-105, one bounce: the photon is stored when the
// adjoint BSDF sample decides for diffuse reflection, then continues (with
// the photon mapper's Russian roulette, luminance + 0.02).
__global__ void __launch_bounds__(128) k_photon_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, int depth) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        bool survive = false;
        float3 o, d, tp;
        Rng seed{0, 0};
    uint32_t gid = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = Rng{A.seed[k], rc.rng};
            gid = A.pixel[k];
            const int32_t slot = H.slot[k];
            if (slot >= 0) {
                const float4 rec = __ldg(rc.s.tris + 3 * (size_t)slot + 2);
                const float3 gN = make_float3(rec.y, rec.z, rec.w);  // cross(e1, e0), not normalised
                o = X::add3(o, X::scale(H.t[k], d));
                const int4 tri = __ldg(rc.s.slots + slot);
                float2 tc;
                const float3 sN = hit_normal(rc.s, tri, H.u[k], H.v[k], &tc);
                const MaterialData m = load_material(rc.s, tri.w, tc);
                float3 thr = f3(1.0f);
                float pdf;
                bool diffuse = false;
                const float3 nd = sample_bsdf(d, m, seed, sN, thr, true, pdf, false, &diffuse);
                if (diffuse) store_photon(rc, o, d, tp);
                thr *= shading_correction(d, nd, gN, sN);
                tp *= thr;
                survive = depth + 1 < rc.maxPathLength;
                if (survive && depth >= rc.rrStartDepth) {
                    const float p = saturate(luminance(thr) + 0.02f);
                    if (random01(seed) >= p) survive = false;
                    else tp /= p;
                }
                d = nd;
                o = o + d * kRAY_HIT_EPSILON;
            }
        }
        uint32_t qb;
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, gid, 0u, 1.0f);
    }
}

// gather.comp:38-50: one eye path per pixel (jitter without -0.5), the
// iteration counted in alpha.
__global__ void k_pm_generate(RenderConst rc, PathSoA A) {
    const uint32_t total = (uint32_t)rc.numPixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < total; pix += gridDim.x * blockDim.x) {
        const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
        Rng seed = rng_init(rc.rng, rc.iteration + rc.sampleBase, pix);
        const float2 r = random2(seed);
        const float sx = X::sub(X::mul(X::div(X::add(r.x, (float)x), (float)rc.width), 2.0f), 1.0f);
        const float sy = X::sub(X::mul(X::div(X::add(r.y, (float)y), (float)rc.height), 2.0f), 1.0f);
        const float3 d = X::normalize(X::add3(X::add3(X::scale(sx, rc.camU), X::scale(sy, rc.camV)), rc.camW));
        store_path(A, pix, rc.camPos, d, f3(1.0f), seed, pix, 0u, 1.0f);
        splat(rc, pix, f3(0.0f), 1.0f);
    }
}

// gather.comp:51-128, one bounce: emission of every hit; at the first
// diffuse decision the photons of the 2x2x2 cells from round(pos / spacing)
// are gathered (irradianceEstimate, gather.comp:11-36) and the path ends;
// otherwise it continues with the +0.02 roulette.
__global__ void __launch_bounds__(128) k_pm_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, int depth) {
    const uint32_t n = rc.cnt->path[depth];
    const float kernel = 1.0f / (kPI * rc.pmRadiusSq);
    WARP_LOOP(n, k, valid) {
        bool survive = false;
        float3 o, d, tp;
        Rng seed{0, 0};
    uint32_t pixel = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = Rng{A.seed[k], rc.rng};
            pixel = A.pixel[k];
            Hit h = load_hit(rc, H, k, o, d);
            if (!h.valid) {
                splat(rc, pixel, tp * rc.sky);
            } else {
                o = h.pos;
                splat(rc, pixel, tp * h.m.Emissivity);
                float3 thr = f3(1.0f);
                float pdf;
                bool diffuse = false;
                const float3 nd = sample_bsdf(d, h.m, seed, h.N, thr, false, pdf, false, &diffuse);
                if (diffuse) {
                    float3 preflect, prefract, pdiffuse;
                    decision_probabilities(h.m, preflect, prefract, pdiffuse);
                    const float3 fr = ((pdiffuse * h.m.Diffuse) / kPI) / avg3(pdiffuse);
                    const float side = dot(d, h.N);
                    float3 irr = f3(0.0f);
                    const int bx = (int)rintf(X::div(o.x, rc.pmSpacing)), by = (int)rintf(X::div(o.y, rc.pmSpacing)),
                              bz = (int)rintf(X::div(o.z, rc.pmSpacing));
                    for (int c = 0; c < 8; ++c) {
                        uint32_t idx = pm_find(rc, pm_cell_hash(bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1)));
                        for (uint32_t steps = 0; idx != 0xFFFFFFFFu && steps < rc.pmCap; ++steps) {
                            const float4 r0 = __ldg(rc.pmPhotons + 2 * (size_t)idx);
                            const float4 r1 = __ldg(rc.pmPhotons + 2 * (size_t)idx + 1);
                            const float3 toPhoton = make_float3(r1.x, r1.y, r1.z) - o;
                            const float rsq = dot(toPhoton, toPhoton);
                            if (rsq <= rc.pmRadiusSq && fabsf(dot(toPhoton, h.N)) < 0.01f) {
                                const float3 pdir = unpack_normal32(__float_as_uint(r1.w));
                                if (!(side * dot(pdir, h.N) < 0.0f))
                                    irr += fr * make_float3(r0.y, r0.z, r0.w) * (1.0f * kernel);
                            }
                            idx = __float_as_uint(r0.x);
                        }
                    }
                    splat(rc, pixel, irr * tp);
                } else {
                    d = nd;
                    o = o + d * kRAY_HIT_EPSILON;
                    tp *= thr;
                    survive = depth + 1 < rc.maxPathLength;
                    if (survive && depth >= rc.rrStartDepth) {
                        const float p = saturate(luminance(thr) + 0.02f);
                        if (random01(seed) >= p) survive = false;
                        else tp /= p;
                    }
                }
            }
        }
        uint32_t qb;
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, pixel, 0u, 1.0f);
    }
}

// ------------------------------------------------------------ importon map light tracer
// PixelMapLighttracer (pixelmaplighttracer.cpp:76-116) with the lossless hash
// grid and DEPTH_BUFFER_OCCLUSION_TEST, its compiled configuration: each
// iteration an eye pass (pixelmaplt/importondistribution.comp) stores at most
// one importon per pixel, at the eye path's first diffuse decision after at
// least one specular bounce, and writes the first hit into a G-buffer; then
// photons (pixelmaplt/photontracing.comp) splat every vertex into the pixels
// of the importons around it and reproject it onto the image, where the
// G-buffer's plane test stands in for a visibility ray.

// PackHDR64 / UnpackHDR64 (helper.glsl:116-156): Y as a float, Cg and Co as
// 12-bit mantissas with a shared exponent. ceil(log2(x)) and exp2 of the
// integer exponent are taken exactly from the binary exponent.
GPUGI_D int hdr64_exponent(float maxValue) {
    if (!(maxValue > 0.0f)) return -126;  // log2(0) = -inf, clamped
    if (isinf(maxValue)) return 127;
    int e;
    const float m = frexpf(maxValue, &e);  // maxValue = m 2^e, m in [0.5, 1)
    if (m == 0.5f) --e;
    return min(max(e, -126), 127);
}
GPUGI_D float2 pack_hdr64(float3 c) {
    const float y = X::add(X::add(X::mul(c.x, 0.25f), X::mul(c.y, 0.5f)), X::mul(c.z, 0.25f));
    const float cg = X::add(X::add(X::mul(c.x, -0.25f), X::mul(c.y, 0.5f)), X::mul(c.z, -0.25f));
    const float co = X::add(X::mul(c.x, 0.5f), X::mul(c.z, -0.5f));
    const int e = hdr64_exponent(fmaxf(fabsf(cg), fabsf(co)));
    const float range = ldexpf(1.0f, e);
    const float mx = fminf(fmaxf(X::add(X::div(X::mul(cg, 2048.0f), range), 2048.0f), 0.0f), 4095.0f);
    const float my = fminf(fmaxf(X::add(X::div(X::mul(co, 2048.0f), range), 2048.0f), 0.0f), 4095.0f);
    return make_float2(y, __uint_as_float(((uint32_t)mx << 20) | ((uint32_t)my << 8) | (uint32_t)(e + 126)));
}
GPUGI_D float3 unpack_hdr64(float2 h) {
    const uint32_t p = __float_as_uint(h.y);
    const float scale = ldexpf(1.0f, (int)(p & 0xFFu) - 126 - 11);  // range / 2048
    const float cg = X::mul((float)(p >> 20) - 2048.0f, scale);
    const float co = X::mul((float)((p >> 8) & 0xFFFu) - 2048.0f, scale);
    const float tmp = X::sub(h.x, cg);
    return make_float3(X::add(tmp, co), X::add(h.x, cg), X::sub(tmp, co));
}

// insertToHashGrid (maps/hashmap.glsl:31-59) of the record idx at pos;
// returns the previous list head of its cell, or false when the table is full.
GPUGI_D bool grid_insert(const RenderConst& rc, float3 pos, uint32_t idx, uint32_t& next) {
    const int cx = (int)ceilf(X::div(pos.x, rc.pmSpacing)), cy = (int)ceilf(X::div(pos.y, rc.pmSpacing)),
              cz = (int)ceilf(X::div(pos.z, rc.pmSpacing));
    const uint32_t hash = pm_cell_hash(cx, cy, cz);
    uint32_t i = hash % rc.pmMapSize, step = 1;
    for (uint32_t probe = 0; probe < rc.pmMapSize; ++probe) {
        const uint32_t key = atomicCAS(rc.pmMap + 2 * (size_t)i, 0xFFFFFFFFu, hash);
        if (key == hash || key == 0xFFFFFFFFu) {
            next = atomicExch(rc.pmMap + 2 * (size_t)i + 1, idx);
            return true;
        }
        i = (uint32_t)(((uint64_t)i + step * 2 + 1) % rc.pmMapSize);
        ++step;
    }
    return false;
}

// importondistribution.comp:21-33: one eye path per pixel (jitter with -0.5);
// the pixel's G-buffer normal half is reset (the reference's alpha write of a
// missed pixel) and the iteration is counted in alpha.
__global__ void k_im_generate(RenderConst rc, PathSoA A) {
    const uint32_t total = (uint32_t)rc.numPixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < total; pix += gridDim.x * blockDim.x) {
        const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
        Rng seed = rng_init(rc.rng, rc.iteration + rc.sampleBase, pix);
        const float3 d = primary_direction(rc, seed, x, y);
        store_path(A, pix, rc.camPos, d, f3(1.0f), seed, pix, 0u, 1.0f);
        rc.imGbufN0[pix] = 0.0f;
        splat(rc, pix, f3(0.0f), 1.0f);
    }
}

// importondistribution.comp:35-120, one bounce: the first hit goes to the
// G-buffer (position, packed geometry normal facing the camera), emission is
// added, and at a diffuse decision after the first vertex the importon
// {throughput, incident direction, position, pixel} is stored in the grid and
// the path ends; otherwise it continues with the +0.02 roulette.
__global__ void __launch_bounds__(128) k_im_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, int depth) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        bool survive = false;
        float3 o, d, tp;
        Rng seed{0, 0};
    uint32_t pixel = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = Rng{A.seed[k], rc.rng};
            pixel = A.pixel[k];
            Hit h = load_hit(rc, H, k, o, d);
            if (!h.valid) {
                splat(rc, pixel, tp * rc.sky);  // addition: the reference's cube-map lookup is commented out
            } else {
                o = h.pos;
                if (depth == 0) {
                    const float4 rec = __ldg(rc.s.tris + 3 * (size_t)H.slot[k] + 2);
                    float3 gN = X::normalize(make_float3(rec.y, rec.z, rec.w));
                    if (dot(gN, d) > 0.0f) gN = -gN;
                    const float2 pn = pack_normal(gN);
                    rc.imGbuf[pixel] = make_float4(o.x, o.y, o.z, pn.y);
                    rc.imGbufN0[pixel] = pn.x;
                }
                splat(rc, pixel, tp * h.m.Emissivity);
                float3 thr = f3(1.0f);
                float pdf;
                bool diffuse = false;
                const float3 nd = sample_bsdf(d, h.m, seed, h.N, thr, false, pdf, false, &diffuse);
                if (diffuse) {
                    if (depth > 0) {
                        float3 preflect, prefract, pdiffuse;
                        decision_probabilities(h.m, preflect, prefract, pdiffuse);
                        tp *= pdiffuse / fmaxf(avg3(pdiffuse), kDIVISOR_EPSILON);
                        uint32_t next;
                        if (grid_insert(rc, o, pixel, next)) {
                            const float2 hdr = pack_hdr64(tp);
                            float4* rec = rc.pmPhotons + 2 * (size_t)pixel;
                            rec[0] = make_float4(__uint_as_float(next), hdr.x, hdr.y, __uint_as_float(pack_normal32(d)));
                            rec[1] = make_float4(o.x, o.y, o.z,
                                                 __uint_as_float((pixel % (uint32_t)rc.width) |
                                                                 ((pixel / (uint32_t)rc.width) << 16)));
                        } else {
                            raise_error(rc.err, DEVERR_QUEUE_OVERFLOW);
                        }
                    }
                } else {
                    d = nd;
                    o = o + d * kRAY_HIT_EPSILON;
                    tp *= thr;
                    survive = depth + 1 < rc.maxPathLength;
                    if (survive && depth >= rc.rrStartDepth) {
                        const float p = saturate(luminance(thr) + 0.02f);
                        if (random01(seed) >= p) survive = false;
                        else tp /= p;
                    }
                }
            }
        }
        uint32_t qb;
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, pixel, 0u, 1.0f);
    }
}

// ProjectToScreen (screenreproject.glsl:55-227) with DEPTH_BUFFER_OCCLUSION_TEST
// and the box filter: the vertex counts for the pixel it projects to when it
// lies on the plane of that pixel's first eye hit (within -5e-4 .. 5e-3 of the
// camera distance) instead of when a visibility ray reaches the camera. With
// computeFullBSDF false only the diffuse part, on the camera's side, counts.
GPUGI_D void project_gbuffer(const RenderConst& rc, float3 pos, float3 inDir, float3 gN, float3 sN,
                             const MaterialData& m, float3 tp, bool computeFullBSDF) {
    float3 cd = rc.camPos - pos;
    const float camViewDotRay = -dot(rc.camW, cd);
    if (!(camViewDotRay > 0.0f)) return;
    float sx = -dot(rc.camU, cd) / camViewDotRay, sy = -dot(rc.camV, cd) / camViewDotRay;
    sx /= dot(rc.camU, rc.camU);
    sy /= dot(rc.camV, rc.camV);
    if (!(sx >= -1.0f && sx < 1.0f && sy > -1.0f && sy <= 1.0f)) return;
    const float distSq = dot(cd, cd);
    const float dist = sqrtf(distSq);
    cd /= dist;
    const float3 ro = cd * kRAY_HIT_EPSILON + pos;
    const int px = (int)rintf((sx * 0.5f + 0.5f) * (float)rc.width);
    const int py = (int)rintf((sy * 0.5f + 0.5f) * (float)rc.height);
    if (px < 0 || py < 0 || px >= rc.width || py >= rc.height) return;  // image loads and atomics outside the image
    const uint32_t pixel = (uint32_t)(py * rc.width + px);
    const float4 g = rc.imGbuf[pixel];
    const float3 occN = unpack_normal(rc.imGbufN0[pixel], g.w);
    const float3 occPos = make_float3(g.x, g.y, g.z) - (4.0f * kRAY_HIT_EPSILON) * occN;
    const float planeDist = dot(ro - occPos, occN) / dist;
    if (!(planeDist >= -5e-4f && planeDist < 5e-3f)) return;
    const float cosAtCamera = saturate(camViewDotRay / dist);
    const float fluxToIrradiance = shading_corrected_out_dot_n(inDir, cd, gN, sN) /
                                   (cosAtCamera * cosAtCamera * cosAtCamera * rc.pixelArea * distSq);
    float3 bsdf;
    if (computeFullBSDF) {
        float pdf;
        bsdf = adjoint_bsdf(inDir, cd, m, sN, pdf);
    } else if (dot(inDir, sN) * dot(cd, sN) < 0.0f) {
        float3 preflect, prefract, pdiffuse;
        decision_probabilities(m, preflect, prefract, pdiffuse);
        bsdf = pdiffuse * m.Diffuse * avg3(pdiffuse) / kPI;
    } else {
        return;
    }
    splat(rc, pixel, tp * fluxToIrradiance * bsdf);
}

// photontracing.comp:40-136, one bounce of one photon: the importons of the
// 2x2x2 cells from round(pos / spacing) that lie within the query radius on
// the surface's plane and on the photon's side receive its irradiance
// estimate (radianceEstimate, :15-36), the vertex is reprojected, and the
// photon continues with the adjoint BSDF and the +0.02 roulette. Info bit 0
// marks a photon whose path is still purely specular (it left a point light).
__global__ void __launch_bounds__(128) k_im_photon_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, int depth) {
    const uint32_t n = rc.cnt->path[depth];
    const float kernel = kPI * rc.pmRadiusSq;
    WARP_LOOP(n, k, valid) {
        bool survive = false;
        float3 o, d, tp;
        Rng seed{0, 0};
    uint32_t gid = 0, info = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = Rng{A.seed[k], rc.rng};
            gid = A.pixel[k];
            info = A.info[k];
            const int32_t slot = H.slot[k];
            if (slot >= 0) {
                const float4 rec = __ldg(rc.s.tris + 3 * (size_t)slot + 2);
                const float3 gN = make_float3(rec.y, rec.z, rec.w);  // cross(e1, e0), not normalised
                o = X::add3(o, X::scale(H.t[k], d));
                const int4 tri = __ldg(rc.s.slots + slot);
                float2 tc;
                const float3 sN = hit_normal(rc.s, tri, H.u[k], H.v[k], &tc);
                const MaterialData m = load_material(rc.s, tri.w, tc);
                float3 preflect, prefract, pdiffuse;
                decision_probabilities(m, preflect, prefract, pdiffuse);
                const float3 bsdfTp = (pdiffuse * m.Diffuse) / kPI * tp;
                const float side = dot(d, sN);
                const int bx = (int)rintf(X::div(o.x, rc.pmSpacing)), by = (int)rintf(X::div(o.y, rc.pmSpacing)),
                          bz = (int)rintf(X::div(o.z, rc.pmSpacing));
                for (int c = 0; c < 8; ++c) {
                    uint32_t idx = pm_find(rc, pm_cell_hash(bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1)));
                    for (uint32_t steps = 0; idx != 0xFFFFFFFFu && steps < rc.pmCap; ++steps) {
                        const float4 r0 = __ldg(rc.pmPhotons + 2 * (size_t)idx);
                        const float4 r1 = __ldg(rc.pmPhotons + 2 * (size_t)idx + 1);
                        const float3 toImporton = make_float3(r1.x, r1.y, r1.z) - o;
                        if (dot(toImporton, toImporton) <= rc.pmRadiusSq && fabsf(dot(toImporton, sN)) < 0.01f &&
                            side * dot(sN, unpack_normal32(__float_as_uint(r0.w))) > 0.0f) {
                            const uint32_t pc = __float_as_uint(r1.w);
                            const float3 vt = unpack_hdr64(make_float2(r0.y, r0.z));
                            splat(rc, (pc >> 16) * (uint32_t)rc.width + (pc & 0xFFFFu), vt * bsdfTp / kernel);
                        }
                        idx = __float_as_uint(r0.x);
                    }
                }
                if (avg3(tp) > 1e-10f) project_gbuffer(rc, o, d, gN, sN, m, tp, (info & 1u) != 0);
                float3 thr = f3(1.0f);
                float pdf;
                bool diffuse = false;
                const float3 nd = sample_bsdf(d, m, seed, sN, thr, true, pdf, false, &diffuse);
                thr *= shading_correction(d, nd, gN, sN);
                tp *= thr;
                if (diffuse) info &= ~1u;
                survive = depth + 1 < rc.maxPathLength;
                if (survive && depth >= rc.rrStartDepth) {
                    const float p = saturate(luminance(thr) + 0.02f);
                    if (random01(seed) >= p) survive = false;
                    else tp /= p;
                }
                d = nd;
                o = o + d * kRAY_HIT_EPSILON;
            }
        }
        uint32_t qb;
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, gid, info, 1.0f);
    }
}

// ------------------------------------------------------------ radiance cache
// Camera paths for the path tracer with a radiance cache: as
// k_camera_generate, plus the choice of training paths (a per-frame hash of
// the pixel below nrcTrainThreshold) and their buffer slot (kept in lastP).
__global__ void k_nrc_generate(RenderConst rc, PathSoA A) {
    const uint32_t total = rc.samples * (uint32_t)rc.numPixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        const uint32_t s = p / (uint32_t)rc.numPixels, pix = p % (uint32_t)rc.numPixels;
        const uint32_t frame = rc.iteration + rc.sampleBase + s;
        const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
        Rng seed = rng_init(rc.rng, frame, pix);
        const float3 d = primary_direction(rc, seed, x, y);
        uint32_t info = s << 8;
        float slotBits = 0.0f;
        if (wanghash(pix ^ wanghash(frame + 0x9E3779B9u)) < rc.nrcTrainThreshold) {
            const uint32_t slot = atomicAdd(rc.trainPaths, 1u);
            if (slot < rc.trainCap) {
                info |= 2u;
                if (wanghash(slot ^ wanghash(frame + 0x7F4A7C15u)) < rc.nrcUnbiasedThreshold) info |= 4u;
                slotBits = __uint_as_float(slot);
                rc.tvCount[slot] = 0;
            }
        }
        store_path(A, p, rc.camPos, d, f3(1.0f), seed, pix, info, slotBits);
        A.job[p] = 0u;
    }
}

GPUGI_D void add3(float* p, float3 c) {
    atomicAdd(p, c.x);
    atomicAdd(p + 1, c.y);
    atomicAdd(p + 2, c.z);
}

// One bounce of the path tracer with a radiance cache, per lane. Render
// paths stop at vertex nrcTerminateDepth and query the cache for the
// radiance reflected there towards the previous vertex; with nrcSpread > 0
// they stop earlier, at the first vertex n >= 1 where the path spread
// a(x1..xn) exceeds nrcSpread x a0 (Mueller et al. 2021, "Real-time Neural
// Radiance Caching for Path Tracing", section 3.4: sqrt(a) is the sum over
// the segments of |x_{i-1} - x_i| / sqrt(p(w_i) |cos theta_i|), a0 =
// |x0 - x1|^2 / (4 pi cos theta_1) at the primary vertex). Training paths
// continue as plain path tracing and record every vertex {position,
// outgoing direction, normal, albedo, throughput}; the radiance that later
// reaches each vertex (NEE via the shadow queue, emission and sky found by
// the next segment) is accumulated into the vertex's tvC entry. With
// self-training (nrcTrainLength > 0) a training path stops at vertex
// nrcTrainLength and queries the cache there; the query's radiance x
// throughput goes to the previous vertex's tvC like emission found by the
// segment, except for the unbiased training paths (info bit 2), which run
// to the path's end. A training path with pixel kNoPixel (BPT with the
// cache) only trains.
// Spread state of a render path: job = sqrt(nrcSpread a0) as float bits,
// lastP = half2 {sqrt(a) / sqrt(nrcSpread a0), 1 / sqrt(pdf of the last
// sampled direction)}.
constexpr uint32_t kTrainQuery = 0x80000000u;  // query record pixel: radiance goes to training vertex (low bits)

struct NrcLane {
    bool survive = false, shadow = false, query = false;
    float3 o, d, tp, sro, srd, contrib, qN, qAlbedo, qT;
    float srl = 0.0f, lastP = 0.0f;
    Rng seed{0, 0};
    uint32_t pixel = 0, info = 0, train = kNoTrain, job = 0, qPixel = 0;
};

GPUGI_D void nrc_pt_lane(const RenderConst& rc, const PathSoA& A, const HitSoA& H, uint32_t k, int depth,
                         NrcLane& L) {
    const float lightSampleWeight = (float)rc.numLightSamples;
    const uint32_t stride = (uint32_t)rc.maxPathLength;
    float3& o = L.o;
    float3& d = L.d;
    float3& tp = L.tp;
    o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
    d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
    tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
    L.seed = Rng{A.seed[k], rc.rng};
    L.pixel = A.pixel[k];
    L.info = A.info[k];
    L.lastP = A.lastP[k];
    const bool training = (L.info & 2u) != 0;
    const uint32_t tslot = __float_as_uint(L.lastP);
    const uint32_t prevVertex = (training && depth > 0) ? tslot * stride + depth - 1 : kNoTrain;
    L.job = A.job[k];
    Hit h = load_hit(rc, H, k, o, d);
    if (!h.valid) {
        const float3 c = tp * rc.sky;
        splat(rc, L.pixel, c);
        if (prevVertex != kNoTrain) add3(rc.tvC + 3 * (size_t)prevVertex, c);
        return;
    }
    o = h.pos;
    if (!(L.info & 1u)) {
        const float3 e = tp * h.m.Emissivity;
        splat(rc, L.pixel, e);
        if (prevVertex != kNoTrain) add3(rc.tvC + 3 * (size_t)prevVertex, e);
    }
    bool stop = training ? (rc.nrcTrainLength > 0 && depth == rc.nrcTrainLength && !(L.info & 4u))
                         : depth == rc.nrcTerminateDepth;
    float spreadSum = 0.0f;
    if (!training && rc.nrcSpread > 0.0f) {
        const float cosIn = fmaxf(fabsf(dot(h.N, d)), 1e-4f);
        if (depth == 0) {
            L.job = __float_as_uint(h.t * sqrtf(rc.nrcSpread / (4.0f * kPI * cosIn)));
        } else {
            const float2 st = __half22float2(*reinterpret_cast<const __half2*>(&L.lastP));
            spreadSum = st.x + h.t * st.y / (sqrtf(cosIn) * fmaxf(__uint_as_float(L.job), 1e-30f));
            stop = stop || spreadSum > 1.0f;
        }
    }
    if (stop) {
        L.query = true;
        L.qN = h.N;
        L.qAlbedo = h.m.Diffuse;
        L.qT = tp;
        L.qPixel = training ? (kTrainQuery | prevVertex) : L.pixel;
        return;
    }
    const bool didNEE = h.m.Reflectiveness.w < 500.0f;
    L.info = (L.info & ~1u) | (didNEE ? 1u : 0u);
    if (training) {
        const uint32_t v = tslot * stride + (uint32_t)depth;
        float* r = rc.tvRec + 16 * (size_t)v;
        r[0] = o.x; r[1] = o.y; r[2] = o.z;
        r[3] = -d.x; r[4] = -d.y; r[5] = -d.z;
        r[6] = h.N.x; r[7] = h.N.y; r[8] = h.N.z;
        r[9] = h.m.Diffuse.x; r[10] = h.m.Diffuse.y; r[11] = h.m.Diffuse.z;
        r[12] = tp.x; r[13] = tp.y; r[14] = tp.z;
        rc.tvC[3 * (size_t)v] = rc.tvC[3 * (size_t)v + 1] = rc.tvC[3 * (size_t)v + 2] = 0.0f;
        rc.tvCount[tslot] = (uint32_t)depth + 1;
        L.train = v;
    }
    const uint32_t li = random_uint(L.seed) % rc.numLightSamples;
    float3 rad;
    if (direct_light(rc, L.info >> 8, o, h.N, li, d, h.m, didNEE, rad, L.sro, L.srd, L.srl)) {
        L.contrib = rad * tp * lightSampleWeight;
        L.shadow = L.contrib.x != 0.0f || L.contrib.y != 0.0f || L.contrib.z != 0.0f;
    }
    float3 thr = f3(1.0f);
    float pdf;
    d = sample_bsdf(d, h.m, L.seed, h.N, thr, false, pdf);
    o = o + d * kRAY_HIT_EPSILON;
    tp *= thr;
    L.survive = roulette(rc, depth, thr, tp, L.seed) && depth + 1 < rc.maxPathLength;
    if (!training && rc.nrcSpread > 0.0f) {
        const __half2 st = __floats2half2_rn(fminf(spreadSum, 60000.0f), fminf(rsqrtf(fmaxf(pdf, 1e-8f)), 60000.0f));
        L.lastP = *reinterpret_cast<const float*>(&st);
    }
}

// Cache query record: 12 floats {position, direction towards the previous
// vertex, normal, albedo}, the throughput it is weighted with and its pixel.
GPUGI_D void store_query(const RenderConst& rc, uint32_t q, float3 o, float3 d, float3 n, float3 albedo, float3 t,
                         uint32_t pixel) {
    float* r = rc.queries + 12 * (size_t)q;
    r[0] = o.x; r[1] = o.y; r[2] = o.z;
    r[3] = -d.x; r[4] = -d.y; r[5] = -d.z;
    r[6] = n.x; r[7] = n.y; r[8] = n.z;
    r[9] = albedo.x; r[10] = albedo.y; r[11] = albedo.z;
    rc.qT[3 * (size_t)q] = t.x;
    rc.qT[3 * (size_t)q + 1] = t.y;
    rc.qT[3 * (size_t)q + 2] = t.z;
    rc.qPixel[q] = pixel;
}

__global__ void __launch_bounds__(128) k_nrc_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                   int depth) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        NrcLane L;
        if (valid) nrc_pt_lane(rc, A, H, k, depth, L);
        uint32_t qs, qb, qq;
        warp_append(&rc.cnt->shadow[depth], L.shadow, qs);
        if (L.shadow) store_shadow(Q, qs, L.sro, L.srd, L.srl, L.contrib, L.pixel, L.train);
        warp_append(rc.queryCount, L.query, qq);
        if (L.query && qq < rc.queryCap) store_query(rc, qq, L.o, L.d, L.qN, L.qAlbedo, L.qT, L.qPixel);
        warp_append(&rc.cnt->path[depth + 1], L.survive, qb);
        if (L.survive) {
            store_path(B, qb, L.o, L.d, L.tp, L.seed, L.pixel, L.info, L.lastP);
            B.job[qb] = L.job;
        }
    }
}

// Eye paths of BPT with a radiance cache: one render path per pixel and
// sample as k_camera_generate(bidir), followed by nTrain training paths at
// hashed pixels. Training paths trace plain PT paths that only feed the
// cache (pixel kNoPixel: no splat), so every pixel keeps the BPT estimator.
__global__ void k_nrc_bpt_generate(RenderConst rc, PathSoA A, uint32_t nTrain) {
    const uint32_t render = rc.samples * (uint32_t)rc.numPixels, total = render + nTrain;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        rc.cnt->path[0] = total;
        *rc.trainPaths = nTrain;
    }
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        if (p < render) {
            const uint32_t s = p / (uint32_t)rc.numPixels, pix = p % (uint32_t)rc.numPixels;
            const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
            Rng seed = rng_init(rc.rng, rc.iteration + rc.sampleBase + s, pix);
            const float3 d = primary_direction(rc, seed, x, y);
            store_path(A, p, rc.camPos, d, f3(1.0f), seed, pix, s << 8, 1.0f);
            A.job[p] = __float_as_uint(1.0f);
            splat(rc, pix, f3(0.0f), 1.0f);
        } else {
            const uint32_t slot = p - render, s = slot % rc.samples;
            const uint32_t frame = rc.iteration + rc.sampleBase + s;
            const uint32_t pix = wanghash(slot ^ wanghash(frame + 0x9E3779B9u)) % (uint32_t)rc.numPixels;
            const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
            Rng seed = rng_init(rc.rng, frame ^ 0x5bd1e995u, slot);
            const float3 d = primary_direction(rc, seed, x, y);
            rc.tvCount[slot] = 0;
            store_path(A, p, rc.camPos, d, f3(1.0f), seed, kNoPixel, (s << 8) | 2u, __uint_as_float(slot));
            A.job[p] = __float_as_uint(1.0f);
        }
    }
}

// One bounce of BPT with a radiance cache: render paths run the BPT eye
// bounce and stop at vertex nrcTerminateDepth (light-cache connections
// limited to paths of that length; longer paths come from the cache query);
// training paths run the PT training bounce.
__global__ void __launch_bounds__(128) k_nrc_bpt_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H,
                                                       ShadowSoA Q, int depth) {
    const uint32_t n = rc.cnt->path[depth];
    const int cap = min(rc.maxPathLength, rc.nrcTerminateDepth);
    WARP_LOOP(n, k, valid) {
        bool survive = false, shadow = false, query = false;
        float3 o, d, tp, sro, srd, contrib, qN, qA, qT;
        float srl = 0.0f, lastP = 0.0f, misProd = 1.0f;
        Rng seed{0, 0};
        uint32_t pixel = 0, info = 0, train = kNoTrain, qPixel = 0;
        if (valid) {
            if (A.info[k] & 2u) {
                NrcLane L;
                nrc_pt_lane(rc, A, H, k, depth, L);
                survive = L.survive; shadow = L.shadow; query = L.query;
                o = L.o; d = L.d; tp = L.tp; sro = L.sro; srd = L.srd; contrib = L.contrib; srl = L.srl;
                qN = L.qN; qA = L.qAlbedo; qT = L.qT; qPixel = L.qPixel;
                lastP = L.lastP; seed = L.seed; pixel = L.pixel; info = L.info; train = L.train;
            } else {
                BptLane L;
                bpt_shade_lane(rc, A, H, k, depth, cap, rc.nrcTerminateDepth, L);
                survive = L.survive; shadow = L.shadow; query = L.query;
                o = L.o; d = L.d; tp = L.tp; sro = L.sro; srd = L.srd; contrib = L.contrib; srl = L.srl;
                qN = L.qN; qA = L.qAlbedo; qT = L.qT; qPixel = L.pixel;
                lastP = L.lastP; misProd = L.misProd; seed = L.seed; pixel = L.pixel; info = L.info;
            }
        }
        uint32_t qs, qb, qq;
        warp_append(&rc.cnt->shadow[depth], shadow, qs);
        if (shadow) store_shadow(Q, qs, sro, srd, srl, contrib, pixel, train);
        warp_append(rc.queryCount, query, qq);
        if (query && qq < rc.queryCap) store_query(rc, qq, o, d, qN, qA, qT, qPixel);
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) {
            store_path(B, qb, o, d, tp, seed, pixel, info, lastP);
            B.job[qb] = __float_as_uint(misProd);
        }
    }
}

// Ray counters of a second wavefront lane folded into the first.
__global__ void k_add_ray_counts(Counters* into, const Counters* from) {
    if (threadIdx.x < 2) into->rays[threadIdx.x] += from->rays[threadIdx.x];
}

// Splat throughput x cache radiance for every query; a self-training query
// adds it to its training vertex instead.
__global__ void k_nrc_apply(RenderConst rc, const float* __restrict__ radiance) {
    const uint32_t n = min(*rc.queryCount, rc.queryCap);
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const float3 t = make_float3(rc.qT[3 * q], rc.qT[3 * q + 1], rc.qT[3 * q + 2]);
        const float3 c = t * make_float3(radiance[3 * q], radiance[3 * q + 1], radiance[3 * q + 2]);
        const uint32_t pix = rc.qPixel[q];
        if (pix != kNoPixel && (pix & kTrainQuery)) add3(rc.tvC + 3 * (size_t)(pix & ~kTrainQuery), c);
        else splat(rc, pix, c);
    }
}

// Training targets: the radiance reflected at vertex k towards vertex k-1 is
// the sum of everything accumulated at vertices >= k divided by the
// throughput at arrival T_k. Samples: 15 floats {query, target}.
__global__ void k_nrc_targets(RenderConst rc, float* __restrict__ samples, uint32_t* sampleCount, uint32_t cap) {
    const uint32_t paths = min(*rc.trainPaths, rc.trainCap);
    const uint32_t stride = (uint32_t)rc.maxPathLength;
    // paths in a shuffled order (multiplication by a prime modulo the count
    // is a permutation), so a full sample buffer drops paths uniformly
    const uint64_t offset = wanghash(rc.iteration + rc.sampleBase);
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < paths; q += gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(((uint64_t)q * 2654435761ull + offset) % paths);
        const uint32_t nv = min(rc.tvCount[p], stride);
        float3 S = f3(0.0f);
        for (int k = (int)nv - 1; k >= 0; --k) {
            const size_t v = (size_t)p * stride + k;
            S += make_float3(rc.tvC[3 * v], rc.tvC[3 * v + 1], rc.tvC[3 * v + 2]);
            const float* r = rc.tvRec + 16 * v;
            const float3 T = make_float3(r[12], r[13], r[14]);
            const float3 y = make_float3(T.x > 1e-20f ? S.x / T.x : 0.0f, T.y > 1e-20f ? S.y / T.y : 0.0f,
                                         T.z > 1e-20f ? S.z / T.z : 0.0f);
            const uint32_t i = atomicAdd(sampleCount, 1u);
            if (i >= cap) continue;
            float* o = samples + 15 * (size_t)i;
            for (int c = 0; c < 12; ++c) o[c] = r[c];
            o[12] = y.x;
            o[13] = y.y;
            o[14] = y.z;
        }
    }
}

// Sum over pixels of |rgb * scale - ref|^2 in FP64 (sqerror.frag:12-17 + the
// mip-chain mean of TextureMSE::ComputeCurrentMSE).
__global__ void k_mse(const float4* __restrict__ rgba, const double* __restrict__ rgb64,
                      const float* __restrict__ ref, size_t n, double scale, double* sum) {
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double r, g, b;
        if (rgb64) {
            r = rgb64[3 * i];
            g = rgb64[3 * i + 1];
            b = rgb64[3 * i + 2];
        } else {
            const float4 c = rgba[i];
            r = c.x;
            g = c.y;
            b = c.z;
        }
        const double dr = r * scale - ref[3 * i], dg = g * scale - ref[3 * i + 1], db = b * scale - ref[3 * i + 2];
        acc += dr * dr + dg * dg + db * db;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    __shared__ double part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (threadIdx.x == 0) atomicAdd(sum, acc);
    }
}

// ------------------------------------------------------------ batched jobs
// Many jobs (each its own scene, camera, image, resolution, sample count,
// path length and pass: PT, LT or BPT) share one wavefront: their paths sit
// in the same queues, every stage is one launch over all of them, and each
// path and shadow ray carries its job index. Phase 0 holds the PT eye paths,
// the LT particles and the BPT light paths (each BPT job writes its own light
// caches); phase 1 the BPT eye paths, which connect to those caches. The job
// constants come from a device table, so the launch sequence does not change
// between rounds and is replayed as one CUDA graph.

// Largest j < numJobs with offsets[j] <= p (offsets[numJobs] > p).
GPUGI_D uint32_t find_job(const uint32_t* __restrict__ offsets, uint32_t numJobs, uint32_t p) {
    uint32_t lo = 0, hi = numJobs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(offsets + mid) <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The first vertices of the phase's paths (offsets: the phase's path range of
// every job). An LT particle that is the first of its light sample also
// queues that sample's camera connection (showlightcaches.comp) as a shadow
// ray of depth 0, so the shadow walker tests its visibility.
__global__ void k_batch_generate(const RenderConst* __restrict__ jobs, const uint32_t* __restrict__ offsets,
                                 uint32_t numJobs, Counters* cnt, PathSoA A, ShadowSoA Q, int phase) {
    const uint32_t total = offsets[numJobs];
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt->path[0] = total;
    WARP_LOOP(total, p, valid) {
        bool view = false;
        float3 ro, rd, color;
        float rl = 0.0f;
        uint32_t pixel = 0, j = 0;
        if (valid) {
            j = find_job(offsets, numJobs, p);
            const RenderConst& rc = jobs[j];
            const uint32_t local = p - offsets[j];
            if (phase == 1 || rc.pass == GPUGI_PASS_PT) {
                camera_path_start(rc, A, p, local / (uint32_t)rc.numPixels, local % (uint32_t)rc.numPixels,
                                  phase == 1);
            } else {
                const uint32_t s = local / rc.lightThreads, gid = local % rc.lightThreads;
                light_path_start(rc, A, p, s, gid, rc.pass == GPUGI_PASS_BPT);
                if (rc.pass == GPUGI_PASS_LT && gid % (uint32_t)rc.numRaysPerLightSample == 0)
                    view = light_sample_view(rc, s * rc.numLightSamples + gid / (uint32_t)rc.numRaysPerLightSample,
                                             ro, rd, rl, color, pixel);
            }
            A.job[p] = j;
        }
        uint32_t qs;
        warp_append(&cnt->shadow[0], view, qs);
        if (view) {
            store_shadow(Q, qs, ro, rd, rl, color, pixel);
            Q.job[qs] = j;
        }
    }
}

// Walks of rays of several scenes: each ray's scene comes from its job, and
// the scene's bounds kind selects the node test per step. As in k_extend,
// queues shorter than groupBelow are walked by 8-lane groups.
template <bool ANY_HIT, typename Load, typename Finish>
GPUGI_D void persistent_walks_multi(uint32_t n, unsigned long long* work, uint32_t* err, Load load, Finish finish) {
    const unsigned lane = threadIdx.x & 31u;
    WalkState w;
    // the ray's scene, copied when its walk starts: the few fields a step
    // reads then stay in registers instead of being loaded every step
    DevScene sc;
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    while (true) {
        const bool need = !active && !exhausted;
        const unsigned needMask = __ballot_sync(0xffffffffu, need);
        if (needMask) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(work, (unsigned long long)__popc(needMask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need) {
                const unsigned long long my = base + (unsigned long long)__popc(needMask & ((1u << lane) - 1u));
                if (my < n) {
                    ray = (uint32_t)my;
                    float3 o, d;
                    float tmax;
                    sc = *load(ray, o, d, tmax);
                    walk_begin(w, sc, o, d, tmax);
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) {
            const bool done = sc.boundsKind == GPUGI_BOUNDS_ELLIPSOID ? walk_step<ANY_HIT, 1>(w, sc, err)
                              : sc.boundsKind == GPUGI_BOUNDS_OBOX    ? walk_step<ANY_HIT, 2>(w, sc, err)
                                                                      : walk_step<ANY_HIT, 0>(w, sc, err);
            if (done) {
                finish(ray, w.slot, w.len, w.u, w.v);
                active = false;
            }
        }
    }
}

template <bool ANY_HIT, typename Load, typename Finish>
GPUGI_D void walks_multi(uint32_t n, uint32_t groupBelow, unsigned long long* work, uint32_t* err, Load load,
                         Finish finish) {
    if (n < groupBelow)
        group_walks_multi<ANY_HIT, 8>(n, work, err, load, [&](uint64_t i, const GroupWalk& g) {
            finish((uint32_t)i, g.slot, g.len, g.u, g.v);
        });
    else
        persistent_walks_multi<ANY_HIT>(n, work, err, load, finish);
}

__global__ void __launch_bounds__(128) k_batch_extend(const RenderConst* __restrict__ jobs, Counters* cnt,
                                                      uint32_t* err, PathSoA A, HitSoA H, int depth,
                                                      uint32_t groupBelow) {
    const uint32_t n = cnt->path[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&cnt->rays[0], (unsigned long long)n);
    walks_multi<false>(
        n, groupBelow, &cnt->extendWork[depth], err,
        [&](uint64_t i, float3& o, float3& d, float& tmax) -> const DevScene* {
            o = make_float3(A.ox[i], A.oy[i], A.oz[i]);
            d = make_float3(A.dx[i], A.dy[i], A.dz[i]);
            tmax = kRAY_MAX;
            return &jobs[A.job[i]].s;
        },
        [&](uint32_t i, int32_t slot, float t, float u, float v) {
            H.slot[i] = slot;
            H.t[i] = t;
            H.u[i] = u;
            H.v[i] = v;
        });
}

__global__ void __launch_bounds__(128) k_batch_shadow(const RenderConst* __restrict__ jobs, Counters* cnt,
                                                      uint32_t* err, ShadowSoA Q, int depth, uint32_t groupBelow) {
    const uint32_t n = cnt->shadow[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&cnt->rays[1], (unsigned long long)n);
    walks_multi<true>(
        n, groupBelow, &cnt->shadowWork[depth], err,
        [&](uint64_t i, float3& o, float3& d, float& tmax) -> const DevScene* {
            o = make_float3(Q.ox[i], Q.oy[i], Q.oz[i]);
            d = make_float3(Q.dx[i], Q.dy[i], Q.dz[i]);
            tmax = Q.tmax[i];
            return &jobs[Q.job[i]].s;
        },
        [&](uint32_t i, int32_t slot, float, float, float) {
            if (slot < 0) splat(jobs[Q.job[i]], Q.pixel[i], make_float3(Q.cr[i], Q.cg[i], Q.cb[i]));
        });
}

// One bounce of the phase-0 paths: PT eye paths, LT particles and BPT light
// paths (the latter append to their job's light cache).
__global__ void __launch_bounds__(128) k_batch_shade(const RenderConst* __restrict__ jobs, Counters* cnt,
                                                     PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q, int depth) {
    const uint32_t n = cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        bool shadow = false, survive = false;
        float3 o, d, tp, sro, srd, c;
        float srl = 0.0f;
        Rng seed{0, 0};
    uint32_t pathPixel = 0, shadowPixel = 0, info = 0, j = 0;
        if (valid) {
            j = A.job[k];
            const RenderConst& rc = jobs[j];
            if (rc.pass == GPUGI_PASS_PT) {
                PtLane L;
                pt_shade_lane(rc, A, H, k, depth, L);
                shadow = L.shadow, survive = L.survive;
                o = L.o, d = L.d, tp = L.tp, sro = L.sro, srd = L.srd, c = L.contrib, srl = L.srl;
                seed = L.seed, pathPixel = shadowPixel = L.pixel, info = L.info;
            } else {
                LightLane L;
                light_shade_lane(rc, A, H, k, depth, rc.pass == GPUGI_PASS_BPT, L);
                shadow = L.shadow, survive = L.survive;
                o = L.o, d = L.d, tp = L.tp, sro = L.sro, srd = L.srd, c = L.color, srl = L.srl;
                seed = L.seed, pathPixel = L.gid, shadowPixel = L.pixel, info = L.info;
            }
        }
        uint32_t qs, qb;
        warp_append(&cnt->shadow[depth], shadow, qs);
        if (shadow) {
            store_shadow(Q, qs, sro, srd, srl, c, shadowPixel);
            Q.job[qs] = j;
        }
        warp_append(&cnt->path[depth + 1], survive, qb);
        if (survive) {
            store_path(B, qb, o, d, tp, seed, pathPixel, info, 1.0f);
            B.job[qb] = j;
        }
    }
}

// One bounce of the phase-1 paths: BPT eye paths.
__global__ void __launch_bounds__(128) k_batch_bpt_shade(const RenderConst* __restrict__ jobs, Counters* cnt,
                                                         PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q, int depth) {
    const uint32_t n = cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        BptLane L;
        uint32_t j = 0;
        if (valid) {
            j = A.job[k];
            bpt_shade_lane(jobs[j], A, H, k, depth, jobs[j].maxPathLength, -1, L);
        }
        uint32_t qs, qb;
        warp_append(&cnt->shadow[depth], L.shadow, qs);
        if (L.shadow) {
            store_shadow(Q, qs, L.sro, L.srd, L.srl, L.contrib, L.pixel);
            Q.job[qs] = j;
        }
        warp_append(&cnt->path[depth + 1], L.survive, qb);
        if (L.survive) {
            store_path(B, qb, L.o, L.d, L.tp, L.seed, L.pixel, L.info, L.lastP);
            B.job[qb] = j;
        }
    }
}

// ------------------------------------------------------------ buffers
struct RenderBuffers {
    size_t pathCap = 0, cacheBytes = 0, lightBytes = 0;
    void* block = nullptr;
    PathSoA A, B;
    HitSoA H;
    ShadowSoA Q;
    Counters* cnt = nullptr;
    CacheEntry* cache = nullptr;
    uint32_t* cacheCount = nullptr;
    float4* lights = nullptr;
    float* hostLights = nullptr;  // pinned staging for light samples
    size_t hostLightBytes = 0;
    uint32_t maxSamples = 0;
    // radiance-cache pass
    void* nrcBlock = nullptr;
    size_t nrcQueryCap = 0, nrcTrainCap = 0, nrcStride = 0, nrcSampleCap = 0;
    float *queries = nullptr, *qT = nullptr, *radiance = nullptr, *tvRec = nullptr, *tvC = nullptr,
          *samples = nullptr;
    uint32_t *qPixel = nullptr, *tvCount = nullptr, *nrcCounters = nullptr;  // counters: queries, paths, samples
    // photon mapper: hash table, photon records, append counter
    void* pmBlock = nullptr;
    size_t pmMapSize = 0, pmMapCap = 0, pmCap = 0;
    uint32_t* pmMap = nullptr;
    float4* pmPhotons = nullptr;
    uint32_t* pmCount = nullptr;
    // importon map light tracer: G-buffer (float4 + float per pixel), zeroed when allocated
    void* imBlock = nullptr;
    size_t imPixels = 0;
    // batched rendering: job table + path offsets (device, pinned staging) and the replayed graph
    RenderConst *dJobs = nullptr, *hJobs = nullptr;
    uint32_t *dOffsets = nullptr, *hOffsets = nullptr;
    uint32_t jobCap = 0;
    cudaGraphExec_t batchExec = nullptr;
    std::vector<uintptr_t> batchKey;  // what the captured launches depend on
    // radiance-cache frames alternate over up to kMaxLanes lanes (this set
    // on the context's stream, extra[l - 1] on xstream[l - 1]), so a frame's
    // wavefront tail overlaps the next frames'; the events order the
    // network's inference and training across the lanes
    static constexpr int kMaxLanes = 4;
    RenderBuffers* extra[kMaxLanes - 1] = {};
    cudaStream_t xstream[kMaxLanes - 1] = {};
    cudaEvent_t evSync[kMaxLanes] = {}, evTrain[kMaxLanes] = {};
};

// Wait (host) for the extra lanes' streams of the context's wavefront buffers.
static void sync_lanes(gpugi_ctx* ctx) {
    if (RenderBuffers* r0 = static_cast<RenderBuffers*>(ctx->render))
        for (cudaStream_t st : r0->xstream)
            if (st) cudaStreamSynchronize(st);
}

static void free_rb(RenderBuffers* rb) {
    if (!rb) return;
    for (RenderBuffers* x : rb->extra) free_rb(x);
    for (cudaStream_t st : rb->xstream)
        if (st) cudaStreamDestroy(st);
    for (int l = 0; l < RenderBuffers::kMaxLanes; ++l) {
        if (rb->evSync[l]) cudaEventDestroy(rb->evSync[l]);
        if (rb->evTrain[l]) cudaEventDestroy(rb->evTrain[l]);
    }
    if (rb->batchExec) cudaGraphExecDestroy(rb->batchExec);
    if (rb->dJobs) cudaFree(rb->dJobs);
    if (rb->dOffsets) cudaFree(rb->dOffsets);
    if (rb->hJobs) cudaFreeHost(rb->hJobs);
    if (rb->hOffsets) cudaFreeHost(rb->hOffsets);
    if (rb->block) cudaFree(rb->block);
    if (rb->nrcBlock) cudaFree(rb->nrcBlock);
    if (rb->pmBlock) cudaFree(rb->pmBlock);
    if (rb->imBlock) cudaFree(rb->imBlock);
    if (rb->hostLights) cudaFreeHost(rb->hostLights);
    delete rb;
}

static void free_render(gpugi_ctx* ctx) {
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if (!rb) return;
    sync_lanes(ctx);
    free_rb(rb);
    ctx->render = nullptr;
}

static gpugi_status ensure_buffers_in(gpugi_ctx* ctx, RenderBuffers* rb, size_t paths, size_t cacheBytes,
                                      size_t lightBytes, uint32_t samples);

static gpugi_status ensure_buffers(gpugi_ctx* ctx, size_t paths, size_t cacheBytes, size_t lightBytes,
                                   uint32_t samples) {
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if (!rb) {
        rb = new RenderBuffers();
        ctx->render = rb;
        ctx->renderFree = free_render;
    }
    return ensure_buffers_in(ctx, rb, paths, cacheBytes, lightBytes, samples);
}

static gpugi_status ensure_buffers_in(gpugi_ctx* ctx, RenderBuffers* rb, size_t paths, size_t cacheBytes,
                                      size_t lightBytes, uint32_t samples) {
    if (paths <= rb->pathCap && cacheBytes <= rb->cacheBytes && lightBytes <= rb->lightBytes &&
        samples <= rb->maxSamples)
        return GPUGI_OK;
    cudaStreamSynchronize(ctx->stream);
    sync_lanes(ctx);
    if (rb->block) cudaFree(rb->block);
    rb->block = nullptr;
    paths = std::max(paths, rb->pathCap);
    cacheBytes = std::max(cacheBytes, rb->cacheBytes);
    lightBytes = std::max(lightBytes, rb->lightBytes);
    samples = std::max(samples, rb->maxSamples);
    auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t col = a(paths * 4);
    const size_t total = 2 * 14 * col + 4 * col + 13 * col + a(sizeof(Counters)) + a(cacheBytes) +
                         a(4 * (size_t)samples) + a(lightBytes);
    if (cudaMalloc(&rb->block, total) != cudaSuccess) {
        rb->block = nullptr;
        rb->pathCap = rb->cacheBytes = rb->lightBytes = 0;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "wavefront buffer allocation failed");
    }
    char* p = static_cast<char*>(rb->block);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += a(bytes);
        return r;
    };
    for (PathSoA* P : {&rb->A, &rb->B}) {
        float** f[] = {&P->ox, &P->oy, &P->oz, &P->dx, &P->dy, &P->dz, &P->tx, &P->ty, &P->tz, &P->lastP};
        for (float** q : f) *q = reinterpret_cast<float*>(take(col));
        P->seed = reinterpret_cast<uint32_t*>(take(col));
        P->pixel = reinterpret_cast<uint32_t*>(take(col));
        P->info = reinterpret_cast<uint32_t*>(take(col));
        P->job = reinterpret_cast<uint32_t*>(take(col));
    }
    rb->H.slot = reinterpret_cast<int32_t*>(take(col));
    rb->H.t = reinterpret_cast<float*>(take(col));
    rb->H.u = reinterpret_cast<float*>(take(col));
    rb->H.v = reinterpret_cast<float*>(take(col));
    float** qf[] = {&rb->Q.ox, &rb->Q.oy, &rb->Q.oz, &rb->Q.dx, &rb->Q.dy, &rb->Q.dz, &rb->Q.tmax, &rb->Q.cr,
                    &rb->Q.cg, &rb->Q.cb};
    for (float** q : qf) *q = reinterpret_cast<float*>(take(col));
    rb->Q.pixel = reinterpret_cast<uint32_t*>(take(col));
    rb->Q.train = reinterpret_cast<uint32_t*>(take(col));
    rb->Q.job = reinterpret_cast<uint32_t*>(take(col));
    rb->cnt = reinterpret_cast<Counters*>(take(sizeof(Counters)));
    rb->cache = reinterpret_cast<CacheEntry*>(take(cacheBytes));
    rb->cacheCount = reinterpret_cast<uint32_t*>(take(4 * (size_t)samples));
    rb->lights = reinterpret_cast<float4*>(take(lightBytes));
    rb->pathCap = paths;
    rb->cacheBytes = cacheBytes;
    rb->lightBytes = lightBytes;
    rb->maxSamples = samples;
    return GPUGI_OK;
}

static gpugi_status walkers_config(gpugi_ctx* ctx, const gpugi_scene* sc, Walkers& W) {
    W.bounds = (int)sc->dev.boundsKind;
    const void* ke = W.bounds == 1 ? (const void*)k_extend<1>
                     : W.bounds == 2 ? (const void*)k_extend<2> : (const void*)k_extend<0>;
    const void* ks = W.bounds == 1 ? (const void*)k_shadow<1>
                     : W.bounds == 2 ? (const void*)k_shadow<2> : (const void*)k_shadow<0>;
    gpugi_status st = walker_launch_config(ctx, sc, ke, 1ull << 40, ctx->renderSharedNodes, W.LE);
    if (!st) st = walker_launch_config(ctx, sc, ks, 1ull << 40, ctx->renderSharedNodes, W.LS);
    // group walks while fewer rays than twice the resident lanes are queued
    // (trace modes 3-5; the lane walk otherwise; measured on the passes
    // workload: 0.5x, 2x, 8x, 64x the lanes gave PT 262 / 264.5 / 250 / 167 M
    // samples/s and the photon mapper 124 / 133 / 133 / 133)
    const bool group = ctx->traceMode >= 3;
    W.groupBelowE = group ? W.LE.grid * 128u * GPUGI_GROUP_BELOW_LANES : 0u;
    W.groupBelowS = group ? W.LS.grid * 128u * GPUGI_GROUP_BELOW_LANES : 0u;
    return st;
}

static void launch_extend(gpugi_ctx* ctx, const Walkers& W, const RenderConst& rc, const PathSoA& A, const HitSoA& H,
                          int depth) {
    const WalkerLaunch& L = W.LE;
    if (W.bounds == 1) k_extend<1><<<L.grid, 128, L.smem, ctx->stream>>>(rc, A, H, depth, L.stage, W.groupBelowE);
    else if (W.bounds == 2) k_extend<2><<<L.grid, 128, L.smem, ctx->stream>>>(rc, A, H, depth, L.stage, W.groupBelowE);
    else k_extend<0><<<L.grid, 128, L.smem, ctx->stream>>>(rc, A, H, depth, L.stage, W.groupBelowE);
}

static void launch_shadow(gpugi_ctx* ctx, const Walkers& W, const RenderConst& rc, const ShadowSoA& Q, int depth) {
    const WalkerLaunch& L = W.LS;
    if (W.bounds == 1) k_shadow<1><<<L.grid, 128, L.smem, ctx->stream>>>(rc, Q, depth, L.stage, W.groupBelowS);
    else if (W.bounds == 2) k_shadow<2><<<L.grid, 128, L.smem, ctx->stream>>>(rc, Q, depth, L.stage, W.groupBelowS);
    else k_shadow<0><<<L.grid, 128, L.smem, ctx->stream>>>(rc, Q, depth, L.stage, W.groupBelowS);
}

// One chunk of `samples` iterations of a pass.
static gpugi_status render_chunk(gpugi_ctx* ctx, const gpugi_scene* sc, RenderConst rc, uint32_t pass) {
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    const int bounds = (int)sc->dev.boundsKind;
    Walkers W;
    gpugi_status cst = walkers_config(ctx, sc, W);
    if (cst) return cst;
    int gridShade = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gridShade, (const void*)k_pt_shade, 128, 0);
    gridShade = ctx->numSMs * std::max(gridShade, 1);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.cnt, 0, offsetof(Counters, rays), ctx->stream));
    PathSoA A = rb->A, B = rb->B;

    auto bounces = [&](int kind /*0 PT, 1 light, 2 light+cache, 3 BPT eye, 4 Whitted*/) -> gpugi_status {
        for (int depth = 0; depth < rc.maxPathLength; ++depth) {
            launch_extend(ctx, W, rc, A, rb->H, depth);
            if (kind == 0) k_pt_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth);
            else if (kind == 3) k_bpt_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth);
            else if (kind == 4) k_whitted_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth);
            else k_light_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth, kind == 2);
            launch_shadow(ctx, W, rc, rb->Q, depth);
            std::swap(A, B);
        }
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        return GPUGI_OK;
    };
    const int genBlocks = ctx->numSMs * 8;
    gpugi_status st;
    if (pass == GPUGI_PASS_PT) {
        k_camera_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A, false);
        if ((st = bounces(0))) return st;
    } else if (pass == GPUGI_PASS_WHITTED) {
        k_whitted_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A);
        if ((st = bounces(4))) return st;
    } else if (pass == GPUGI_PASS_PM) {
        // PhotonMapper::Draw (photonmapper.cpp:79-114): clear the grid, distribute
        // the photons of this iteration, gather (one iteration per call)
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.pmMap, 0xFF, 8 * (size_t)rc.pmMapSize, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.pmCount, 0, 4, ctx->stream));
        k_photon_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A);
        for (int depth = 0; depth < rc.maxPathLength; ++depth) {
            launch_extend(ctx, W, rc, A, rb->H, depth);
            k_photon_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, depth);
            std::swap(A, B);
        }
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.cnt, 0, offsetof(Counters, rays), ctx->stream));
        A = rb->A;
        B = rb->B;
        k_pm_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A);
        for (int depth = 0; depth < rc.maxPathLength; ++depth) {
            launch_extend(ctx, W, rc, A, rb->H, depth);
            k_pm_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, depth);
            std::swap(A, B);
        }
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    } else if (pass == GPUGI_PASS_IM) {
        // PixelMapLighttracer::Draw (pixelmaplighttracer.cpp:76-116): clear the
        // grid, the eye pass stores the importons, then the photons are traced
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.pmMap, 0xFF, 8 * (size_t)rc.pmMapSize, ctx->stream));
        k_im_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A);
        for (int depth = 0; depth < rc.maxPathLength; ++depth) {
            launch_extend(ctx, W, rc, A, rb->H, depth);
            k_im_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, depth);
            std::swap(A, B);
        }
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.cnt, 0, offsetof(Counters, rays), ctx->stream));
        A = rb->A;
        B = rb->B;
        k_photon_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A);
        for (int depth = 0; depth < rc.maxPathLength; ++depth) {
            launch_extend(ctx, W, rc, A, rb->H, depth);
            k_im_photon_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, depth);
            std::swap(A, B);
        }
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    } else if (pass == GPUGI_PASS_LT) {
        k_light_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A, false);
        if ((st = bounces(1))) return st;
        if (bounds == 1) k_show_light_samples<1><<<ctx->numSMs, 128, 0, ctx->stream>>>(rc);
        else if (bounds == 2) k_show_light_samples<2><<<ctx->numSMs, 128, 0, ctx->stream>>>(rc);
        else k_show_light_samples<0><<<ctx->numSMs, 128, 0, ctx->stream>>>(rc);
    } else {
        k_light_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A, true);
        if ((st = bounces(2))) return st;
        // The eye pass reuses the queues: its counters start from zero again.
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.cnt, 0, offsetof(Counters, rays), ctx->stream));
        A = rb->A;
        B = rb->B;
        k_camera_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A, true);
        if ((st = bounces(3))) return st;
    }
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}


// LightPathtracer::SetScreenSize (gpugi/renderer/lightpathtracer.cpp:34):
// particles per light sample and iteration.
static uint32_t rays_per_light_sample(const gpugi_render_params* p) {
    return std::max<uint32_t>(64u, (p->width * p->height / p->numLightSamples / 64u) * 64u);
}

static RenderConst make_render_const(gpugi_ctx* ctx, const gpugi_scene* sc, const gpugi_camera* cam,
                                     const gpugi_render_params* p, gpugi_image* im, RenderBuffers* rb) {
    RenderConst rc{};
    rc.s = sc->dev;
    rc.camU = f3(cam->U[0], cam->U[1], cam->U[2]);
    rc.camV = f3(cam->V[0], cam->V[1], cam->V[2]);
    rc.camW = f3(cam->W[0], cam->W[1], cam->W[2]);
    rc.camPos = f3(cam->position[0], cam->position[1], cam->position[2]);
    rc.pixelArea = cam->pixelArea;
    rc.width = (int)p->width;
    rc.height = (int)p->height;
    rc.numPixels = (int)(p->width * p->height);
    rc.maxPathLength = (int)p->maxPathLength;
    rc.rrStartDepth = (int)p->rrStartDepth;
    rc.iteration = p->iteration;
    rc.pass = p->pass;
    rc.rng = (p->flags & GPUGI_RENDER_REFERENCE_RNG) ? 0u : 1u;
    rc.numLightSamples = p->numLightSamples;
    rc.sky = f3(p->sky[0], p->sky[1], p->sky[2]);
    rc.image = im->rgba;
    rc.image64 = im->rgb64;
    rc.cache = rb->cache;
    rc.cacheCount = rb->cacheCount;
    rc.cnt = rb->cnt;
    rc.err = ctx->errWord;
    rc.lightSamples = rb->lights;
    return rc;
}

// Light samples of `ns` iterations into the pinned staging buffer and on to
// the device (host sampler or caller's arrays).
static gpugi_status upload_light_sets(gpugi_ctx* ctx, const gpugi_scene* sc, RenderBuffers* rb, const float* lightSamples,
                                      uint64_t* rngState, uint32_t first, uint32_t ns, uint32_t numLightSamples) {
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // the staging buffer may still feed a copy
    const size_t setFloats = (size_t)numLightSamples * 8;
    if (lightSamples) {
        std::memcpy(rb->hostLights, lightSamples + (size_t)first * setFloats, ns * setFloats * sizeof(float));
    } else {
        for (uint32_t s = 0; s < ns; ++s)
            generate_light_samples(const_cast<gpugi_scene*>(sc), *rngState, numLightSamples,
                                   rb->hostLights + s * setFloats);
    }
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rb->lights, rb->hostLights, ns * setFloats * sizeof(float),
                                        cudaMemcpyHostToDevice, ctx->stream));
    return GPUGI_OK;
}

static gpugi_status ensure_nrc_buffers(gpugi_ctx* ctx, RenderBuffers* rb, size_t queries, size_t trainPaths,
                                       size_t stride, size_t samples) {
    if (queries <= rb->nrcQueryCap && trainPaths <= rb->nrcTrainCap && stride <= rb->nrcStride &&
        samples <= rb->nrcSampleCap)
        return GPUGI_OK;
    cudaStreamSynchronize(ctx->stream);
    sync_lanes(ctx);
    if (rb->nrcBlock) cudaFree(rb->nrcBlock);
    rb->nrcBlock = nullptr;
    queries = std::max(queries, rb->nrcQueryCap);
    trainPaths = std::max(trainPaths, rb->nrcTrainCap);
    stride = std::max(stride, rb->nrcStride);
    samples = std::max(samples, rb->nrcSampleCap);
    auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t verts = trainPaths * stride;
    const size_t total = a(queries * 48) + a(queries * 12) + a(queries * 4) + a(queries * 12) + a(verts * 64) +
                         a(verts * 12) + a(trainPaths * 4) + a(samples * 60) + a(64);
    if (cudaMalloc(&rb->nrcBlock, total) != cudaSuccess) {
        rb->nrcBlock = nullptr;
        rb->nrcQueryCap = rb->nrcTrainCap = rb->nrcStride = rb->nrcSampleCap = 0;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "radiance-cache buffers");
    }
    char* p = static_cast<char*>(rb->nrcBlock);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += a(bytes);
        return r;
    };
    rb->queries = reinterpret_cast<float*>(take(queries * 48));
    rb->qT = reinterpret_cast<float*>(take(queries * 12));
    rb->qPixel = reinterpret_cast<uint32_t*>(take(queries * 4));
    rb->radiance = reinterpret_cast<float*>(take(queries * 12));
    rb->tvRec = reinterpret_cast<float*>(take(verts * 64));
    rb->tvC = reinterpret_cast<float*>(take(verts * 12));
    rb->tvCount = reinterpret_cast<uint32_t*>(take(trainPaths * 4));
    rb->samples = reinterpret_cast<float*>(take(samples * 60));
    rb->nrcCounters = reinterpret_cast<uint32_t*>(take(64));
    rb->nrcQueryCap = queries;
    rb->nrcTrainCap = trainPaths;
    rb->nrcStride = stride;
    rb->nrcSampleCap = samples;
    return GPUGI_OK;
}

// Smallest prime >= n (the hash table size, photonmapper.cpp:138-143).
static size_t next_prime(size_t n) {
    if (n <= 2) return 2;
    for (size_t c = n | 1;; c += 2) {
        bool prime = true;
        for (size_t d = 3; d * d <= c && prime; d += 2) prime = c % d != 0;
        if (prime) return c;
    }
}

// Hash table of at least mapMin entries (a prime) and cap records of 32
// bytes. The photon mapper asks for 1.5x the photons of an iteration and a
// record for every diffuse bounce of every photon (never overflows); the
// importon map for 1.5x the pixels and one record per pixel
// (pixelmaplighttracer.cpp:150-158).
static gpugi_status ensure_pm_buffers(gpugi_ctx* ctx, RenderBuffers* rb, uint64_t mapMin, uint64_t records) {
    // The block only grows: the photon mapper (1.5 x photons) and the
    // importon map (1.5 x pixels) ask for different table sizes, and a switch
    // between them must not free and allocate again (which synchronises).
    // pmMapSize is the prime in use, pmMapCap the table entries allocated.
    const size_t mapSize = next_prime((size_t)mapMin);
    const size_t cap = (size_t)records;
    if (mapSize <= rb->pmMapCap && cap <= rb->pmCap) {
        rb->pmMapSize = mapSize;
        return GPUGI_OK;
    }
    const size_t mapCap = mapSize > rb->pmMapCap ? mapSize : rb->pmMapCap;
    const size_t recCap = cap > rb->pmCap ? cap : rb->pmCap;
    cudaStreamSynchronize(ctx->stream);
    if (rb->pmBlock) cudaFree(rb->pmBlock);
    rb->pmBlock = nullptr;
    rb->pmMapSize = rb->pmMapCap = rb->pmCap = 0;
    const size_t mapBytes = (8 * mapCap + 255) & ~size_t(255), photonBytes = 32 * recCap;
    if (cudaMalloc(&rb->pmBlock, mapBytes + photonBytes + 256) != cudaSuccess) {
        rb->pmBlock = nullptr;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "photon map buffers");
    }
    char* base = static_cast<char*>(rb->pmBlock);
    rb->pmMap = reinterpret_cast<uint32_t*>(base);
    rb->pmPhotons = reinterpret_cast<float4*>(base + mapBytes);
    rb->pmCount = reinterpret_cast<uint32_t*>(base + mapBytes + photonBytes);
    rb->pmMapSize = mapSize;
    rb->pmMapCap = mapCap;
    rb->pmCap = recCap;
    return GPUGI_OK;
}

// G-buffer of the importon map light tracer, zeroed when allocated and at
// the first iteration of an accumulation (PixelMapLighttracer::SetScreenSize,
// pixelmaplighttracer.cpp:63-65).
static gpugi_status ensure_im_buffers(gpugi_ctx* ctx, RenderBuffers* rb, size_t pixels, bool clear) {
    if (pixels > rb->imPixels) {
        cudaStreamSynchronize(ctx->stream);
        if (rb->imBlock) cudaFree(rb->imBlock);
        rb->imBlock = nullptr;
        rb->imPixels = 0;
        if (cudaMalloc(&rb->imBlock, 20 * pixels) != cudaSuccess) {
            rb->imBlock = nullptr;
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "importon map G-buffer");
        }
        rb->imPixels = pixels;
        clear = true;
    }
    if (clear) GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rb->imBlock, 0, 20 * rb->imPixels, ctx->stream));
    return GPUGI_OK;
}

// Query radius of an iteration: fixed, or shrunk by Knaus-Zwicker's
// r_k = r_(k-1) sqrt((k + 0.7) / (k + 1)) from iteration 1 on
// (photonmapper.cpp:84-87, pixelmaplighttracer.cpp:82-87), in closed form
// through log-gamma.
static float grid_radius(double r0, bool progressive, uint32_t iteration) {
    if (!progressive || iteration == 0) return (float)r0;
    const double k = iteration;
    const double logProd = std::lgamma(k + 1.7) - std::lgamma(1.7) - (std::lgamma(k + 2.0) - std::lgamma(2.0));
    return (float)(r0 * std::exp(0.5 * logProd));
}

static gpugi_status ensure_host_lights(gpugi_ctx* ctx, RenderBuffers* rb, size_t lightBytes) {
    if (rb->hostLightBytes >= lightBytes) return GPUGI_OK;
    if (rb->hostLights) cudaFreeHost(rb->hostLights);
    rb->hostLights = nullptr;
    rb->hostLightBytes = 0;
    GPUGI_CUDA_TRY(ctx, cudaMallocHost(&rb->hostLights, lightBytes));
    rb->hostLightBytes = lightBytes;
    return GPUGI_OK;
}

}  // namespace gpugi

using namespace gpugi;

extern "C" {

gpugi_status gpugi_image_create(gpugi_ctx* ctx, uint32_t width, uint32_t height, uint32_t flags, gpugi_image** out) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!out || width == 0 || height == 0 || (uint64_t)width * height > (1ull << 31))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad image size");
    gpugi_image* im = new gpugi_image();
    attach_child(ctx, &im->ctx);
    im->width = width;
    im->height = height;
    im->flags = flags;
    const size_t n = (size_t)width * height;
    if (cudaMalloc(&im->rgba, n * sizeof(float4)) != cudaSuccess ||
        ((flags & 1u) && cudaMalloc(&im->rgb64, n * 3 * sizeof(double)) != cudaSuccess)) {
        gpugi_image_destroy(im);
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "image allocation failed");
    }
    *out = im;
    return gpugi_image_clear(ctx, im);
}

void gpugi_image_destroy(gpugi_image* im) {
    if (!im) return;
    if (im->ctx) cudaStreamSynchronize(im->ctx->stream);
    detach_child(&im->ctx);
    if (im->rgba) cudaFree(im->rgba);
    if (im->rgb64) cudaFree(im->rgb64);
    delete im;
}

gpugi_status gpugi_image_clear(gpugi_ctx* ctx, gpugi_image* im) {
    if (!ctx || !im) return GPUGI_ERROR_INVALID_ARGUMENT;
    const size_t n = (size_t)im->width * im->height;
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(im->rgba, 0, n * sizeof(float4), ctx->stream));
    if (im->rgb64) GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(im->rgb64, 0, n * 3 * sizeof(double), ctx->stream));
    return GPUGI_OK;
}

gpugi_status gpugi_image_read(gpugi_ctx* ctx, const gpugi_image* im, float* rgba, double* rgb64) {
    if (!ctx || !im) return GPUGI_ERROR_INVALID_ARGUMENT;
    const size_t n = (size_t)im->width * im->height;
    if (rgba) GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rgba, im->rgba, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    if (rgb64) {
        if (!im->rgb64) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "image has no FP64 accumulation");
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rgb64, im->rgb64, n * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return gpugi_sync(ctx);
}

gpugi_status gpugi_image_write(gpugi_ctx* ctx, gpugi_image* im, const float* rgba, const double* rgb64) {
    if (!ctx || !im) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!rgba) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "rgba is required");
    if (rgb64 && !im->rgb64) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "image has no FP64 accumulation");
    const size_t n = (size_t)im->width * im->height;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(im->rgba, rgba, n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
    if (im->rgb64) {
        if (rgb64)
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(im->rgb64, rgb64, n * 3 * sizeof(double), cudaMemcpyHostToDevice,
                                                ctx->stream));
        else
            GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(im->rgb64, 0, n * 3 * sizeof(double), ctx->stream));
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return GPUGI_OK;
}

gpugi_status gpugi_image_mse(gpugi_ctx* ctx, const gpugi_image* im, double divisor, const float* reference,
                             uint32_t useFp64, double* mse) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!im || !reference || !mse || !(divisor > 0.0))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad argument");
    if (useFp64 && !im->rgb64) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "image has no FP64 accumulation");
    const size_t n = (size_t)im->width * im->height;
    gpugi_status st = ensure_stage(ctx, 256 + n * 3 * sizeof(float));
    if (st) return st;
    double* dSum = static_cast<double*>(ctx->stageDev);
    float* dRef = reinterpret_cast<float*>(static_cast<char*>(ctx->stageDev) + 256);
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dRef, reference, n * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(dSum, 0, sizeof(double), ctx->stream));
    k_mse<<<ctx->numSMs * 4, 256, 0, ctx->stream>>>(im->rgba, useFp64 ? im->rgb64 : nullptr, dRef, n, 1.0 / divisor,
                                                   dSum);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    double sum = 0.0;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&sum, dSum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *mse = sum / (double)n;
    return GPUGI_OK;
}

gpugi_status gpugi_render_ray_counts(gpugi_ctx* ctx, uint64_t counts[2]) {
    if (!ctx || !counts) return GPUGI_ERROR_INVALID_ARGUMENT;
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if (!rb) {
        counts[0] = counts[1] = 0;
        return GPUGI_OK;
    }
    unsigned long long c[2];
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(c, rb->cnt->rays, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    counts[0] = c[0];
    counts[1] = c[1];
    return GPUGI_OK;
}

gpugi_status gpugi_render(gpugi_ctx* ctx, const gpugi_scene* sc, const gpugi_camera* cam,
                          const gpugi_render_params* p, const float* lightSamples, uint64_t* rngState,
                          gpugi_image* im) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || !cam || !p || !im) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (p->pass > GPUGI_PASS_IM) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown pass");
    if (p->flags & ~GPUGI_RENDER_KNOWN_FLAGS) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown render flags");
    if (p->width != im->width || p->height != im->height)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "params size differs from the image");
    if (p->maxPathLength == 0 || p->maxPathLength > (uint32_t)kMaxDepth)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "maxPathLength must be in [1, 64]");
    if (p->numLightSamples == 0 || p->samples == 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "numLightSamples and samples must be > 0");
    if (!sc->dev.vinfo || !sc->dev.materials)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene lacks vertex info or materials");
    if (!lightSamples && !rngState)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "either lightSamples or rngState is required");

    if (p->pass == GPUGI_PASS_HIERARCHY)
        return render_hierarchy(ctx, const_cast<gpugi_scene*>(sc), cam, p, lightSamples, rngState, im);

    const uint32_t numPixels = p->width * p->height;
    const uint32_t raysPerLight = rays_per_light_sample(p);
    const uint32_t lightThreads = raysPerLight * p->numLightSamples;
    // Whitted: up to two shadow rays per path, so the queues get twice the paths
    const bool pm = p->pass == GPUGI_PASS_PM, imap = p->pass == GPUGI_PASS_IM, grid = pm || imap;
    const uint64_t photons =
        grid ? (uint64_t)p->numLightSamples * (imap ? ctx->imPhotonsPerSample : ctx->pmPhotonsPerSample) : 0;
    if (photons > (64ull << 20)) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "more than 64M photons per iteration");
    const uint32_t perSamplePaths = p->pass == GPUGI_PASS_PT        ? numPixels
                                    : p->pass == GPUGI_PASS_WHITTED ? 2 * numPixels
                                    : grid                          ? std::max<uint32_t>(numPixels, (uint32_t)photons)
                                                                    : std::max(numPixels, lightThreads);
    // Light-cache capacity: the worst case (every particle stores its light
    // sample plus one entry per bounce) so it can never overflow.
    const uint64_t cachePerSample = p->pass == GPUGI_PASS_BPT ? (uint64_t)lightThreads * (p->maxPathLength + 1) : 0;
    // Samples per chunk: at most 16M paths and 4 GiB of light cache in flight.
    uint64_t chunk = std::max<uint64_t>(1, (16ull << 20) / perSamplePaths);
    if (cachePerSample) chunk = std::min<uint64_t>(chunk, std::max<uint64_t>(1, (4ull << 30) / (cachePerSample * 64)));
    chunk = std::min<uint64_t>(chunk, p->samples);
    if (grid) chunk = 1;  // one photon (importon) map per iteration
    const size_t lightBytes = chunk * p->numLightSamples * 32;
    gpugi_status st = ensure_buffers(ctx, chunk * perSamplePaths, chunk * cachePerSample * 64, lightBytes,
                                     (uint32_t)chunk);
    if (st) return st;
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if ((st = ensure_host_lights(ctx, rb, lightBytes))) return st;
    if (pm && (st = ensure_pm_buffers(ctx, rb, photons * 3 / 2, photons * p->maxPathLength))) return st;
    if (imap && ((st = ensure_pm_buffers(ctx, rb, (uint64_t)numPixels * 3 / 2, numPixels)) ||
               (st = ensure_im_buffers(ctx, rb, numPixels, p->iteration == 0))))
        return st;

    RenderConst rc = make_render_const(ctx, sc, cam, p, im, rb);
    rc.numRaysPerLightSample = (int)raysPerLight;
    rc.lightThreads = lightThreads;
    rc.cacheCap = (uint32_t)cachePerSample;
    if (pm) {
        rc.pmMap = rb->pmMap;
        rc.pmMapSize = (uint32_t)rb->pmMapSize;
        rc.pmPhotons = rb->pmPhotons;
        rc.pmCount = rb->pmCount;
        rc.pmCap = (uint32_t)(photons * p->maxPathLength);
        rc.photonsPerSample = (int)ctx->pmPhotonsPerSample;
    }
    if (imap) {
        rc.pmMap = rb->pmMap;
        rc.pmMapSize = (uint32_t)rb->pmMapSize;
        rc.pmPhotons = rb->pmPhotons;
        rc.pmCount = rb->pmCount;
        rc.pmCap = numPixels;
        rc.photonsPerSample = (int)ctx->imPhotonsPerSample;
        rc.imGbuf = static_cast<float4*>(rb->imBlock);
        rc.imGbufN0 = reinterpret_cast<float*>(static_cast<char*>(rb->imBlock) + 16 * (size_t)numPixels);
    }
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rb->cnt, 0, sizeof(Counters), ctx->stream));
    for (uint32_t s0 = 0; s0 < p->samples; s0 += (uint32_t)chunk) {
        const uint32_t ns = std::min<uint32_t>((uint32_t)chunk, p->samples - s0);
        if ((st = upload_light_sets(ctx, sc, rb, lightSamples, rngState, s0, ns, p->numLightSamples))) return st;
        rc.samples = ns;
        rc.sampleBase = s0;
        if (grid) {
            const float r = imap ? grid_radius(ctx->imQueryRadius, ctx->imProgressive, p->iteration + s0)
                               : grid_radius(ctx->pmQueryRadius, ctx->pmProgressive, p->iteration + s0);
            rc.pmRadiusSq = r * r;
            rc.pmSpacing = r * 2.01f;
        }
        if ((st = render_chunk(ctx, sc, rc, p->pass))) return st;
    }
    return GPUGI_OK;
}


gpugi_status gpugi_render_nrc(gpugi_ctx* ctx, const gpugi_scene* sc, const gpugi_camera* cam,
                              const gpugi_render_params* p, const float* lightSamples, uint64_t* rngState,
                              gpugi_nrc* nn, const gpugi_nrc_params* np, gpugi_image* im) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || !cam || !p || !im || !nn || !np) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (p->pass != GPUGI_PASS_PT && p->pass != GPUGI_PASS_BPT)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "the radiance cache serves the PT and BPT passes");
    if (p->flags & ~GPUGI_RENDER_KNOWN_FLAGS) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown render flags");
    const bool bpt = p->pass == GPUGI_PASS_BPT;
    if (p->width != im->width || p->height != im->height)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "params size differs from the image");
    if (p->maxPathLength == 0 || p->maxPathLength > (uint32_t)kMaxDepth || p->numLightSamples == 0 ||
        p->samples == 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad render parameters");
    if (!sc->dev.vinfo || !sc->dev.materials)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene lacks vertex info or materials");
    if (!lightSamples && !rngState)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "either lightSamples or rngState is required");
    if (!(np->trainFraction >= 0.0f && np->trainFraction <= 1.0f))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "trainFraction must be in [0, 1]");
    if (!(np->unbiasedFraction >= 0.0f && np->unbiasedFraction <= 1.0f) || !(np->terminateSpread >= 0.0f) ||
        np->trainLength >= p->maxPathLength + 1u)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT,
                    "unbiasedFraction must be in [0, 1], terminateSpread >= 0, trainLength <= maxPathLength");
    const uint32_t numPixels = p->width * p->height;
    const uint32_t spf = std::max<uint32_t>(1u, std::min(np->samplesPerFrame, p->samples));
    if ((uint64_t)spf * numPixels > (64ull << 20))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "samplesPerFrame x pixels exceeds 64M paths");
    const uint32_t framePaths = spf * numPixels;
    // light samples go up in blocks of whole frames (up to 64 MB), so the
    // staging buffer is reused, and waited for, once per block
    const size_t setBytes = (size_t)p->numLightSamples * 32;
    uint32_t blockFrames = (uint32_t)std::min<size_t>((p->samples + spf - 1) / spf,
                                                      std::max<size_t>(1, (64u << 20) / (setBytes * spf)));
    const uint32_t blockSamples = blockFrames * spf;
    const size_t lightBytes = (size_t)blockSamples * setBytes;
    // BPT: light particles per sample as LightPathtracer::SetScreenSize
    // (gpugi/renderer/lightpathtracer.cpp:34); the light pass only needs
    // min(maxPathLength, terminateDepth) bounces, since longer paths are the
    // cache's; training paths come on top of the render paths.
    uint32_t lightThreads = 0, raysPerLight = 0, lightDepth = 0, nTrain = 0;
    uint64_t cachePerSample = 0;
    size_t paths = framePaths;
    if (bpt) {
        raysPerLight = std::max<uint32_t>(64u, (numPixels / p->numLightSamples / 64u) * 64u);
        lightThreads = raysPerLight * p->numLightSamples;
        lightDepth = std::min(p->maxPathLength, np->terminateDepth);
        cachePerSample = (uint64_t)lightThreads * (lightDepth + 1);
        nTrain = np->train ? (uint32_t)(np->trainFraction * (double)framePaths) : 0u;
        paths = std::max<size_t>((size_t)framePaths + nTrain, (size_t)spf * lightThreads);
    }
    gpugi_status st = ensure_buffers(ctx, paths, (size_t)spf * cachePerSample * 64, lightBytes, spf);
    if (st) return st;
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if ((st = ensure_host_lights(ctx, rb, lightBytes))) return st;
    const size_t trainCap = bpt ? (size_t)nTrain + 64 : (size_t)(np->trainFraction * framePaths * 1.25) + 64;
    const size_t sampleCap = np->maxTrainSamples ? np->maxTrainSamples : 65536;
    if ((uint64_t)trainCap * p->maxPathLength >= (uint64_t)kTrainQuery)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "too many training vertices per frame");
    // queries: one per render path, and one per self-training path
    const size_t queryCap = (size_t)framePaths + (np->trainLength ? trainCap : 0);
    if ((st = ensure_nrc_buffers(ctx, rb, queryCap, trainCap, p->maxPathLength, sampleCap))) return st;

    // Frames alternate over `lanes` lanes (buffer sets and streams; 4 by
    // default): a frame's wavefront tail overlaps the next frames' bulk. The
    // network's inference and training stay in frame order (events), so
    // every frame sees the weights trained by the previous one.
    const uint32_t nFrames = (p->samples + spf - 1) / spf;
    const int nLanes = (int)std::max<uint32_t>(
        1u, std::min<uint32_t>(np->lanes ? std::min<uint32_t>(np->lanes, RenderBuffers::kMaxLanes) : 4u, nFrames));
    RenderBuffers* lanes[RenderBuffers::kMaxLanes] = {rb, rb, rb, rb};
    cudaStream_t streams[RenderBuffers::kMaxLanes] = {ctx->stream, ctx->stream, ctx->stream, ctx->stream};
    if (nLanes > 1 && !rb->evSync[0])
        for (int l = 0; l < RenderBuffers::kMaxLanes; ++l) {
            GPUGI_CUDA_TRY(ctx, cudaEventCreateWithFlags(&rb->evSync[l], cudaEventDisableTiming));
            GPUGI_CUDA_TRY(ctx, cudaEventCreateWithFlags(&rb->evTrain[l], cudaEventDisableTiming));
        }
    for (int l = 1; l < nLanes; ++l) {
        if (!rb->extra[l - 1]) {
            rb->extra[l - 1] = new RenderBuffers();
            GPUGI_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&rb->xstream[l - 1], cudaStreamNonBlocking));
        }
        if ((st = ensure_buffers_in(ctx, rb->extra[l - 1], paths, (size_t)spf * cachePerSample * 64, 0, spf)))
            return st;
        if ((st = ensure_nrc_buffers(ctx, rb->extra[l - 1], queryCap, trainCap, p->maxPathLength, sampleCap)))
            return st;
        lanes[l] = rb->extra[l - 1];
        streams[l] = rb->xstream[l - 1];
    }
    auto lane_const = [&](RenderBuffers* L) {
        RenderConst c = make_render_const(ctx, sc, cam, p, im, L);
        c.nrcTerminateDepth = (int)np->terminateDepth;
        c.nrcTrainThreshold = (uint32_t)std::min(4294967295.0, (double)np->trainFraction * 4294967296.0);
        c.nrcTrainLength = (int)np->trainLength;
        c.nrcUnbiasedThreshold = (uint32_t)std::min(4294967295.0, (double)np->unbiasedFraction * 4294967296.0);
        c.nrcSpread = bpt ? 0.0f : np->terminateSpread;
        c.tvRec = L->tvRec;
        c.tvC = L->tvC;
        c.tvCount = L->tvCount;
        c.trainPaths = L->nrcCounters + 1;
        c.trainCap = (uint32_t)trainCap;
        c.queries = L->queries;
        c.qT = L->qT;
        c.qPixel = L->qPixel;
        c.queryCount = L->nrcCounters;
        c.queryCap = (uint32_t)queryCap;
        c.numRaysPerLightSample = (int)raysPerLight;
        c.lightThreads = lightThreads;
        c.cacheCap = (uint32_t)cachePerSample;
        return c;
    };
    RenderConst rcs[RenderBuffers::kMaxLanes];
    for (int l = 0; l < nLanes; ++l) rcs[l] = lane_const(lanes[l]);
    // The wavefront's bounces: render paths stop by vertex terminateDepth;
    // training paths run to the path's end unless there are none or every
    // one of them stops at trainLength (self-training, no unbiased share).
    const bool trainingEnds = np->trainFraction <= 0.0f || (np->trainLength && np->unbiasedFraction <= 0.0f);
    const int lastDepth = trainingEnds ? std::min<int>((int)p->maxPathLength,
                                                       (int)std::max(np->terminateDepth, np->trainLength) + 1)
                                       : (int)p->maxPathLength;
    Walkers W;
    if ((st = walkers_config(ctx, sc, W))) return st;
    // Frames in flight on several lanes: each lane's walkers launch 150 /
    // lanes percent of the persistent grid (37 % with four lanes), so about
    // one and a half grids of walks run side by side and one frame's walker
    // tails overlap the others' bulk instead of waiting for the SMs a
    // full-grid walker holds (1-spp frames on the 1280 x 720 heightfield:
    // 2.12 ms per frame with full grids, 1.90 at 50 %, 1.84 at 35 %, 1.89
    // at 25 %, 2.15 at 20 %). The group-walk threshold follows the grid.
    if (nLanes > 1) {
        const unsigned share = std::min(100u, 150u / (unsigned)nLanes);
        W.LE.grid = std::max(1u, W.LE.grid * share / 100u);
        W.LS.grid = std::max(1u, W.LS.grid * share / 100u);
        if (W.groupBelowE) W.groupBelowE = W.LE.grid * 128u * GPUGI_GROUP_BELOW_LANES;
        if (W.groupBelowS) W.groupBelowS = W.LS.grid * 128u * GPUGI_GROUP_BELOW_LANES;
    }
    int perSM = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, bpt ? (const void*)k_nrc_bpt_shade : (const void*)k_nrc_shade,
                                                  128, 0);
    const int gridShade = ctx->numSMs * std::max(perSM, 1);
    const int genBlocks = ctx->numSMs * 8;
    const cudaStream_t base = ctx->stream;
    // the library's launch helpers queue on ctx->stream: point it at the
    // frame's lane, and back at the context's stream on every way out
    struct StreamScope {
        gpugi_ctx* c;
        cudaStream_t s;
        ~StreamScope() { c->stream = s; }
    } scope{ctx, base};
    for (int l = 0; l < nLanes; ++l) GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(lanes[l]->cnt, 0, sizeof(Counters), base));
    uint32_t fi = 0;
    for (uint32_t frame = 0; frame < p->samples; frame += spf, ++fi) {
        const uint32_t ns = std::min(spf, p->samples - frame);
        const uint32_t inBlock = frame % blockSamples;
        if (inBlock == 0) {
            // the other lanes have read the previous block of light samples
            for (int l = 1; l < nLanes && fi > 0; ++l) {
                GPUGI_CUDA_TRY(ctx, cudaEventRecord(rb->evSync[l], streams[l]));
                GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(base, rb->evSync[l], 0));
            }
            if ((st = upload_light_sets(ctx, sc, rb, lightSamples, rngState, frame,
                                        std::min(blockSamples, p->samples - frame), p->numLightSamples)))
                return st;
            if (nLanes > 1) GPUGI_CUDA_TRY(ctx, cudaEventRecord(rb->evSync[0], base));
            for (int l = 1; l < nLanes; ++l) GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(streams[l], rb->evSync[0], 0));
        }
        const int li = (int)(fi % (uint32_t)nLanes);
        RenderBuffers* L = lanes[li];
        RenderConst& rc = rcs[li];
        ctx->stream = streams[li];
        rc.lightSamples = rb->lights + 2 * (size_t)inBlock * p->numLightSamples;
        rc.samples = ns;
        rc.sampleBase = frame;
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(L->cnt, 0, offsetof(Counters, rays), ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(L->nrcCounters, 0, 64, ctx->stream));
        PathSoA A = L->A, B = L->B;
        if (bpt) {
            // light pass with the light cache (lighttracer.comp with
            // SAVE_LIGHT_CACHE), bounded to lightDepth bounces
            RenderConst rl = rc;
            rl.maxPathLength = (int)lightDepth;
            k_light_generate<<<genBlocks, 256, 0, ctx->stream>>>(rl, A, true);
            for (int depth = 0; depth < rl.maxPathLength; ++depth) {
                launch_extend(ctx, W, rl, A, L->H, depth);
                k_light_shade<<<gridShade, 128, 0, ctx->stream>>>(rl, A, B, L->H, L->Q, depth, true);
                launch_shadow(ctx, W, rl, L->Q, depth);
                std::swap(A, B);
            }
            GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(L->cnt, 0, offsetof(Counters, rays), ctx->stream));
            A = L->A;
            B = L->B;
            k_nrc_bpt_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A, nTrain);
        } else {
            k_nrc_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A);
        }
        for (int depth = 0; depth < lastDepth; ++depth) {
            launch_extend(ctx, W, rc, A, L->H, depth);
            if (bpt) k_nrc_bpt_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, L->H, L->Q, depth);
            else k_nrc_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, L->H, L->Q, depth);
            launch_shadow(ctx, W, rc, L->Q, depth);
            std::swap(A, B);
        }
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        // cache lookups of this frame with the network as trained by the
        // previous frame (on the other lane); counts stay on the device, so
        // frames queue back to back
        if (nLanes > 1 && fi > 0)
            GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, rb->evTrain[(li + nLanes - 1) % nLanes], 0));
        if ((st = nrc_infer_counted(ctx, nn, L->queries, queryCap, L->nrcCounters, L->radiance))) return st;
        k_nrc_apply<<<ctx->numSMs * 4, 256, 0, ctx->stream>>>(rc, L->radiance);
        // training on this frame's training paths
        if (np->train && np->trainFraction > 0.0f) {
            k_nrc_targets<<<ctx->numSMs * 2, 128, 0, ctx->stream>>>(rc, L->samples, L->nrcCounters + 2,
                                                                     (uint32_t)sampleCap);
            for (uint32_t k = 0; k < std::max<uint32_t>(1u, np->trainSteps); ++k)
                if ((st = nrc_train_counted(ctx, nn, L->samples, sampleCap, L->nrcCounters + 2))) return st;
        }
        if (nLanes > 1) GPUGI_CUDA_TRY(ctx, cudaEventRecord(rb->evTrain[li], ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        ctx->stream = base;
    }
    for (int l = 1; l < nLanes; ++l) {  // the call's work ends on the context's stream, its ray counts in lane 0's
        GPUGI_CUDA_TRY(ctx, cudaEventRecord(rb->evSync[l], streams[l]));
        GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(base, rb->evSync[l], 0));
        k_add_ray_counts<<<1, 32, 0, base>>>(rb->cnt, lanes[l]->cnt);
    }
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}


// Validation shared by gpugi_render and the jobs of gpugi_render_batch.
static gpugi_status check_render_args(gpugi_ctx* ctx, const gpugi_scene* sc, const gpugi_camera* cam,
                                      const gpugi_render_params* p, const float* lightSamples,
                                      const uint64_t* rngState, const gpugi_image* im) {
    if (!sc || !cam || !p || !im) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (p->pass > GPUGI_PASS_IM) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown pass");
    if (p->flags & ~GPUGI_RENDER_KNOWN_FLAGS) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown render flags");
    if (p->width != im->width || p->height != im->height)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "params size differs from the image");
    if (p->maxPathLength == 0 || p->maxPathLength > (uint32_t)kMaxDepth)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "maxPathLength must be in [1, 64]");
    if (p->numLightSamples == 0 || p->samples == 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "numLightSamples and samples must be > 0");
    if (!sc->dev.vinfo || !sc->dev.materials)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene lacks vertex info or materials");
    if (!lightSamples && !rngState)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "either lightSamples or rngState is required");
    return GPUGI_OK;
}

gpugi_status gpugi_set_photon_config(gpugi_ctx* ctx, uint32_t photonsPerLightSample, float queryRadius,
                                     uint32_t progressive) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (photonsPerLightSample == 0 || photonsPerLightSample > (1u << 20))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "photonsPerLightSample must be in [1, 2^20]");
    if (!(queryRadius > 0.0f) || !(queryRadius < 1e30f))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "queryRadius must be positive and finite");
    ctx->pmPhotonsPerSample = photonsPerLightSample;
    ctx->pmQueryRadius = queryRadius;
    ctx->pmProgressive = progressive ? 1u : 0u;
    return GPUGI_OK;
}

gpugi_status gpugi_set_importon_config(gpugi_ctx* ctx, uint32_t photonsPerLightSample, float queryRadius,
                                       uint32_t progressive) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (photonsPerLightSample == 0 || photonsPerLightSample > (1u << 20))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "photonsPerLightSample must be in [1, 2^20]");
    if (!(queryRadius > 0.0f) || !(queryRadius < 1e30f))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "queryRadius must be positive and finite");
    ctx->imPhotonsPerSample = photonsPerLightSample;
    ctx->imQueryRadius = queryRadius;
    ctx->imProgressive = progressive ? 1u : 0u;
    return GPUGI_OK;
}

gpugi_status gpugi_set_batch_config(gpugi_ctx* ctx, uint32_t pathsPerRound, uint32_t useGraph) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (pathsPerRound < 1024 || pathsPerRound > (64u << 20))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "pathsPerRound must be in [1024, 64M]");
    ctx->batchPaths = pathsPerRound;
    ctx->batchGraph = useGraph ? 1u : 0u;
    return GPUGI_OK;
}

gpugi_status gpugi_render_batch(gpugi_ctx* ctx, const gpugi_job* jobs, uint32_t numJobs) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (numJobs && !jobs) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL jobs");
    // The PT, LT and BPT jobs share the wavefront. Per sample a job needs
    // paths0 phase-0 paths (plus extraQ shadow-queue entries: the LT light
    // samples' camera connections), paths1 phase-1 paths and cacheBytes of
    // light cache.
    struct Fused {
        uint32_t job, raysPerLight, lightThreads;
        uint64_t paths0, extraQ, paths1, cacheBytes;
    };
    std::vector<Fused> fused;
    uint32_t depth0 = 0, depth1 = 0;
    uint64_t lightBytes = 0, cacheNeed = 0, maxCache = 0, cacheSamples = 0;
    const uint32_t cap = ctx->batchPaths;
    for (uint32_t j = 0; j < numJobs; ++j) {
        const gpugi_job& J = jobs[j];
        gpugi_status st = check_render_args(ctx, J.scene, &J.camera, &J.params, J.lightSamples, J.rngState, J.image);
        if (st) return st;
        const gpugi_render_params& P = J.params;
        if (P.pass > GPUGI_PASS_BPT) continue;
        Fused F{j, rays_per_light_sample(&P), 0, 0, 0, 0, 0};
        F.lightThreads = F.raysPerLight * P.numLightSamples;
        const uint64_t pix = (uint64_t)P.width * P.height;
        if (P.pass == GPUGI_PASS_PT) {
            F.paths0 = pix;
        } else {
            F.paths0 = F.lightThreads;
            if (P.pass == GPUGI_PASS_LT) F.extraQ = P.numLightSamples;
            else F.paths1 = pix, F.cacheBytes = (uint64_t)F.lightThreads * (P.maxPathLength + 1) * sizeof(CacheEntry);
        }
        if (F.paths0 + F.extraQ > cap || F.paths1 > cap)
            return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "one sample of a job needs more paths than the path queue");
        uint64_t most = std::min<uint64_t>(P.samples, cap / (F.paths0 + F.extraQ));
        if (F.paths1) most = std::min<uint64_t>(most, cap / F.paths1);
        lightBytes += most * P.numLightSamples * 32ull;
        depth0 = std::max(depth0, P.maxPathLength);
        if (P.pass == GPUGI_PASS_BPT) {
            depth1 = std::max(depth1, P.maxPathLength);
            cacheNeed += most * F.cacheBytes;
            maxCache = std::max(maxCache, F.cacheBytes);
            cacheSamples += most;
        }
        fused.push_back(F);
    }
    if (!fused.empty()) {
        const uint32_t nj = (uint32_t)fused.size();
        // light caches of one round: at most 4 GiB, but always one sample of the largest job
        const uint64_t cacheBudget = std::max<uint64_t>(maxCache, std::min<uint64_t>(cacheNeed, 4ull << 30));
        gpugi_status st = ensure_buffers(ctx, cap, cacheBudget, lightBytes, (uint32_t)std::max<uint64_t>(1, cacheSamples));
        if (st) return st;
        RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
        if ((st = ensure_host_lights(ctx, rb, lightBytes))) return st;
        if (nj > rb->jobCap) {
            GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            if (rb->dJobs) cudaFree(rb->dJobs);
            if (rb->dOffsets) cudaFree(rb->dOffsets);
            if (rb->hJobs) cudaFreeHost(rb->hJobs);
            if (rb->hOffsets) cudaFreeHost(rb->hOffsets);
            rb->dJobs = rb->hJobs = nullptr;
            rb->dOffsets = rb->hOffsets = nullptr;
            rb->jobCap = 0;
            GPUGI_CUDA_TRY(ctx, cudaMalloc(&rb->dJobs, nj * sizeof(RenderConst)));
            GPUGI_CUDA_TRY(ctx, cudaMalloc(&rb->dOffsets, 2 * (nj + 1) * sizeof(uint32_t)));
            GPUGI_CUDA_TRY(ctx, cudaMallocHost(&rb->hJobs, nj * sizeof(RenderConst)));
            GPUGI_CUDA_TRY(ctx, cudaMallocHost(&rb->hOffsets, 2 * (nj + 1) * sizeof(uint32_t)));
            rb->jobCap = nj;
        }
        // launch shapes (no node staging: the walkers serve several scenes)
        WalkerLaunch LE, LS;
        const gpugi_scene* sc0 = jobs[fused[0].job].scene;
        if ((st = walker_launch_config(ctx, sc0, (const void*)k_batch_extend, 1ull << 40, 0, LE)) ||
            (st = walker_launch_config(ctx, sc0, (const void*)k_batch_shadow, 1ull << 40, 0, LS)))
            return st;
        int perSM0 = 0, perSM1 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM0, (const void*)k_batch_shade, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM1, (const void*)k_batch_bpt_shade, 128, 0);
        const unsigned gridShade0 = (unsigned)(ctx->numSMs * std::max(perSM0, 1));
        const unsigned gridShade1 = (unsigned)(ctx->numSMs * std::max(perSM1, 1));
        const unsigned genBlocks = (unsigned)ctx->numSMs * 8;
        const uint32_t groupE = ctx->traceMode >= 3 ? LE.grid * 128u / 2u : 0u;
        const uint32_t groupS = ctx->traceMode >= 3 ? LS.grid * 128u / 2u : 0u;
        auto phase = [&](cudaStream_t stream, int ph, uint32_t maxDepth) {
            cudaMemsetAsync(rb->cnt, 0, offsetof(Counters, rays), stream);
            PathSoA A = rb->A, B = rb->B;
            k_batch_generate<<<genBlocks, 256, 0, stream>>>(rb->dJobs, rb->dOffsets + ph * (nj + 1), nj, rb->cnt, A,
                                                            rb->Q, ph);
            for (int depth = 0; depth < (int)maxDepth; ++depth) {
                k_batch_extend<<<LE.grid, 128, 0, stream>>>(rb->dJobs, rb->cnt, ctx->errWord, A, rb->H, depth,
                                                            groupE);
                if (ph == 0) k_batch_shade<<<gridShade0, 128, 0, stream>>>(rb->dJobs, rb->cnt, A, B, rb->H, rb->Q, depth);
                else k_batch_bpt_shade<<<gridShade1, 128, 0, stream>>>(rb->dJobs, rb->cnt, A, B, rb->H, rb->Q, depth);
                k_batch_shadow<<<LS.grid, 128, 0, stream>>>(rb->dJobs, rb->cnt, ctx->errWord, rb->Q, depth, groupS);
                std::swap(A, B);
            }
        };
        auto record = [&](cudaStream_t stream) {
            phase(stream, 0, depth0);
            if (depth1) phase(stream, 1, depth1);
        };
        if (ctx->batchGraph) {
            const std::vector<uintptr_t> key = {(uintptr_t)rb->block, (uintptr_t)rb->dJobs, nj, depth0, depth1,
                                                LE.grid, LS.grid, gridShade0, gridShade1, (uintptr_t)ctx->errWord,
                                                groupE, groupS};
            if (!rb->batchExec || key != rb->batchKey) {
                if (rb->batchExec) cudaGraphExecDestroy(rb->batchExec);
                rb->batchExec = nullptr;
                cudaGraph_t graph = nullptr;
                GPUGI_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
                record(ctx->stream);
                const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
                if (ce != cudaSuccess) return cuda_fail(ctx, ce, "capturing the batch wavefront");
                const cudaError_t ie = cudaGraphInstantiate(&rb->batchExec, graph, 0);
                cudaGraphDestroy(graph);
                if (ie != cudaSuccess) {
                    rb->batchExec = nullptr;
                    return cuda_fail(ctx, ie, "instantiating the batch graph");
                }
                rb->batchKey = key;
            }
        }
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rb->cnt, 0, sizeof(Counters), ctx->stream));
        std::vector<uint32_t> done(nj, 0);
        uint32_t* off0 = rb->hOffsets;
        uint32_t* off1 = rb->hOffsets + nj + 1;
        for (;;) {
            // plan a round: each unfinished job adds as many samples as still fit
            GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // staging buffers are free again
            uint64_t used0 = 0, paths0 = 0, paths1 = 0, usedCache = 0, lightOff = 0, cacheSlot = 0;
            bool any = false;
            off0[0] = off1[0] = 0;
            for (uint32_t q = 0; q < nj; ++q) {
                const Fused& F = fused[q];
                const gpugi_job& J = jobs[F.job];
                uint64_t c = std::min<uint64_t>(J.params.samples - done[q], (cap - used0) / (F.paths0 + F.extraQ));
                if (F.paths1) c = std::min<uint64_t>(c, (cap - paths1) / F.paths1);
                if (F.cacheBytes) c = std::min<uint64_t>(c, (cacheBudget - usedCache) / F.cacheBytes);
                RenderConst rc = make_render_const(ctx, J.scene, &J.camera, &J.params, J.image, rb);
                rc.samples = (uint32_t)c;
                rc.sampleBase = done[q];
                rc.lightSamples = rb->lights + lightOff / 16;
                rc.numRaysPerLightSample = (int)F.raysPerLight;
                rc.lightThreads = F.lightThreads;
                if (F.cacheBytes) {
                    rc.cache = rb->cache + usedCache / sizeof(CacheEntry);
                    rc.cacheCount = rb->cacheCount + cacheSlot;
                    rc.cacheCap = (uint32_t)(F.cacheBytes / sizeof(CacheEntry));
                }
                if (c) {
                    const size_t setFloats = (size_t)J.params.numLightSamples * 8;
                    float* dst = rb->hostLights + lightOff / 4;
                    if (J.lightSamples)
                        std::memcpy(dst, J.lightSamples + (size_t)done[q] * setFloats, c * setFloats * sizeof(float));
                    else
                        for (uint64_t k = 0; k < c; ++k)
                            generate_light_samples(const_cast<gpugi_scene*>(J.scene), *J.rngState,
                                                   J.params.numLightSamples, dst + k * setFloats);
                    lightOff += c * setFloats * sizeof(float);
                    any = true;
                }
                rb->hJobs[q] = rc;
                used0 += c * (F.paths0 + F.extraQ);
                paths0 += c * F.paths0;
                paths1 += c * F.paths1;
                usedCache += c * F.cacheBytes;
                if (F.cacheBytes) cacheSlot += c;
                off0[q + 1] = (uint32_t)paths0;
                off1[q + 1] = (uint32_t)paths1;
                done[q] += (uint32_t)c;
            }
            if (!any) break;
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rb->lights, rb->hostLights, lightOff, cudaMemcpyHostToDevice,
                                                ctx->stream));
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rb->dJobs, rb->hJobs, nj * sizeof(RenderConst),
                                                cudaMemcpyHostToDevice, ctx->stream));
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rb->dOffsets, rb->hOffsets, 2 * (nj + 1) * sizeof(uint32_t),
                                                cudaMemcpyHostToDevice, ctx->stream));
            if (ctx->batchGraph) GPUGI_CUDA_TRY(ctx, cudaGraphLaunch(rb->batchExec, ctx->stream));
            else record(ctx->stream);
            GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        }
    }
    // the Whitted ray tracer and the photon mapper: one job after another
    for (uint32_t j = 0; j < numJobs; ++j) {
        const gpugi_job& J = jobs[j];
        if (J.params.pass <= GPUGI_PASS_BPT) continue;
        gpugi_status st = gpugi_render(ctx, J.scene, &J.camera, &J.params, J.lightSamples, J.rngState, J.image);
        if (st) return st;
    }
    return GPUGI_OK;
}

}  // extern "C"
