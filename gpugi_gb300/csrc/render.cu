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
#include <algorithm>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "shade.cuh"
#include "trace.cuh"

struct gpugi_image {
    gpugi_ctx* ctx = nullptr;
    uint32_t width = 0, height = 0, flags = 0;
    float4* rgba = nullptr;
    double* rgb64 = nullptr;
};

namespace gpugi {

constexpr int kMaxDepth = 64;

struct PathSoA {
    float *ox, *oy, *oz, *dx, *dy, *dz, *tx, *ty, *tz, *lastP;
    uint32_t *seed, *pixel, *info;  // info: bit 0 = didNEE, bits 8..31 = sample (iteration) index
};
struct HitSoA {
    int32_t* slot;
    float *t, *u, *v;
};
struct ShadowSoA {
    float *ox, *oy, *oz, *dx, *dy, *dz, *tmax, *cr, *cg, *cb;
    uint32_t* pixel;
};

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
};

// ------------------------------------------------------------ accumulation
GPUGI_D void splat(const RenderConst& rc, uint32_t pixel, float3 c, float w = 0.0f) {
    if (!(c.x != 0.0f || c.y != 0.0f || c.z != 0.0f || w != 0.0f)) return;
    atomicAdd(rc.image + pixel, make_float4(c.x, c.y, c.z, w));
    if (rc.image64) {
        atomicAdd(rc.image64 + 3 * (size_t)pixel, (double)c.x);
        atomicAdd(rc.image64 + 3 * (size_t)pixel + 1, (double)c.y);
        atomicAdd(rc.image64 + 3 * (size_t)pixel + 2, (double)c.z);
    }
}

GPUGI_D void store_path(const PathSoA& P, uint32_t i, float3 o, float3 d, float3 tp, uint32_t seed, uint32_t pixel,
                        uint32_t info, float lastP) {
    P.ox[i] = o.x; P.oy[i] = o.y; P.oz[i] = o.z;
    P.dx[i] = d.x; P.dy[i] = d.y; P.dz[i] = d.z;
    P.tx[i] = tp.x; P.ty[i] = tp.y; P.tz[i] = tp.z;
    P.seed[i] = seed; P.pixel[i] = pixel; P.info[i] = info; P.lastP[i] = lastP;
}
GPUGI_D void store_shadow(const ShadowSoA& Q, uint32_t i, float3 o, float3 d, float tmax, float3 c, uint32_t pixel) {
    Q.ox[i] = o.x; Q.oy[i] = o.y; Q.oz[i] = o.z;
    Q.dx[i] = d.x; Q.dy[i] = d.y; Q.dz[i] = d.z;
    Q.tmax[i] = tmax; Q.cr[i] = c.x; Q.cg[i] = c.y; Q.cb[i] = c.z; Q.pixel[i] = pixel;
}

// Persistent refill loop shared by the extend and shadow kernels.
template <bool ANY_HIT, int BOUNDS, typename Load, typename Finish>
GPUGI_D void persistent_walks(const DevScene& s, uint32_t n, unsigned long long* work, uint32_t* err, Load load,
                              Finish finish) {
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
        if (active && walk_step<ANY_HIT, BOUNDS>(w, s, err)) {
            finish(ray, w);
            active = false;
        }
    }
}

template <int BOUNDS>
__global__ void __launch_bounds__(128) k_extend(RenderConst rc, PathSoA A, HitSoA H, int depth) {
    const uint32_t n = rc.cnt->path[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&rc.cnt->rays[0], (unsigned long long)n);
    persistent_walks<false, BOUNDS>(
        rc.s, n, &rc.cnt->extendWork[depth], rc.err,
        [&](uint32_t i, float3& o, float3& d, float& tmax) {
            o = make_float3(A.ox[i], A.oy[i], A.oz[i]);
            d = make_float3(A.dx[i], A.dy[i], A.dz[i]);
            tmax = kRAY_MAX;
        },
        [&](uint32_t i, const WalkState& w) {
            H.slot[i] = w.slot;
            H.t[i] = w.len;
            H.u[i] = w.u;
            H.v[i] = w.v;
        });
}

template <int BOUNDS>
__global__ void __launch_bounds__(128) k_shadow(RenderConst rc, ShadowSoA Q, int depth) {
    const uint32_t n = rc.cnt->shadow[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&rc.cnt->rays[1], (unsigned long long)n);
    persistent_walks<true, BOUNDS>(
        rc.s, n, &rc.cnt->shadowWork[depth], rc.err,
        [&](uint32_t i, float3& o, float3& d, float& tmax) {
            o = make_float3(Q.ox[i], Q.oy[i], Q.oz[i]);
            d = make_float3(Q.dx[i], Q.dy[i], Q.dz[i]);
            tmax = Q.tmax[i];
        },
        [&](uint32_t i, const WalkState& w) {
            if (w.slot < 0) splat(rc, Q.pixel[i], make_float3(Q.cr[i], Q.cg[i], Q.cb[i]));
        });
}

// ------------------------------------------------------------ generation
// Primary ray (pathtracer.comp:132-139) in exact IEEE operations, so camera
// rays, and with them the first hits, are bit-identical to the oracle's.
GPUGI_D float3 primary_direction(const RenderConst& rc, uint32_t& seed, int x, int y) {
    float2 r = random2(seed);
    const float sx = X::sub(X::mul(X::div(X::add(X::sub(r.x, 0.5f), (float)x), (float)rc.width), 2.0f), 1.0f);
    const float sy = X::sub(X::mul(X::div(X::add(X::sub(r.y, 0.5f), (float)y), (float)rc.height), 2.0f), 1.0f);
    return X::normalize(X::add3(X::add3(X::scale(sx, rc.camU), X::scale(sy, rc.camV)), rc.camW));
}

// pathtracer.comp:16-46 / pathtracer_bidir.comp:16-24: one camera path per
// pixel and iteration. BPT also counts the iteration in the alpha channel.
__global__ void k_camera_generate(RenderConst rc, PathSoA A, bool bidir) {
    const uint32_t total = rc.samples * (uint32_t)rc.numPixels;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        const uint32_t s = p / (uint32_t)rc.numPixels, pix = p % (uint32_t)rc.numPixels;
        const int x = (int)(pix % (uint32_t)rc.width), y = (int)(pix / (uint32_t)rc.width);
        uint32_t seed = wanghash(wanghash(rc.iteration + rc.sampleBase + s) + pix);
        const float3 d = primary_direction(rc, seed, x, y);
        store_path(A, p, rc.camPos, d, f3(1.0f), seed, pix, s << 8, 1.0f);
        if (bidir) splat(rc, pix, f3(0.0f), 1.0f);
    }
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
__global__ void k_light_generate(RenderConst rc, PathSoA A, bool withCache) {
    const uint32_t total = rc.samples * rc.lightThreads;
    if (blockIdx.x == 0 && threadIdx.x == 0) rc.cnt->path[0] = total;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t s = g / rc.lightThreads, gid = g % rc.lightThreads;
        uint32_t seed = wanghash(wanghash(rc.iteration + rc.sampleBase + s) + gid);
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
        store_path(A, g, xyz(pn0), d, tp, seed, gid, s << 8, 1.0f);
    }
}

// ------------------------------------------------------------ shading
struct Hit {
    bool valid;
    float3 pos, N;
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
    h.N = hit_normal(rc.s, h.tri, H.u[k], H.v[k], nullptr);
    h.m = load_material(rc.s, h.tri.w);
    return h;
}

// EstimateDirectLight (lightsource.glsl:3-93), split: returns the radiance
// assuming visibility and the shadow ray that decides it.
GPUGI_D bool direct_light(const RenderConst& rc, uint32_t s, float3 pos, float3 N, uint32_t idx, float3 viewDir,
                          const MaterialData& m, bool sampleAreaLights, float3& radiance, float3& ro, float3& rd,
                          float& rlen) {
    const float4* ls = rc.lightSamples + 2 * ((size_t)s * rc.numLightSamples + idx);
    const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
    float pdf;
    if (in1.w > 2.5f) {  // directional light (addition)
        rd = xyz(pn0);
        float cosS = saturate(dot(rd, N));
        if (cosS <= 0.0f) return false;
        radiance = (cosS * xyz(in1)) * eval_bsdf(viewDir, rd, m, N, pdf, false);
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
        radiance = ((cosS / distSq) * xyz(in1)) * eval_bsdf(viewDir, L, m, N, pdf, false);
    } else if (sampleAreaLights) {
        const float f = saturate(dot(unpack_normal(pn0.w, in1.w), -L));
        if (!(f > 0.0f)) return false;
        radiance = ((cosS / distSq) * (xyz(in1) * f)) * eval_bsdf(viewDir, L, m, N, pdf, false);
    } else {
        return false;
    }
    ro = kRAY_HIT_EPSILON * L + pos;
    rd = L;
    rlen = dist - kRAY_HIT_EPSILON * 2;
    return true;
}

// Russian roulette (pathtracer.comp:99-104); rrStartDepth > 0 delays it.
GPUGI_D bool roulette(const RenderConst& rc, int depth, float3 throughput, float3& tp, uint32_t& seed) {
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

// pathtracer.comp:48-105, one bounce.
__global__ void __launch_bounds__(128) k_pt_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                  int depth) {
    const uint32_t n = rc.cnt->path[depth];
    const float lightSampleWeight = (float)rc.numLightSamples;
    WARP_LOOP(n, k, valid) {
        bool survive = false, shadow = false;
        float3 o, d, tp, sro, srd, contrib;
        float srl = 0.0f;
        uint32_t seed = 0, pixel = 0, info = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = A.seed[k];
            pixel = A.pixel[k];
            info = A.info[k];
            Hit h = load_hit(rc, H, k, o, d);
            if (!h.valid) {
                splat(rc, pixel, tp * rc.sky);
            } else {
                o = h.pos;
                if (!(info & 1u)) splat(rc, pixel, tp * h.m.Emissivity);
                const bool didNEE = h.m.Reflectiveness.w < 500.0f;
                info = (info & ~1u) | (didNEE ? 1u : 0u);
                const uint32_t li = random_uint(seed) % rc.numLightSamples;
                float3 rad;
                if (direct_light(rc, info >> 8, o, h.N, li, d, h.m, didNEE, rad, sro, srd, srl)) {
                    contrib = rad * tp * lightSampleWeight;
                    shadow = contrib.x != 0.0f || contrib.y != 0.0f || contrib.z != 0.0f;
                }
                float3 thr = f3(1.0f);
                float pdf;
                d = sample_bsdf(d, h.m, seed, h.N, thr, false, pdf);
                o = o + d * kRAY_HIT_EPSILON;
                tp *= thr;
                survive = roulette(rc, depth, thr, tp, seed) && depth + 1 < rc.maxPathLength;
            }
        }
        uint32_t qs, qb;
        warp_append(&rc.cnt->shadow[depth], shadow, qs);
        if (shadow) store_shadow(Q, qs, sro, srd, srl, contrib, pixel);
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, pixel, info, 1.0f);
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

// lighttracer.comp:95-192, one bounce (with SAVE_LIGHT_CACHE when withCache).
__global__ void __launch_bounds__(128) k_light_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                     int depth, bool withCache) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        bool survive = false, shadow = false;
        float3 o, d, tp, sro, srd, color;
        float srl = 0.0f;
        uint32_t seed = 0, pixel = 0, info = 0, gid = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = A.seed[k];
            gid = A.pixel[k];
            info = A.info[k];
            const int32_t slot = H.slot[k];
            if (slot >= 0) {
                const float t = H.t[k];
                const float4 rec = __ldg(rc.s.tris + 3 * (size_t)slot + 2);
                const float3 gN = make_float3(rec.y, rec.z, rec.w);  // cross(e1, e0), not normalised
                o = o + t * d;
                const int4 tri = __ldg(rc.s.slots + slot);
                float2 tc;
                const float3 sN = hit_normal(rc.s, tri, H.u[k], H.v[k], &tc);
                const MaterialData m = load_material(rc.s, tri.w);
                const uint32_t s = info >> 8;
                if (withCache && m.Reflectiveness.w < 100.0f) {
                    const uint32_t e = atomicAdd(rc.cacheCount + s, 1u);
                    if (e < rc.cacheCap) {
                        float2 pn = pack_normal(sN);
                        write_cache(rc, s, e, tp, tri.w, o, pn.x, pn.y, tc, pack_normal(d), depth + 1);
                    } else {
                        raise_error(rc.err, DEVERR_QUEUE_OVERFLOW);
                    }
                }
                shadow = project_to_screen(rc, o, d, gN, sN, m, tp, withCache, sro, srd, srl, color, pixel);
                float3 thr = f3(1.0f);
                float pdf;
                const float3 nd = sample_bsdf(d, m, seed, sN, thr, true, pdf);
                thr *= shading_correction(d, nd, gN, sN);
                tp *= thr;
                survive = roulette(rc, depth, thr, tp, seed) && depth + 1 < rc.maxPathLength;
                d = nd;
                o = o + d * kRAY_HIT_EPSILON;
            }
        }
        uint32_t qs, qb;
        warp_append(&rc.cnt->shadow[depth], shadow, qs);
        if (shadow) store_shadow(Q, qs, sro, srd, srl, color, pixel);
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, gid, info, 1.0f);
    }
}

// showlightcaches.comp:9-65: light samples seen directly by the camera.
template <int BOUNDS>
__global__ void k_show_light_samples(RenderConst rc) {
    const uint32_t total = rc.samples * rc.numLightSamples;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const float4* ls = rc.lightSamples + 2 * (size_t)i;
        const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
        if (in1.w > 2.5f) continue;  // directional samples have no position
        float3 cd = rc.camPos - xyz(pn0);
        const float camViewDotRay = -dot(rc.camW, cd);
        if (!(camViewDotRay > 0.0f)) continue;
        float sx = -dot(rc.camU, cd) / camViewDotRay, sy = -dot(rc.camV, cd) / camViewDotRay;
        sx /= dot(rc.camU, rc.camU);
        sy /= dot(rc.camV, rc.camV);
        if (!(sx >= -1.0f && sx < 1.0f && sy > -1.0f && sy <= 1.0f)) continue;
        const float distSq = dot(cd, cd);
        const float dist = sqrtf(distSq);
        cd /= dist;
        TraceResult r = trace_ray<true, BOUNDS>(rc.s, cd * kRAY_HIT_EPSILON + xyz(pn0), cd, dist, rc.err);
        if (r.slot >= 0) continue;
        const float3 n = unpack_normal(pn0.w, in1.w);
        const float cosTheta = dot(n, cd);
        const float cosAtCamera = saturate(camViewDotRay / dist);
        const float i2r = cosTheta / (kPI_2 * cosAtCamera * cosAtCamera * cosAtCamera * rc.pixelArea * distSq);
        const int px = (int)((sx * 0.5f + 0.5f) * (float)rc.width), py = (int)((sy * 0.5f + 0.5f) * (float)rc.height);
        if (px < 0 || py < 0 || px >= rc.width || py >= rc.height) continue;
        splat(rc, (uint32_t)(py * rc.width + px), xyz(in1) * i2r);
    }
}

// pathtracer_bidir.comp:54-245, one bounce of the eye pass.
__global__ void __launch_bounds__(128) k_bpt_shade(RenderConst rc, PathSoA A, PathSoA B, HitSoA H, ShadowSoA Q,
                                                   int depth) {
    const uint32_t n = rc.cnt->path[depth];
    WARP_LOOP(n, k, valid) {
        bool survive = false, shadow = false;
        float3 o, d, tp, sro, srd, contrib;
        float srl = 0.0f, lastP = 1.0f;
        uint32_t seed = 0, pixel = 0, info = 0;
        if (valid) {
            o = make_float3(A.ox[k], A.oy[k], A.oz[k]);
            d = make_float3(A.dx[k], A.dy[k], A.dz[k]);
            tp = make_float3(A.tx[k], A.ty[k], A.tz[k]);
            seed = A.seed[k];
            pixel = A.pixel[k];
            info = A.info[k];
            lastP = A.lastP[k];
            Hit h = load_hit(rc, H, k, o, d);
            if (!h.valid) {
                splat(rc, pixel, tp * rc.sky);
            } else {
                const uint32_t s = info >> 8;
                o = h.pos;
                const float rayHit = h.t;
                const float incCos = saturate(-dot(h.N, d));
                const float cLE = distance_mis(rayHit) * mis_heuristic(incCos / kPI);
                float mis = depth == 0 ? 1.0f : lastP / fmaxf(lastP + cLE, kDIVISOR_EPSILON);
                splat(rc, pixel, mis * tp * h.m.Emissivity);
                const uint32_t actual = min(rc.cacheCount[s], rc.cacheCap);
                if (actual > 0) {
                    const uint32_t li = random_uint(seed) % actual;
                    const CacheEntry* ep = rc.cache + (size_t)s * rc.cacheCap + li;
                    const float4 e0 = ep->fluxMat, e1 = ep->posN0, e2 = ep->tcN1Len, e3 = ep->incident;
                    const int pathLength = __float_as_int(e2.w) + depth + 1;
                    if (pathLength <= rc.maxPathLength) {
                        float3 L = xyz(e1) - o;
                        const float lightDistSq = dot(L, L);
                        const float lightDist = sqrtf(lightDistSq);
                        L /= fmaxf(lightDist, kDIVISOR_EPSILON);
                        float3 lN = f3(0.0f, 1.0f, 0.0f);
                        float cosLight = 0.0f;
                        const float cosCamera = fabsf(dot(L, h.N));
                        const bool lambertian = e2.z < 1.5f;
                        if (lambertian) {
                            lN = unpack_normal_raw(e1.w, e2.z);
                            cosLight = fabsf(dot(L, lN));
                        }
                        float pdf;
                        const float3 bsdf = eval_bsdf(d, L, h.m, h.N, pdf, false);
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
                                const MaterialData lm = load_material(rc.s, lmat);
                                const float3 inc = unpack_normal(e3.x, e3.y);
                                const float3 lb = adjoint_bsdf(L, -inc, lm, lN, pdf);
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
                        contrib = irr * tp * bsdf;
                        shadow = contrib.x != 0.0f || contrib.y != 0.0f || contrib.z != 0.0f;
                        sro = kRAY_HIT_EPSILON * L + o;
                        srd = L;
                        srl = lightDist - kRAY_HIT_EPSILON * 2;
                    }
                }
                float3 thr = f3(1.0f);
                float samplePDF;
                d = sample_bsdf(d, h.m, seed, h.N, thr, false, samplePDF);
                o = o + d * kRAY_HIT_EPSILON;
                tp *= thr;
                survive = roulette(rc, depth, thr, tp, seed) && depth + 1 < rc.maxPathLength;
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
                lastP = rcp;
            }
        }
        uint32_t qs, qb;
        warp_append(&rc.cnt->shadow[depth], shadow, qs);
        if (shadow) store_shadow(Q, qs, sro, srd, srl, contrib, pixel);
        warp_append(&rc.cnt->path[depth + 1], survive, qb);
        if (survive) store_path(B, qb, o, d, tp, seed, pixel, info, lastP);
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
};

static void free_render(gpugi_ctx* ctx) {
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if (!rb) return;
    if (rb->block) cudaFree(rb->block);
    if (rb->hostLights) cudaFreeHost(rb->hostLights);
    delete rb;
    ctx->render = nullptr;
}

static gpugi_status ensure_buffers(gpugi_ctx* ctx, size_t paths, size_t cacheBytes, size_t lightBytes,
                                   uint32_t samples) {
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if (!rb) {
        rb = new RenderBuffers();
        ctx->render = rb;
        ctx->renderFree = free_render;
    }
    if (paths <= rb->pathCap && cacheBytes <= rb->cacheBytes && lightBytes <= rb->lightBytes &&
        samples <= rb->maxSamples)
        return GPUGI_OK;
    cudaStreamSynchronize(ctx->stream);
    if (rb->block) cudaFree(rb->block);
    rb->block = nullptr;
    paths = std::max(paths, rb->pathCap);
    cacheBytes = std::max(cacheBytes, rb->cacheBytes);
    lightBytes = std::max(lightBytes, rb->lightBytes);
    samples = std::max(samples, rb->maxSamples);
    auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t col = a(paths * 4);
    const size_t total = 2 * 13 * col + 4 * col + 11 * col + a(sizeof(Counters)) + a(cacheBytes) +
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
    }
    rb->H.slot = reinterpret_cast<int32_t*>(take(col));
    rb->H.t = reinterpret_cast<float*>(take(col));
    rb->H.u = reinterpret_cast<float*>(take(col));
    rb->H.v = reinterpret_cast<float*>(take(col));
    float** qf[] = {&rb->Q.ox, &rb->Q.oy, &rb->Q.oz, &rb->Q.dx, &rb->Q.dy, &rb->Q.dz, &rb->Q.tmax, &rb->Q.cr,
                    &rb->Q.cg, &rb->Q.cb};
    for (float** q : qf) *q = reinterpret_cast<float*>(take(col));
    rb->Q.pixel = reinterpret_cast<uint32_t*>(take(col));
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

static int persistent_grid(gpugi_ctx* ctx, const void* kernel) {
    int perSM = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, 128, 0);
    return ctx->numSMs * (perSM > 0 ? perSM : 1);
}

// One chunk of `samples` iterations of a pass.
static gpugi_status render_chunk(gpugi_ctx* ctx, const gpugi_scene* sc, RenderConst rc, uint32_t pass) {
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    const bool ell = sc->dev.boundsKind == GPUGI_BOUNDS_ELLIPSOID;
    auto extend = ell ? (const void*)k_extend<1> : (const void*)k_extend<0>;
    auto shadowK = ell ? (const void*)k_shadow<1> : (const void*)k_shadow<0>;
    const int gridE = persistent_grid(ctx, extend), gridS = persistent_grid(ctx, shadowK);
    int gridShade = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gridShade, (const void*)k_pt_shade, 128, 0);
    gridShade = ctx->numSMs * std::max(gridShade, 1);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rc.cnt, 0, offsetof(Counters, rays), ctx->stream));
    PathSoA A = rb->A, B = rb->B;

    auto bounces = [&](int kind /*0 PT, 1 light, 2 light+cache, 3 BPT eye*/) -> gpugi_status {
        for (int depth = 0; depth < rc.maxPathLength; ++depth) {
            if (ell) k_extend<1><<<gridE, 128, 0, ctx->stream>>>(rc, A, rb->H, depth);
            else k_extend<0><<<gridE, 128, 0, ctx->stream>>>(rc, A, rb->H, depth);
            if (kind == 0) k_pt_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth);
            else if (kind == 3) k_bpt_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth);
            else k_light_shade<<<gridShade, 128, 0, ctx->stream>>>(rc, A, B, rb->H, rb->Q, depth, kind == 2);
            if (ell) k_shadow<1><<<gridS, 128, 0, ctx->stream>>>(rc, rb->Q, depth);
            else k_shadow<0><<<gridS, 128, 0, ctx->stream>>>(rc, rb->Q, depth);
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
    } else if (pass == GPUGI_PASS_LT) {
        k_light_generate<<<genBlocks, 256, 0, ctx->stream>>>(rc, A, false);
        if ((st = bounces(1))) return st;
        if (ell) k_show_light_samples<1><<<ctx->numSMs, 128, 0, ctx->stream>>>(rc);
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

}  // namespace gpugi

using namespace gpugi;

extern "C" {

gpugi_status gpugi_image_create(gpugi_ctx* ctx, uint32_t width, uint32_t height, uint32_t flags, gpugi_image** out) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!out || width == 0 || height == 0 || (uint64_t)width * height > (1ull << 31))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad image size");
    gpugi_image* im = new gpugi_image();
    im->ctx = ctx;
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
    if (p->pass > GPUGI_PASS_BPT) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown pass");
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

    const uint32_t numPixels = p->width * p->height;
    // LightPathtracer::SetScreenSize (gpugi/renderer/lightpathtracer.cpp:34)
    const uint32_t raysPerLight =
        std::max<uint32_t>(64u, (numPixels / p->numLightSamples / 64u) * 64u);
    const uint32_t lightThreads = raysPerLight * p->numLightSamples;
    const uint32_t perSamplePaths = p->pass == GPUGI_PASS_PT ? numPixels : std::max(numPixels, lightThreads);
    // Light-cache capacity: the worst case (every particle stores its light
    // sample plus one entry per bounce) so it can never overflow.
    const uint64_t cachePerSample = p->pass == GPUGI_PASS_BPT ? (uint64_t)lightThreads * (p->maxPathLength + 1) : 0;
    // Samples per chunk: at most 16M paths and 4 GiB of light cache in flight.
    uint64_t chunk = std::max<uint64_t>(1, (16ull << 20) / perSamplePaths);
    if (cachePerSample) chunk = std::min<uint64_t>(chunk, std::max<uint64_t>(1, (4ull << 30) / (cachePerSample * 64)));
    chunk = std::min<uint64_t>(chunk, p->samples);
    const size_t lightBytes = chunk * p->numLightSamples * 32;
    gpugi_status st = ensure_buffers(ctx, chunk * perSamplePaths, chunk * cachePerSample * 64, lightBytes,
                                     (uint32_t)chunk);
    if (st) return st;
    RenderBuffers* rb = static_cast<RenderBuffers*>(ctx->render);
    if (rb->hostLightBytes < lightBytes) {
        if (rb->hostLights) cudaFreeHost(rb->hostLights);
        rb->hostLights = nullptr;
        rb->hostLightBytes = 0;
        GPUGI_CUDA_TRY(ctx, cudaMallocHost(&rb->hostLights, lightBytes));
        rb->hostLightBytes = lightBytes;
    }

    RenderConst rc;
    rc.s = sc->dev;
    rc.camU = f3(cam->U[0], cam->U[1], cam->U[2]);
    rc.camV = f3(cam->V[0], cam->V[1], cam->V[2]);
    rc.camW = f3(cam->W[0], cam->W[1], cam->W[2]);
    rc.camPos = f3(cam->position[0], cam->position[1], cam->position[2]);
    rc.pixelArea = cam->pixelArea;
    rc.width = (int)p->width;
    rc.height = (int)p->height;
    rc.numPixels = (int)numPixels;
    rc.maxPathLength = (int)p->maxPathLength;
    rc.rrStartDepth = (int)p->rrStartDepth;
    rc.iteration = p->iteration;
    rc.numLightSamples = p->numLightSamples;
    rc.sky = f3(p->sky[0], p->sky[1], p->sky[2]);
    rc.numRaysPerLightSample = (int)raysPerLight;
    rc.lightThreads = lightThreads;
    rc.image = im->rgba;
    rc.image64 = im->rgb64;
    rc.cache = rb->cache;
    rc.cacheCount = rb->cacheCount;
    rc.cacheCap = (uint32_t)cachePerSample;
    rc.cnt = rb->cnt;
    rc.err = ctx->errWord;
    rc.lightSamples = rb->lights;
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(rb->cnt, 0, sizeof(Counters), ctx->stream));
    for (uint32_t s0 = 0; s0 < p->samples; s0 += (uint32_t)chunk) {
        const uint32_t ns = std::min<uint32_t>((uint32_t)chunk, p->samples - s0);
        // the pinned staging buffer may still feed the previous chunk's copy
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        const size_t setFloats = (size_t)p->numLightSamples * 8;
        if (lightSamples) {
            std::memcpy(rb->hostLights, lightSamples + (size_t)s0 * setFloats, ns * setFloats * sizeof(float));
        } else {
            for (uint32_t s = 0; s < ns; ++s)
                generate_light_samples(const_cast<gpugi_scene*>(sc), *rngState, p->numLightSamples,
                                       rb->hostLights + s * setFloats);
        }
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(rb->lights, rb->hostLights, ns * setFloats * sizeof(float),
                                            cudaMemcpyHostToDevice, ctx->stream));
        rc.samples = ns;
        rc.sampleBase = s0;
        if ((st = render_chunk(ctx, sc, rc, p->pass))) return st;
    }
    return GPUGI_OK;
}

}  // extern "C"
