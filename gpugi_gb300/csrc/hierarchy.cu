// Hierarchy-importance renderer (HierarchyImportance, gpugi/renderer/
// hierarchyimportance.cpp) on AABB hierarchies.
//
// The reference measures how densely camera paths cross every node and
// triangle (importance acquisition), derives per node how well the node
// stands in for its subtree (propagation), and renders with a traversal that
// stops at nodes whose subtree is not worth descending (TRACERAY_IMPORTANCE_
// BREAK), shading such a node with an area-averaged material and a normal
// drawn from its SGGX normal distribution. Here:
//
//   k_hier_parents, k_hier_materials   parent links; node materials bottom up
//                                      (sampleleafmaterials.comp, pullmaterials.comp)
//   k_acq_*                            acquisition2.comp + counthits.glsl as a
//                                      wavefront (per path vertex: closest hits, hit
//                                      counting, shading, next-event rays), float atomics
//   k_hier_prop_init, k_hier_prop_up   hierarchypropagation_init.comp / _nodes.comp
//                                      as one bottom-up pass (the second child to
//                                      finish continues to the parent)
//   k_hier_render                      hierarchypathtracer.comp, one thread per pixel
//                                      and sample (at most 4 vertices per path)
//
// The reference runs the node passes to convergence, level by level
// (hierarchyimportance.cpp:112-134,150-159); a node's value only depends on
// its children's final values, so one bottom-up pass gives the same numbers.
// All buffers are in the device node order; gpugi_hierarchy_read maps them
// back to the uploaded order. Arithmetic whose results are compared exactly
// (materials, propagation, the importance-break walk) uses the
// non-contracted helpers of common.cuh.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "shade.cuh"
#include "trace.cuh"

namespace gpugi {

struct HierBuffers {
    void* block = nullptr;
    float2* imp = nullptr;        // {x, y} per node, then per leaf slot
    float* subtree = nullptr;     // per node
    uint32_t* parents = nullptr;  // per node, kNoParent at the root
    uint32_t* arrive = nullptr;   // per node: children finished (bottom-up passes)
    uint2* mats = nullptr;        // 6 per node: packed halves
    uint16_t* ndf = nullptr;      // 6 per node: sigma.xyz, r.xyz (unorm16)
    bool ndfReady = false, importanceReady = false;
    float4* lights = nullptr;     // light-sample sets of a chunk
    size_t lightCap = 0;          // bytes
    float* hostLights = nullptr;  // pinned staging
    size_t hostLightCap = 0;      // bytes
    void* acq = nullptr;          // wavefront state of the importance acquisition
    uint64_t acqCap = 0;          // paths it holds
};

namespace {

constexpr uint32_t kNoParent = 0xFFFFFFFFu;
constexpr float kNotificationBias = 1.19e-07f;  // hierarchypropagation_init.comp:18
constexpr int kAcquirePathLength = 8;           // acquisition2.comp:24

struct HierConst {
    DevScene s;
    float3 camU, camV, camW, camPos;
    int width, height;
    uint32_t numLightSamples;
    const float4* lightSamples;  // [set][numLightSamples][2]
    float3 sky;
    int maxPathLength;
    uint32_t iteration, samples;  // render: sample s of the call has frame seed FrameSeed(iteration + s)
    uint32_t rng;                 // render: 1 PCG streams, 0 the reference's (acquisition always the reference's)
    float4* image;
    double* image64;
    float2* imp;
    const uint2* mats;
    const uint16_t* ndf;
    uint32_t* err;
};

GPUGI_D uint32_t node_child(const DevScene& s, uint32_t i) { return __float_as_uint(__ldg(s.nodes + 2 * i).w); }
GPUGI_D uint32_t node_escape(const DevScene& s, uint32_t i) { return __float_as_uint(__ldg(s.nodes + 2 * i + 1).w); }

// IntersectBox (intersectiontests.glsl:9-20) with the exit distance.
GPUGI_D bool intersect_box_exit(float3 o, float3 inv, float4 lo, float4 hi, float& firstHit, float& lastHit) {
    float tbx = X::mul(inv.x, X::sub(lo.x, o.x)), tby = X::mul(inv.y, X::sub(lo.y, o.y)),
          tbz = X::mul(inv.z, X::sub(lo.z, o.z));
    float ttx = X::mul(inv.x, X::sub(hi.x, o.x)), tty = X::mul(inv.y, X::sub(hi.y, o.y)),
          ttz = X::mul(inv.z, X::sub(hi.z, o.z));
    float mnx = fminf(ttx, tbx), mny = fminf(tty, tby), mnz = fminf(ttz, tbz);
    float mxx = fmaxf(ttx, tbx), mxy = fmaxf(tty, tby), mxz = fmaxf(ttz, tbz);
    firstHit = fmaxf(0.0f, fmaxf(fmaxf(mnx, mny), fmaxf(mnx, mnz)));
    lastHit = fminf(fminf(mxx, mxy), fminf(mxx, mxz));
    return firstHit <= lastHit;
}

GPUGI_D float3 inv_dir(float3 d) { return make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z)); }

// Adds importance to *dst for every converged lane of the warp that adds to
// the same address: one atomic of importance x lanes. The callers' lanes all
// carry the same importance (a power of two), so the product is exact.
GPUGI_D void add_importance(float* dst, float importance) {
    const unsigned peers = __match_any_sync(__activemask(), (unsigned long long)dst);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(peers) - 1)) atomicAdd(dst, importance * (float)__popc(peers));
}

// TraceRayCountHits (hierarchy/counthits.glsl:1-71) as a resumable walk, one
// node (with its leaf block) per step, for the persistent loop below. Every
// ray of a launch carries the same importance (acquisition2.comp halves it
// per vertex for all paths alike), which add_importance relies on.
struct CountWalk {
    float3 o, d, inv;
    float len, importance;
    uint32_t node, budget;
};
GPUGI_D bool count_step(CountWalk& w, const DevScene& s, float2* imp, uint32_t* err) {
    if (w.budget-- == 0) {
        raise_error(err, DEVERR_TRAVERSAL_CAP);
        return true;
    }
    const float4 a = __ldg(s.nodes + 2 * w.node), b = __ldg(s.nodes + 2 * w.node + 1);
    const uint32_t child = __float_as_uint(a.w), escape = __float_as_uint(b.w);
    float fh, lh;
    if (intersect_box_exit(w.o, w.inv, a, b, fh, lh) && fh <= w.len) {
        add_importance(&imp[w.node].x, w.importance);
        if (child & LEAF_FLAG) {
            const uint32_t count = (child >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK;
            const uint32_t slot0 = (child & LEAF_BLOCK_MASK) * s.leafSize;
            for (uint32_t k = 0; k < count; ++k) {
                float h, by, bz;
                if (intersect_triangle(w.o, w.d, s.tris + 3 * (size_t)(slot0 + k), h, by, bz) && h <= w.len)
                    add_importance(&imp[s.numNodes + slot0 + k].x, w.importance);
            }
            w.node = escape;
        } else {
            w.node = child;
        }
    } else {
        w.node = escape;
    }
    return w.node == 0;
}

// Count walks of n items: a lane whose walk ends takes the next item
// (warp-aggregated increments of *work), so lanes do not wait for the longest
// walk of their warp. load(i, o, d, len, importance) returns false for an
// item without a walk.
template <typename Load>
GPUGI_D void persistent_count_walks(const DevScene& s, uint32_t n, unsigned long long* work, float2* imp,
                                    uint32_t* err, Load load) {
    const unsigned lane = threadIdx.x & 31u;
    CountWalk w;
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
                    if (load((uint32_t)my, w.o, w.d, w.len, w.importance)) {
                        w.inv = inv_dir(w.d);
                        w.node = 0;
                        w.budget = s.numNodes;
                        active = true;
                    }
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active && count_step(w, s, imp, err)) active = false;
    }
}

// TraceRay / TraceRayAnyHit with TRACERAY_IMPORTANCE_BREAK and
// HIT_INDEX_OUTPUT (traceray.glsl:25-180) at IMPORTANCE_THRESHOLD 0
// (hierarchypathtracer.comp:4): a node with importance y <= threshold x
// entry distance is not descended. The closest-hit walk takes it as a hit at
// a hashed point between entry and exit and goes on at its escape; the
// any-hit walk reports an occluder when the node ends within rayLength and
// skips the node otherwise.
struct ImportanceHit {
    int32_t node = -1, slot = -1;  // slot -1: the node itself was hit
    float nodeImportance = 0.0f, nodeSizeSq = 0.0f;
    float u = 0.0f, v = 0.0f;
};
template <bool ANY_HIT>
GPUGI_D bool trace_importance(const DevScene& s, const float2* __restrict__ imp, float3 o, float3 d, float& len,
                              float threshold, ImportanceHit* out, uint32_t* err) {
    const float3 inv = inv_dir(d);
    uint32_t node = 0, budget = s.numNodes, lastNode = 0;
    float lastImportance = 0.0f, lastSizeSq = 0.0f;
    while (true) {
        if (budget-- == 0) {
            raise_error(err, DEVERR_TRAVERSAL_CAP);
            return false;
        }
        if (kChecked && node >= s.numNodes) {
            raise_error(err, DEVERR_BOUNDS);
            return false;
        }
        const float4 a = __ldg(s.nodes + 2 * node), b = __ldg(s.nodes + 2 * node + 1);
        const uint32_t child = __float_as_uint(a.w), escape = __float_as_uint(b.w);
        float fh, lh;
        if (intersect_box_exit(o, inv, a, b, fh, lh) && fh <= len) {
            const float2 im = __ldg(imp + node);
            const float3 ext = X::sub3(xyz(b), xyz(a));
            lastNode = node;
            lastImportance = im.x;
            lastSizeSq = X::dot(ext, ext);
            if ((im.x < 0.0f && fh > 0.0f) || im.y <= X::mul(threshold, fh)) {
                if (ANY_HIT) {
                    if (lh <= len) return true;
                } else {
                    out->nodeImportance = im.x;
                    out->nodeSizeSq = lastSizeSq;
                    out->node = (int32_t)node;
                    // fh + ((lh - fh) * h) / 8388593, grouped as traceray.glsl:95 groups it
                    const float h = __uint2float_rn(wanghash(__float_as_uint(lh)) % 8388593u);
                    len = X::add(fh, X::div(X::mul(X::sub(lh, fh), h), 8388593.0f));
                    out->slot = -1;
                }
                node = escape;
            } else if (child & LEAF_FLAG) {
                const uint32_t count = (child >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK;
                const uint32_t slot0 = (child & LEAF_BLOCK_MASK) * s.leafSize;
                if (kChecked && (uint64_t)slot0 + count > s.numSlots) {
                    raise_error(err, DEVERR_BOUNDS);
                    return false;
                }
                for (uint32_t k = 0; k < count; ++k) {
                    float h, by, bz;
                    if (intersect_triangle(o, d, s.tris + 3 * (size_t)(slot0 + k), h, by, bz) && h < len) {
                        if (ANY_HIT) return true;
                        len = h;
                        out->slot = (int32_t)(slot0 + k);
                        out->node = (int32_t)lastNode;
                        out->u = by;
                        out->v = bz;
                        out->nodeImportance = lastImportance;
                        out->nodeSizeSq = lastSizeSq;
                    }
                }
                node = escape;
            } else {
                node = child;
            }
        } else {
            node = escape;
        }
        if (node == 0) break;
    }
    return false;
}

// ------------------------------------------------------------ node materials
struct HMat {  // MaterialData accumulator
    float4 r;
    float3 op, di, em, f0, f1;
    float ri;
};
GPUGI_D void hmat_zero(HMat& m) {
    m.r = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    m.op = m.di = m.em = m.f0 = m.f1 = f3(0.0f);
    m.ri = 0.0f;
}
GPUGI_D float3 madd3(float3 acc, float3 v, float w) { return X::add3(acc, X::scale(w, v)); }
GPUGI_D float3 div3s(float3 v, float a) { return make_float3(X::div(v.x, a), X::div(v.y, a), X::div(v.z, a)); }
GPUGI_D uint32_t pack_half2(float a, float b) {
    return (uint32_t)__half_as_ushort(__float2half_rn(a)) | ((uint32_t)__half_as_ushort(__float2half_rn(b)) << 16);
}
GPUGI_D float2 unpack_half2(uint32_t p) {
    return make_float2(__half2float(__ushort_as_half((unsigned short)(p & 0xFFFFu))),
                       __half2float(__ushort_as_half((unsigned short)(p >> 16))));
}
GPUGI_D void store_hmat(uint2* o, const HMat& m, float area) {
    __stcg(o + 0, make_uint2(pack_half2(m.r.x, m.r.y), pack_half2(m.r.z, m.r.w)));
    __stcg(o + 1, make_uint2(pack_half2(m.op.x, m.op.y), pack_half2(m.op.z, area)));
    __stcg(o + 2, make_uint2(pack_half2(m.di.x, m.di.y), pack_half2(m.di.z, 0.0f)));
    __stcg(o + 3, make_uint2(pack_half2(m.em.x, m.em.y), pack_half2(m.em.z, 0.0f)));
    __stcg(o + 4, make_uint2(pack_half2(m.f0.x, m.f0.y), pack_half2(m.f0.z, m.ri)));
    __stcg(o + 5, make_uint2(pack_half2(m.f1.x, m.f1.y), pack_half2(m.f1.z, 0.0f)));
}
// The node material as hierarchypathtracer.comp:61-68 unpacks it.
GPUGI_D MaterialData load_hmat(const uint2* __restrict__ o) {
    MaterialData m;
    uint2 w = __ldg(o);
    float2 a = unpack_half2(w.x), b = unpack_half2(w.y);
    m.Reflectiveness = make_float4(a.x, a.y, b.x, b.y);
    w = __ldg(o + 1);
    a = unpack_half2(w.x);
    m.Opacity = f3(a.x, a.y, unpack_half2(w.y).x);
    w = __ldg(o + 2);
    a = unpack_half2(w.x);
    m.Diffuse = f3(a.x, a.y, unpack_half2(w.y).x);
    w = __ldg(o + 3);
    a = unpack_half2(w.x);
    m.Emissivity = f3(a.x, a.y, unpack_half2(w.y).x);
    w = __ldg(o + 4);
    a = unpack_half2(w.x);
    b = unpack_half2(w.y);
    m.Fresnel0 = f3(a.x, a.y, b.x);
    m.RefractionIndexAvg = b.y;
    w = __ldg(o + 5);
    a = unpack_half2(w.x);
    m.Fresnel1 = f3(a.x, a.y, unpack_half2(w.y).x);
    return m;
}

__global__ void k_hier_parents(DevScene s, uint32_t* parents, uint32_t* arrive) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.numNodes) return;
    arrive[i] = 0;
    if (i == 0) parents[0] = kNoParent;
    const uint32_t child = node_child(s, i);
    if (child & LEAF_FLAG) return;
    parents[child] = i;                       // first child
    parents[node_escape(s, child)] = i;       // its escape is the second child
}

// sampleleafmaterials.comp:9-97 for a leaf-parent node, then
// pullmaterials.comp:9-93 towards the root.
__global__ void k_hier_materials(DevScene s, const uint32_t* __restrict__ parents, uint32_t* arrive, uint2* mats,
                                 uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.numNodes) return;
    const uint32_t child = node_child(s, i);
    if (!(child & LEAF_FLAG)) return;
    HMat m;
    hmat_zero(m);
    float area = 0.0f;
    const uint32_t count = (child >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK;
    const uint32_t slot0 = (child & LEAF_BLOCK_MASK) * s.leafSize;
    for (uint32_t k = 0; k < count; ++k) {
        const int4 t = __ldg(s.slots + slot0 + k);
        const float* P = s.positions;
        const float3 p0 = f3(P[3 * t.x], P[3 * t.x + 1], P[3 * t.x + 2]);
        const float3 p1 = f3(P[3 * t.y], P[3 * t.y + 1], P[3 * t.y + 2]);
        const float3 p2 = f3(P[3 * t.z], P[3 * t.z + 1], P[3 * t.z + 2]);
        const float3 c = X::cross(X::sub3(p1, p0), X::sub3(p2, p0));
        const float ta = X::div(__fsqrt_rn(X::dot(c, c)), 2.0f);
        area = X::add(area, ta);
        const MaterialData md = load_material(s, t.w);
        m.r = make_float4(X::add(m.r.x, X::mul(md.Reflectiveness.x, ta)), X::add(m.r.y, X::mul(md.Reflectiveness.y, ta)),
                          X::add(m.r.z, X::mul(md.Reflectiveness.z, ta)), X::add(m.r.w, X::mul(md.Reflectiveness.w, ta)));
        m.op = madd3(m.op, md.Opacity, ta);
        m.di = madd3(m.di, md.Diffuse, ta);
        m.em = madd3(m.em, md.Emissivity, ta);
        m.f0 = madd3(m.f0, md.Fresnel0, ta);
        m.f1 = madd3(m.f1, md.Fresnel1, ta);
        m.ri = X::add(m.ri, X::mul(md.RefractionIndexAvg, ta));
    }
    auto finish = [&](uint32_t node, HMat& acc, float ar) {
        acc.r = make_float4(X::div(acc.r.x, ar), X::div(acc.r.y, ar), X::div(acc.r.z, ar), X::div(acc.r.w, ar));
        acc.op = div3s(acc.op, ar);
        acc.di = div3s(acc.di, ar);
        acc.em = div3s(acc.em, ar);
        acc.f0 = div3s(acc.f0, ar);
        acc.f1 = div3s(acc.f1, ar);
        acc.ri = X::div(acc.ri, ar);
        store_hmat(mats + 6 * (size_t)node, acc, ar);
    };
    finish(i, m, area);
    uint32_t node = i;
    for (uint32_t level = 0;; ++level) {
        const uint32_t p = parents[node];
        if (p == kNoParent) return;
        if (level > s.numNodes || p >= s.numNodes) {
            raise_error(err, DEVERR_HIERARCHY);
            return;
        }
        __threadfence();
        if (atomicAdd(arrive + p, 1u) == 0) return;  // the sibling is still on its way
        __threadfence();
        HMat acc;
        hmat_zero(acc);
        float ar = 0.0f;
        const uint32_t c0 = node_child(s, p), kids[2] = {c0, node_escape(s, c0)};
        for (uint32_t c : kids) {
            const uint2* o = mats + 6 * (size_t)c;
            uint2 w1 = __ldcg(o + 1);
            const float childArea = unpack_half2(w1.y).y;
            ar = X::add(ar, childArea);
            uint2 w = __ldcg(o);
            float2 h0 = unpack_half2(w.x), h1 = unpack_half2(w.y);
            acc.r = make_float4(X::add(acc.r.x, X::mul(h0.x, childArea)), X::add(acc.r.y, X::mul(h0.y, childArea)),
                                X::add(acc.r.z, X::mul(h1.x, childArea)), X::add(acc.r.w, X::mul(h1.y, childArea)));
            auto pull3 = [&](float3 v, uint2 q) {
                const float2 xy = unpack_half2(q.x);
                return make_float3(X::add(v.x, X::mul(xy.x, childArea)), X::add(v.y, X::mul(xy.y, childArea)),
                                   X::add(v.z, X::mul(unpack_half2(q.y).x, childArea)));
            };
            acc.op = pull3(acc.op, w1);
            acc.di = pull3(acc.di, __ldcg(o + 2));
            acc.em = pull3(acc.em, __ldcg(o + 3));
            const uint2 w4 = __ldcg(o + 4);
            acc.f0 = pull3(acc.f0, w4);
            acc.ri = X::add(acc.ri, X::mul(unpack_half2(w4.y).y, childArea));
            acc.f1 = pull3(acc.f1, __ldcg(o + 5));
        }
        finish(p, acc, ar);
        node = p;
    }
}

// ------------------------------------------------------------ importance
// acquisition2.comp:26-112 as a wavefront: per path vertex, one launch each
// for the closest hits, the hit counting along the path segments, the
// shading (next-event ray and BSDF sample, the same random draws in the same
// order as the shader), the next-event rays' closest hits and their hit
// counting. Each launch runs one kind of walk in every lane, instead of one
// thread per path alternating between walks and shading.
struct AcqPaths {
    float *ox, *oy, *oz, *dx, *dy, *dz, *imp;
    uint32_t* seed;
};
struct AcqRays {  // next-event rays of one vertex
    float *ox, *oy, *oz, *dx, *dy, *dz, *dist, *imp, *t;
};
struct AcqState {
    AcqPaths A, B;
    int32_t* slot;  // closest hits of the current paths
    float *t, *u, *v;
    AcqRays L;
    uint32_t* cnt;  // paths per vertex [kAcquirePathLength + 1], then next-event rays per vertex
    unsigned long long* work;  // work counters of the walks, 4 per vertex
};

GPUGI_D float3 load3(const float* x, const float* y, const float* z, uint64_t i) {
    return make_float3(x[i], y[i], z[i]);
}
GPUGI_D void store3(float* x, float* y, float* z, uint64_t i, float3 v) {
    x[i] = v.x;
    y[i] = v.y;
    z[i] = v.z;
}

__global__ void k_acq_generate(HierConst c, uint32_t iterations, AcqPaths A, uint32_t* cnt) {
    const uint32_t numPixels = (uint32_t)(c.width * c.height);
    const uint64_t total = (uint64_t)numPixels * iterations;
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[0] = (uint32_t)total;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < total; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t it = 1u + (uint32_t)(q / numPixels), pix = (uint32_t)(q % numPixels);
        const int x = (int)(pix % (uint32_t)c.width), y = (int)(pix / (uint32_t)c.width);
        Rng seed = rng_init(0u, it, pix);  // acquisition: the reference's streams
        const float2 r = random2(seed);
        const float sx = X::sub(X::mul(X::div(X::add(r.x, (float)x), (float)c.width), 2.0f), 1.0f);
        const float sy = X::sub(X::mul(X::div(X::add(r.y, (float)y), (float)c.height), 2.0f), 1.0f);
        store3(A.ox, A.oy, A.oz, q, c.camPos);
        store3(A.dx, A.dy, A.dz, q, X::normalize(X::add3(X::add3(X::scale(sx, c.camU), X::scale(sy, c.camV)), c.camW)));
        A.imp[q] = 1.0f;
        A.seed[q] = seed.s;
    }
}

// Closest hits with the 8-lane group walk of the ray queries (same results
// as trace_ray): work items are taken through *work.
__global__ void __launch_bounds__(128) k_acq_trace(HierConst c, AcqPaths A, const uint32_t* __restrict__ count,
                                                   AcqState S, unsigned long long* work) {
    group_walks<false, 0, 8>(
        c.s, *count, work, c.err,
        [&](uint64_t i, float3& o, float3& d, float& tmax) {
            o = load3(A.ox, A.oy, A.oz, i);
            d = load3(A.dx, A.dy, A.dz, i);
            tmax = kRAY_MAX;
        },
        [&](uint64_t i, const GroupWalk& g) {
            S.slot[i] = g.slot;
            S.t[i] = g.len;
            S.u[i] = g.u;
            S.v[i] = g.v;
        });
}

__global__ void __launch_bounds__(128) k_acq_count(HierConst c, AcqPaths A, const uint32_t* __restrict__ count,
                                                   const float* __restrict__ t, unsigned long long* work) {
    persistent_count_walks(c.s, *count, work, c.imp, c.err,
                           [&](uint32_t k, float3& o, float3& d, float& len, float& importance) {
                               o = load3(A.ox, A.oy, A.oz, k);
                               d = load3(A.dx, A.dy, A.dz, k);
                               len = X::mul(t[k], 1.000001f);
                               importance = A.imp[k];
                               return true;
                           });
}

// One vertex of the shader's path loop after its two walks: the vertex, the
// halved importance, the next-event ray (when the light sample faces it) and
// the BSDF-sampled continuation (when another vertex follows).
__global__ void __launch_bounds__(128) k_acq_shade(HierConst c, AcqPaths A, AcqPaths B, AcqState S, int vertex) {
    const uint32_t n = S.cnt[vertex];
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t k = base + lane;
        bool light = false, next = false;
        float3 o, d, ld;
        float imp = 0.0f, dist = 0.0f;
        Rng seed{0, 0};
        if (k < n && S.slot[k] >= 0) {
            const int4 tri = __ldg(c.s.slots + S.slot[k]);
            const float3 N = hit_normal(c.s, tri, S.u[k], S.v[k], nullptr);
            const MaterialData m = load_material(c.s, tri.w);
            d = load3(A.dx, A.dy, A.dz, k);
            o = X::add3(load3(A.ox, A.oy, A.oz, k), X::scale(S.t[k], d));
            imp = X::mul(A.imp[k], 0.5f);
            seed.s = A.seed[k];
            const uint32_t li = random_uint(seed) % c.numLightSamples;
            const float4 pn0 = __ldg(c.lightSamples + 2 * li), in1 = __ldg(c.lightSamples + 2 * li + 1);
            ld = X::sub3(xyz(pn0), o);
            dist = __fsqrt_rn(X::dot(ld, ld));
            ld = make_float3(X::div(ld.x, dist), X::div(ld.y, dist), X::div(ld.z, dist));
            light = saturate(dot(unpack_normal(pn0.w, in1.w), -ld)) > 0.0f;
            float3 thr = f3(1.0f);
            float pdf;
            d = sample_bsdf(d, m, seed, N, thr, false, pdf);
            next = vertex + 1 < kAcquirePathLength;
        }
        uint32_t ql, qn;
        warp_append(S.cnt + kAcquirePathLength + 1 + vertex, light, ql);
        if (light) {
            store3(S.L.ox, S.L.oy, S.L.oz, ql, o);
            store3(S.L.dx, S.L.dy, S.L.dz, ql, ld);
            S.L.dist[ql] = dist;
            S.L.imp[ql] = imp;
        }
        warp_append(S.cnt + vertex + 1, next, qn);
        if (next) {
            store3(B.ox, B.oy, B.oz, qn, X::add3(o, X::scale(kRAY_HIT_EPSILON, d)));
            store3(B.dx, B.dy, B.dz, qn, d);
            B.imp[qn] = imp;
            B.seed[qn] = seed.s;
        }
    }
}

// The next-event rays: closest hit within the light distance (no offset
// from the surface, as in the shader), then the counting up to an occluder.
__global__ void __launch_bounds__(128) k_acq_light_trace(HierConst c, AcqRays L, const uint32_t* __restrict__ count,
                                                         unsigned long long* work) {
    group_walks<false, 0, 8>(
        c.s, *count, work, c.err,
        [&](uint64_t i, float3& o, float3& d, float& tmax) {
            o = load3(L.ox, L.oy, L.oz, i);
            d = load3(L.dx, L.dy, L.dz, i);
            tmax = L.dist[i];
        },
        [&](uint64_t i, const GroupWalk& g) { L.t[i] = g.len; });
}

__global__ void __launch_bounds__(128) k_acq_light_count(HierConst c, AcqRays L, const uint32_t* __restrict__ count,
                                                         unsigned long long* work) {
    persistent_count_walks(c.s, *count, work, c.imp, c.err,
                           [&](uint32_t k, float3& o, float3& d, float& len, float& importance) {
                               if (!(L.t[k] < L.dist[k])) return false;  // unoccluded: nothing to count
                               o = load3(L.ox, L.oy, L.oz, k);
                               d = load3(L.dx, L.dy, L.dz, k);
                               len = X::mul(L.t[k], 1.000001f);
                               importance = L.imp[k];
                               return true;
                           });
}

__global__ void k_hier_prop_init(float2* imp, float* subtree, uint32_t* arrive, uint32_t numNodes, float iterations) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numNodes) return;
    imp[i] = make_float2(X::div(imp[i].x, iterations), 0.0f);
    subtree[i] = 0.0f;
    arrive[i] = 0;
}

GPUGI_D float node_avg_area(const DevScene& s, uint32_t i) {
    const float4 a = __ldg(s.nodes + 2 * i), b = __ldg(s.nodes + 2 * i + 1);
    const float sx = X::sub(b.x, a.x), sy = X::sub(b.y, a.y), sz = X::sub(b.z, a.z);
    return X::div(X::mul(X::add(X::add(X::mul(sx, sy), X::mul(sx, sz)), X::mul(sy, sz)), 2.0f), 6.0f);
}

// hierarchypropagation_init.comp:25-69 for a leaf-parent node, then
// hierarchypropagation_nodes.comp:25-81 towards the root.
__global__ void k_hier_prop_up(DevScene s, float2* imp, float* subtree, const uint32_t* __restrict__ parents,
                               uint32_t* arrive, float iterations, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.numNodes) return;
    const uint32_t child = node_child(s, i);
    if (!(child & LEAF_FLAG)) return;
    float ci = 0.0f;
    const uint32_t slot0 = (child & LEAF_BLOCK_MASK) * s.leafSize;
    for (uint32_t k = 0; k < s.leafSize; ++k) ci = X::add(ci, imp[s.numNodes + slot0 + k].x);
    ci = X::div(ci, iterations);
    __stcg(subtree + i, fmaxf(ci, kNotificationBias));
    float approx = X::div(imp[i].x, ci);
    __stcg(&imp[i].y, X::mul(X::mul(approx, approx), node_avg_area(s, i)));
    uint32_t node = i;
    for (uint32_t level = 0;; ++level) {
        const uint32_t p = parents[node];
        if (p == kNoParent) return;
        if (level > s.numNodes || p >= s.numNodes) {
            raise_error(err, DEVERR_HIERARCHY);
            return;
        }
        __threadfence();
        if (atomicAdd(arrive + p, 1u) == 0) return;
        __threadfence();
        const uint32_t c0 = node_child(s, p), c1 = node_escape(s, c0);
        const float sum = X::add(X::add(0.0f, __ldcg(subtree + c0)), __ldcg(subtree + c1));
        __stcg(subtree + p, sum);
        approx = X::div(__ldcg(&imp[p].x), sum);
        __stcg(&imp[p].y, X::mul(X::mul(approx, approx), node_avg_area(s, p)));
        node = p;
    }
}

// ------------------------------------------------------------ the path tracer
// loadSGGX + sampleNormal (hierarchy/sggx.glsl): a visible normal of the
// node's NDF seen from `incident`.
GPUGI_D float3 mat_col(const float3 S[3], float3 v) {  // S * v, columns S[0..2]
    return X::add3(X::add3(X::scale(v.x, S[0]), X::scale(v.y, S[1])), X::scale(v.z, S[2]));
}
GPUGI_D float3 sample_sggx_normal(const uint16_t* __restrict__ n, float3 incident, Rng& seed) {
    const float sgx = __ldg(n) / 65535.0f, sgy = __ldg(n + 1) / 65535.0f, sgz = __ldg(n + 2) / 65535.0f;
    const float rx = __ldg(n + 3) / 65535.0f * 2.0f - 1.0f, ry = __ldg(n + 4) / 65535.0f * 2.0f - 1.0f,
                rz = __ldg(n + 5) / 65535.0f * 2.0f - 1.0f;
    float3 S[3];
    S[0].x = saturate(sgx * sgx);
    S[1].y = saturate(sgy * sgy);
    S[2].z = saturate(sgz * sgz);
    S[0].y = S[1].x = fminf(fmaxf(rx * sgx * sgy, -1.0f), 1.0f);
    S[0].z = S[2].x = fminf(fmaxf(ry * sgx * sgz, -1.0f), 1.0f);
    S[1].z = S[2].y = fminf(fmaxf(rz * sgy * sgz, -1.0f), 1.0f);
    float3 L[3];
    L[2] = -incident;
    create_onb(incident, L[0], L[1]);
    const float Sxx = dot(L[0], mat_col(S, L[0])), Sxy = dot(L[0], mat_col(S, L[1])),
                Sxz = dot(L[0], mat_col(S, L[2])), Syy = dot(L[1], mat_col(S, L[1])),
                Syz = dot(L[1], mat_col(S, L[2])), Szz = dot(L[2], mat_col(S, L[2]));
    const float det = fmaxf(0.0f, Sxx * Syy * Szz + Sxy * Syz * Sxz * 2.0f - Sxz * Sxz * Syy - Sxy * Sxy * Szz -
                                      Syz * Syz * Sxx - kDIVISOR_EPSILON);
    float tmp = Syy * Szz - Syz * Syz + kDIVISOR_EPSILON;
    const float3 mi = tmp != 0.0f ? f3(sqrtf(det / tmp), 0.0f, 0.0f) : f3(0.0f);
    tmp = sqrtf(tmp);
    const float3 mj = (tmp != 0.0f && Szz != 0.0f) ? f3((Sxy * Szz - Sxz * Syz) / tmp, tmp, 0.0f) / sqrtf(Szz) : f3(0.0f);
    const float3 mk = Szz != 0.0f ? f3(Sxz, Syz, Szz) / sqrtf(Szz) : f3(0.0f);
    float chi0 = random01(seed);
    const float w = sqrtf(1.0f - chi0);
    chi0 = sqrtf(chi0);
    const float chi1 = random01(seed) * 6.283185307f;
    float sn, cs;
    sincosf(chi1, &sn, &cs);
    const float3 nrm = (chi0 * cs) * mi + (chi0 * sn) * mj + w * mk;
    return normalize(L[0] * nrm.x + L[1] * nrm.y + L[2] * nrm.z);
}

// EstimateDirectLight with TRACERAY_IMPORTANCE_BREAK (lightsource.glsl:3-93);
// directional samples (normalThetaCos 3, the sun addition) are offset like
// point lights.
GPUGI_D float3 direct_light_importance(const HierConst& c, uint32_t set, float3 pos, float3 N, uint32_t idx,
                                       float3 viewDir, const MaterialData& m, bool sampleAreaLights, float threshold,
                                       float distEpsilon) {
    const float4* ls = c.lightSamples + 2 * ((size_t)set * c.numLightSamples + idx);
    const float4 pn0 = __ldg(ls), in1 = __ldg(ls + 1);
    float pdf;
    if (in1.w > 2.5f) {
        const float3 dir = xyz(pn0);
        const float surfaceCos = saturate(dot(dir, N));
        if (surfaceCos <= 0.0f) return f3(0.0f);
        float len = kRAY_MAX;
        if (trace_importance<true>(c.s, c.imp, distEpsilon * dir + pos, dir, len, threshold, nullptr, c.err))
            return f3(0.0f);
        return (surfaceCos * xyz(in1)) * eval_bsdf(viewDir, dir, m, N, pdf, false);
    }
    float3 dir = xyz(pn0) - pos;
    const float distSq = dot(dir, dir) + kDIVISOR_EPSILON;
    const float dist = sqrtf(distSq);
    dir = dir / dist;
    const float surfaceCos = saturate(dot(dir, N));
    if (surfaceCos <= 0.0f) return f3(0.0f);
    if (in1.w > 1.5f) {
        float len = dist - kRAY_HIT_EPSILON - distEpsilon;
        if (trace_importance<true>(c.s, c.imp, distEpsilon * dir + pos, dir, len, threshold, nullptr, c.err))
            return f3(0.0f);
        return ((surfaceCos / distSq) * xyz(in1)) * eval_bsdf(viewDir, dir, m, N, pdf, false);
    }
    if (!sampleAreaLights) return f3(0.0f);
    const float f = saturate(dot(unpack_normal(pn0.w, in1.w), -dir));
    if (!(f > 0.0f)) return f3(0.0f);
    float len = dist - kRAY_HIT_EPSILON * 2;
    if (trace_importance<true>(c.s, c.imp, kRAY_HIT_EPSILON * dir + pos, dir, len, threshold, nullptr, c.err))
        return f3(0.0f);
    return ((surfaceCos / distSq) * (xyz(in1) * f)) * eval_bsdf(viewDir, dir, m, N, pdf, false);
}

// hierarchypathtracer.comp:20-149, one path of pixel pix for sample s.
__global__ void k_hier_render(HierConst c) {
    const uint32_t numPixels = (uint32_t)(c.width * c.height);
    const uint64_t total = (uint64_t)numPixels * c.samples;
    const float lightSampleWeight = (float)c.numLightSamples;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < total; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = (uint32_t)(q / numPixels), pix = (uint32_t)(q % numPixels);
        const int x = (int)(pix % (uint32_t)c.width), y = (int)(pix / (uint32_t)c.width);
        Rng seed = rng_init(c.rng, c.iteration + s, pix);
        const float2 r = random2(seed);
        const float sx = X::sub(X::mul(X::div(X::add(r.x, (float)x), (float)c.width), 2.0f), 1.0f);
        const float sy = X::sub(X::mul(X::div(X::add(r.y, (float)y), (float)c.height), 2.0f), 1.0f);
        float3 o = c.camPos;
        float3 d = X::normalize(X::add3(X::add3(X::scale(sx, c.camU), X::scale(sy, c.camV)), c.camW));
        float3 color = f3(0.0f), tp = f3(1.0f);
        float threshold = 0.000430915f;  // tan(yFOV/2) / height / 4 in the shader
        bool didNEE = false;
        for (int i = 0; i < c.maxPathLength; ++i) {
            ImportanceHit h;
            float len = kRAY_MAX;
            trace_importance<false>(c.s, c.imp, o, d, len, threshold, &h, c.err);
            if (len == kRAY_MAX) {
                color = color + tp * c.sky;
                break;
            }
            o = X::add3(o, X::scale(len, d));
            float3 N;
            MaterialData m;
            if (h.slot < 0) {
                m = load_hmat(c.mats + 6 * (size_t)h.node);
                N = sample_sggx_normal(c.ndf + 6 * (size_t)h.node, d, seed);
            } else {
                const int4 tri = __ldg(c.s.slots + h.slot);
                N = hit_normal(c.s, tri, h.u, h.v, nullptr);
                m = load_material(c.s, tri.w);
            }
            const float nextThreshold = threshold * 20.0f;
            const float eps = h.slot < 0 ? sqrtf(h.nodeSizeSq) * 0.1f : kRAY_HIT_EPSILON;
            if (!didNEE) color = color + tp * m.Emissivity;
            didNEE = m.Reflectiveness.w < 500.0f;
            const uint32_t li = random_uint(seed) % c.numLightSamples;
            const float3 rad = direct_light_importance(c, s, o, N, li, d, m, didNEE, threshold, eps);
            color = color + rad * tp * lightSampleWeight;
            float3 thr = f3(1.0f);
            float pdf;
            bool reflectedDiffuse;
            d = sample_bsdf(d, m, seed, N, thr, true, pdf, false, &reflectedDiffuse);
            o = o + d * eps;
            tp = tp * thr;
            threshold = nextThreshold;
            const float p = saturate(luminance(thr));
            if (random01(seed) >= p) break;
            tp = tp / p;
        }
        atomicAdd(c.image + pix, make_float4(color.x, color.y, color.z, 1.0f));
        if (c.image64) {
            atomicAdd(c.image64 + 3 * (size_t)pix, (double)color.x);
            atomicAdd(c.image64 + 3 * (size_t)pix + 1, (double)color.y);
            atomicAdd(c.image64 + 3 * (size_t)pix + 2, (double)color.z);
        }
    }
}

// ------------------------------------------------------------ host side
gpugi_status ensure_hier(gpugi_ctx* ctx, gpugi_scene* sc) {
    if (sc->hier) return GPUGI_OK;
    const uint32_t nn = sc->dev.numNodes, ns = sc->dev.numSlots;
    auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t bytes = a(8 * ((size_t)nn + ns)) + a(4 * (size_t)nn) * 3 + a(48 * (size_t)nn) + a(12 * (size_t)nn);
    HierBuffers* h = new HierBuffers();
    if (cudaMalloc(&h->block, bytes) != cudaSuccess) {
        delete h;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "hierarchy buffers");
    }
    char* p = static_cast<char*>(h->block);
    auto take = [&](size_t b) {
        char* r = p;
        p += a(b);
        return r;
    };
    h->imp = reinterpret_cast<float2*>(take(8 * ((size_t)nn + ns)));
    h->subtree = reinterpret_cast<float*>(take(4 * (size_t)nn));
    h->parents = reinterpret_cast<uint32_t*>(take(4 * (size_t)nn));
    h->arrive = reinterpret_cast<uint32_t*>(take(4 * (size_t)nn));
    h->mats = reinterpret_cast<uint2*>(take(48 * (size_t)nn));
    h->ndf = reinterpret_cast<uint16_t*>(take(12 * (size_t)nn));
    sc->hier = h;
    // zeros until the NDFs and the importance pass fill them (gpugi_hierarchy_read may come first)
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(h->block, 0, bytes, ctx->stream));
    return GPUGI_OK;
}

gpugi_status check_scene(gpugi_ctx* ctx, const gpugi_scene* sc) {
    if (!sc || sc->ctx != ctx) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene of another context");
    if (sc->dev.boundsKind != GPUGI_BOUNDS_AABB)
        return fail(ctx, GPUGI_ERROR_UNSUPPORTED, "the hierarchy-importance renderer needs AABB nodes");
    if (!sc->dev.vinfo || !sc->dev.materials)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene lacks vertex info or materials");
    return GPUGI_OK;
}

HierConst make_const(gpugi_ctx* ctx, gpugi_scene* sc, const gpugi_camera* cam, uint32_t width, uint32_t height) {
    HierConst c{};
    c.s = sc->dev;
    c.s.matTex = nullptr;  // the hierarchy pass shades with the materials' constant values
    c.camU = f3(cam->U[0], cam->U[1], cam->U[2]);
    c.camV = f3(cam->V[0], cam->V[1], cam->V[2]);
    c.camW = f3(cam->W[0], cam->W[1], cam->W[2]);
    c.camPos = f3(cam->position[0], cam->position[1], cam->position[2]);
    c.width = (int)width;
    c.height = (int)height;
    c.imp = sc->hier->imp;
    c.mats = sc->hier->mats;
    c.ndf = sc->hier->ndf;
    c.err = ctx->errWord;
    return c;
}

gpugi_status ensure_lights(gpugi_ctx* ctx, HierBuffers* h, size_t bytes) {
    if (bytes > h->lightCap) {
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (h->lights) cudaFree(h->lights);
        h->lights = nullptr;
        h->lightCap = 0;
        GPUGI_CUDA_TRY(ctx, cudaMalloc(&h->lights, bytes));
        h->lightCap = bytes;
    }
    if (bytes > h->hostLightCap) {
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (h->hostLights) cudaFreeHost(h->hostLights);
        h->hostLights = nullptr;
        h->hostLightCap = 0;
        GPUGI_CUDA_TRY(ctx, cudaMallocHost(&h->hostLights, bytes));
        h->hostLightCap = bytes;
    }
    return GPUGI_OK;
}

// counters: 2 x (kAcquirePathLength + 1) uint32 in the first 128 bytes, then
// 4 x kAcquirePathLength uint64 work counters (per vertex: path hits, path
// counting, next-event hits, next-event counting)
constexpr size_t kAcqCounterBytes = 128 + 8 * 4 * kAcquirePathLength;
static_assert(4 * 2 * (kAcquirePathLength + 1) <= 128, "counter layout");

// Wavefront buffers of the acquisition for `paths` paths (grown on demand).
gpugi_status ensure_acq(gpugi_ctx* ctx, HierBuffers* h, uint64_t paths, AcqState& S) {
    auto a = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t col = a(4 * paths);
    if (paths > h->acqCap) {
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (h->acq) cudaFree(h->acq);
        h->acq = nullptr;
        h->acqCap = 0;
        if (cudaMalloc(&h->acq, (2 * 8 + 4 + 9) * col + a(kAcqCounterBytes)) != cudaSuccess) {
            h->acq = nullptr;
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "acquisition wavefront buffers");
        }
        h->acqCap = paths;
    }
    const size_t ccol = a(4 * h->acqCap);
    char* p = static_cast<char*>(h->acq);
    auto f = [&]() {
        float* r = reinterpret_cast<float*>(p);
        p += ccol;
        return r;
    };
    for (AcqPaths* P : {&S.A, &S.B}) {
        P->ox = f(), P->oy = f(), P->oz = f(), P->dx = f(), P->dy = f(), P->dz = f(), P->imp = f();
        P->seed = reinterpret_cast<uint32_t*>(f());
    }
    S.slot = reinterpret_cast<int32_t*>(f());
    S.t = f(), S.u = f(), S.v = f();
    S.L.ox = f(), S.L.oy = f(), S.L.oz = f(), S.L.dx = f(), S.L.dy = f(), S.L.dz = f(), S.L.dist = f(),
    S.L.imp = f(), S.L.t = f();
    S.cnt = reinterpret_cast<uint32_t*>(p);
    S.work = reinterpret_cast<unsigned long long*>(p + 128);
    return GPUGI_OK;
}

// The importance pass with light samples already on the device.
gpugi_status importance_pass(gpugi_ctx* ctx, gpugi_scene* sc, const gpugi_camera* cam, uint32_t width,
                             uint32_t height, const float4* lights, uint32_t numLightSamples, uint32_t iterations) {
    HierBuffers* h = sc->hier;
    const uint32_t nn = sc->dev.numNodes;
    HierConst c = make_const(ctx, sc, cam, width, height);
    c.lightSamples = lights;
    c.numLightSamples = numLightSamples;
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(h->imp, 0, 8 * ((size_t)nn + sc->dev.numSlots), ctx->stream));
    const uint64_t work = (uint64_t)width * height * iterations;
    if (work > 0xFFFFFFFFull) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "more than 2^32 acquisition paths");
    AcqState S;
    gpugi_status st = ensure_acq(ctx, h, work, S);
    if (st) return st;
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(S.cnt, 0, kAcqCounterBytes, ctx->stream));
    const unsigned grid = (unsigned)ctx->numSMs * 8;
    WalkerLaunch LT, LC;
    if ((st = walker_launch_config(ctx, sc, (const void*)k_acq_trace, 1ull << 40, 0, LT)) ||
        (st = walker_launch_config(ctx, sc, (const void*)k_acq_count, 1ull << 40, 0, LC)))
        return st;
    k_acq_generate<<<grid, 256, 0, ctx->stream>>>(c, iterations, S.A, S.cnt);
    for (int vtx = 0; vtx < kAcquirePathLength; ++vtx) {
        const uint32_t* np = S.cnt + vtx;
        const uint32_t* nl = S.cnt + kAcquirePathLength + 1 + vtx;
        unsigned long long* w = S.work + 4 * vtx;
        k_acq_trace<<<LT.grid, 128, 0, ctx->stream>>>(c, S.A, np, S, w);
        k_acq_count<<<LC.grid, 128, 0, ctx->stream>>>(c, S.A, np, S.t, w + 1);
        k_acq_shade<<<grid, 128, 0, ctx->stream>>>(c, S.A, S.B, S, vtx);
        k_acq_light_trace<<<LT.grid, 128, 0, ctx->stream>>>(c, S.L, nl, w + 2);
        k_acq_light_count<<<LC.grid, 128, 0, ctx->stream>>>(c, S.L, nl, w + 3);
        std::swap(S.A, S.B);
    }
    const unsigned nb = (nn + 127) / 128;
    k_hier_prop_init<<<nb, 128, 0, ctx->stream>>>(h->imp, h->subtree, h->arrive, nn, (float)iterations);
    k_hier_prop_up<<<nb, 128, 0, ctx->stream>>>(sc->dev, h->imp, h->subtree, h->parents, h->arrive,
                                                (float)iterations, ctx->errWord);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    h->importanceReady = true;
    return GPUGI_OK;
}

}  // namespace

void free_hierarchy(gpugi_scene* sc) {
    HierBuffers* h = sc->hier;
    if (!h) return;
    if (h->block) cudaFree(h->block);
    if (h->lights) cudaFree(h->lights);
    if (h->hostLights) cudaFreeHost(h->hostLights);
    if (h->acq) cudaFree(h->acq);
    delete h;
    sc->hier = nullptr;
}

gpugi_status render_hierarchy(gpugi_ctx* ctx, gpugi_scene* sc, const gpugi_camera* cam,
                              const gpugi_render_params* p, const float* lightSamples, uint64_t* rngState,
                              gpugi_image* im) {
    gpugi_status st = check_scene(ctx, sc);
    if (st) return st;
    if (!sc->hier || !sc->hier->ndfReady)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "no node NDFs: call gpugi_scene_set_hierarchy_ndf first");
    HierBuffers* h = sc->hier;
    const uint64_t numPixels = (uint64_t)p->width * p->height;
    const uint32_t chunk = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(p->samples, (16ull << 20) / numPixels));
    const size_t setFloats = (size_t)p->numLightSamples * 8;
    if ((st = ensure_lights(ctx, h, chunk * setFloats * sizeof(float)))) return st;
    HierConst c = make_const(ctx, sc, cam, p->width, p->height);
    c.numLightSamples = p->numLightSamples;
    c.lightSamples = h->lights;
    c.sky = f3(p->sky[0], p->sky[1], p->sky[2]);
    c.maxPathLength = (int)p->maxPathLength;
    c.image = im->rgba;
    c.image64 = im->rgb64;
    for (uint32_t s0 = 0; s0 < p->samples; s0 += chunk) {
        const uint32_t ns = std::min(chunk, p->samples - s0);
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // the staging buffer may still feed a copy
        if (lightSamples) {
            std::memcpy(h->hostLights, lightSamples + (size_t)s0 * setFloats, ns * setFloats * sizeof(float));
        } else {
            for (uint32_t k = 0; k < ns; ++k)
                generate_light_samples(sc, *rngState, p->numLightSamples, h->hostLights + k * setFloats);
        }
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(h->lights, h->hostLights, ns * setFloats * sizeof(float),
                                            cudaMemcpyHostToDevice, ctx->stream));
        // HierarchyImportance::Draw: importance from scratch at iteration 0
        // (10 acquisition passes, hierarchyimportance.cpp:94-105)
        if (s0 == 0 && (p->iteration == 0 || !h->importanceReady) &&
            (st = importance_pass(ctx, sc, cam, p->width, p->height, h->lights, p->numLightSamples, 10)))
            return st;
        c.iteration = p->iteration + s0;
        c.samples = ns;
        c.rng = (p->flags & GPUGI_RENDER_REFERENCE_RNG) ? 0u : 1u;
        const uint64_t work = numPixels * ns;
        const unsigned grid = (unsigned)std::min<uint64_t>((work + 127) / 128, (uint64_t)ctx->numSMs * 16);
        k_hier_render<<<grid, 128, 0, ctx->stream>>>(c);
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    }
    return GPUGI_OK;
}

}  // namespace gpugi

using namespace gpugi;

extern "C" {

gpugi_status gpugi_scene_set_hierarchy_ndf(gpugi_ctx* ctx, gpugi_scene* sc, const uint16_t* sggx) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sggx) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL sggx");
    gpugi_status st = check_scene(ctx, sc);
    if (st || (st = ensure_hier(ctx, sc))) return st;
    HierBuffers* h = sc->hier;
    const uint32_t nn = sc->dev.numNodes;
    std::vector<uint16_t> dev((size_t)nn * 6);
    for (uint32_t i = 0; i < nn; ++i) {
        const uint32_t d = sc->nodeMap.empty() ? i : sc->nodeMap[i];
        std::memcpy(&dev[6 * (size_t)d], sggx + 6 * (size_t)i, 12);
    }
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(h->ndf, dev.data(), dev.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
    const unsigned nb = (nn + 127) / 128;
    k_hier_parents<<<nb, 128, 0, ctx->stream>>>(sc->dev, h->parents, h->arrive);
    DevScene untextured = sc->dev;  // node materials average the materials' constant values
    untextured.matTex = nullptr;
    k_hier_materials<<<nb, 128, 0, ctx->stream>>>(untextured, h->parents, h->arrive, h->mats, ctx->errWord);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // `dev` goes out of scope
    h->ndfReady = true;
    return GPUGI_OK;
}

gpugi_status gpugi_hierarchy_importance(gpugi_ctx* ctx, gpugi_scene* sc, const gpugi_camera* cam, uint32_t width,
                                        uint32_t height, const float* lightSamples, uint32_t numLightSamples,
                                        uint32_t iterations) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!cam || !lightSamples) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (width == 0 || height == 0 || numLightSamples == 0 || iterations == 0 || iterations > 1024)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "width, height, numLightSamples > 0, iterations in [1, 1024]");
    gpugi_status st = check_scene(ctx, sc);
    if (st || (st = ensure_hier(ctx, sc))) return st;
    if (!sc->hier->ndfReady) {  // parents come with the NDFs; without them set up the links only
        const unsigned nb = (sc->dev.numNodes + 127) / 128;
        k_hier_parents<<<nb, 128, 0, ctx->stream>>>(sc->dev, sc->hier->parents, sc->hier->arrive);
    }
    const size_t bytes = (size_t)numLightSamples * 32;
    if ((st = ensure_lights(ctx, sc->hier, bytes))) return st;
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::memcpy(sc->hier->hostLights, lightSamples, bytes);
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(sc->hier->lights, sc->hier->hostLights, bytes, cudaMemcpyHostToDevice,
                                        ctx->stream));
    return importance_pass(ctx, sc, cam, width, height, sc->hier->lights, numLightSamples, iterations);
}

gpugi_status gpugi_hierarchy_read(gpugi_ctx* ctx, const gpugi_scene* sc, float* importance, float* subtree,
                                  uint32_t* materials) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || sc->ctx != ctx) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene of another context");
    if (!sc->hier) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "no hierarchy data on this scene");
    const HierBuffers* h = sc->hier;
    const uint32_t nn = sc->dev.numNodes, ns = sc->dev.numSlots;
    auto map = [&](uint32_t i) { return sc->nodeMap.empty() ? i : sc->nodeMap[i]; };
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (importance) {
        std::vector<float> d(2 * ((size_t)nn + ns));
        GPUGI_CUDA_TRY(ctx, cudaMemcpy(d.data(), h->imp, d.size() * 4, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < nn; ++i) {
            importance[2 * (size_t)i] = d[2 * (size_t)map(i)];
            importance[2 * (size_t)i + 1] = d[2 * (size_t)map(i) + 1];
        }
        std::memcpy(importance + 2 * (size_t)nn, d.data() + 2 * (size_t)nn, 8 * (size_t)ns);
    }
    if (subtree) {
        std::vector<float> d(nn);
        GPUGI_CUDA_TRY(ctx, cudaMemcpy(d.data(), h->subtree, 4 * (size_t)nn, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < nn; ++i) subtree[i] = d[map(i)];
    }
    if (materials) {
        std::vector<uint32_t> d(12 * (size_t)nn);
        GPUGI_CUDA_TRY(ctx, cudaMemcpy(d.data(), h->mats, 48 * (size_t)nn, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < nn; ++i) std::memcpy(materials + 12 * (size_t)i, &d[12 * (size_t)map(i)], 48);
    }
    return GPUGI_OK;
}

}  // extern "C"
