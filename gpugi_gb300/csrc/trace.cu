// Ray-query kernels behind gpugi_trace_closest / gpugi_trace_any.
//
// One ray per thread; rays and results are structure-of-arrays so every
// load and store of a warp is a single coalesced 128-B transaction. The
// walk itself reads 32-B nodes and 48-B triangle records through the
// read-only (non-coherent) path with 16-B vector loads.
#include "ctx.cuh"
#include "trace.cuh"

namespace gpugi {

template <int BOUNDS>
__global__ void __launch_bounds__(256) k_trace_closest(DevScene s, const float* __restrict__ ox,
                                                       const float* __restrict__ oy, const float* __restrict__ oz,
                                                       const float* __restrict__ dx, const float* __restrict__ dy,
                                                       const float* __restrict__ dz, const float* __restrict__ tmax,
                                                       uint64_t n, int32_t* __restrict__ slot, float* __restrict__ t,
                                                       float* __restrict__ u, float* __restrict__ v, uint32_t* err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 o = make_float3(__ldg(ox + i), __ldg(oy + i), __ldg(oz + i));
    const float3 d = make_float3(__ldg(dx + i), __ldg(dy + i), __ldg(dz + i));
    TraceResult r = trace_ray<false, BOUNDS>(s, o, d, __ldg(tmax + i), err);
    slot[i] = r.slot;
    t[i] = r.t;
    u[i] = r.u;
    v[i] = r.v;
}

template <int BOUNDS>
__global__ void __launch_bounds__(256) k_trace_any(DevScene s, const float* __restrict__ ox,
                                                   const float* __restrict__ oy, const float* __restrict__ oz,
                                                   const float* __restrict__ dx, const float* __restrict__ dy,
                                                   const float* __restrict__ dz, const float* __restrict__ tmax,
                                                   uint64_t n, uint8_t* __restrict__ occluded, uint32_t* err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 o = make_float3(__ldg(ox + i), __ldg(oy + i), __ldg(oz + i));
    const float3 d = make_float3(__ldg(dx + i), __ldg(dy + i), __ldg(dz + i));
    TraceResult r = trace_ray<true, BOUNDS>(s, o, d, __ldg(tmax + i), err);
    occluded[i] = r.slot >= 0 ? 1 : 0;
}

gpugi_status walker_launch_config(gpugi_ctx* ctx, const gpugi_scene* sc, const void* kernel, uint64_t n,
                                  uint32_t maxStage, WalkerLaunch& out) {
    out.stage = sc->dev.topNodes < maxStage ? sc->dev.topNodes : maxStage;
    out.smem = (size_t)out.stage * 32;
    if (out.smem > 48 * 1024)
        GPUGI_CUDA_TRY(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)out.smem));
    int perSM = 0;
    GPUGI_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, 128, out.smem));
    uint64_t grid = (uint64_t)ctx->numSMs * (uint64_t)(perSM > 0 ? perSM : 1);
    const uint64_t needed = (n + 127) / 128;
    if (grid > needed) grid = needed;
    out.grid = (unsigned)(grid > 0 ? grid : 1);
    return GPUGI_OK;
}

// Persistent walk: a grid sized to fill the GPU once; every warp keeps all 32
// lanes busy by handing each finished lane the next ray index from a global
// counter (one atomic per warp per refill). Each ray still performs exactly
// trace_ray's sequence of tests, so results are identical.
template <bool ANY_HIT, int BOUNDS>
__global__ void __launch_bounds__(128) k_trace_persistent(
    DevScene s, const float* __restrict__ ox, const float* __restrict__ oy, const float* __restrict__ oz,
    const float* __restrict__ dx, const float* __restrict__ dy, const float* __restrict__ dz,
    const float* __restrict__ tmax, uint64_t n, int32_t* __restrict__ slot, float* __restrict__ t,
    float* __restrict__ u, float* __restrict__ v, uint8_t* __restrict__ occluded, unsigned long long* counter,
    uint32_t* err, uint32_t stage) {
    extern __shared__ float4 s_top[];
    stage_top_nodes(s, s_top, stage);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanesBelow = (1u << lane) - 1u;
    WalkState w;
    uint64_t ray = 0;
    bool active = false, exhausted = false;
    while (true) {
        const bool need = !active && !exhausted;
        const unsigned needMask = __ballot_sync(0xffffffffu, need);
        if (needMask) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(counter, (unsigned long long)__popc(needMask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need) {
                const uint64_t my = base + (uint64_t)__popc(needMask & lanesBelow);
                if (my < n) {
                    ray = my;
                    walk_begin(w, s, make_float3(__ldg(ox + my), __ldg(oy + my), __ldg(oz + my)),
                               make_float3(__ldg(dx + my), __ldg(dy + my), __ldg(dz + my)), __ldg(tmax + my));
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active && walk_step<ANY_HIT, BOUNDS>(w, s, err, s_top, stage)) {
            if (ANY_HIT) {
                occluded[ray] = w.slot >= 0 ? 1 : 0;
            } else {
                slot[ray] = w.slot;
                t[ray] = w.len;
                u[ray] = w.u;
                v[ray] = w.v;
            }
            active = false;
        }
    }
}

gpugi_status launch_trace_persistent(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                     const float* oy, const float* oz, const float* dx, const float* dy,
                                     const float* dz, const float* tmax, uint64_t n, int32_t* slot, float* t,
                                     float* u, float* v, uint8_t* occluded) {
    if (n == 0) return GPUGI_OK;
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(ctx->scratch);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream));
    const bool ell = sc->dev.boundsKind == GPUGI_BOUNDS_ELLIPSOID;
    void (*k)(DevScene, const float*, const float*, const float*, const float*, const float*, const float*,
              const float*, uint64_t, int32_t*, float*, float*, float*, uint8_t*, unsigned long long*, uint32_t*,
              uint32_t);
    if (!ell) k = anyHit ? k_trace_persistent<true, 0> : k_trace_persistent<false, 0>;
    else k = anyHit ? k_trace_persistent<true, 1> : k_trace_persistent<false, 1>;
    WalkerLaunch L;
    gpugi_status st = walker_launch_config(ctx, sc, (const void*)k, n, ctx->sharedNodes, L);
    if (st) return st;
    k<<<L.grid, 128, L.smem, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, occluded,
                                            counter, ctx->errWord, L.stage);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

// Root prefilter (mode 2), first of two launches: one thread per ray with
// fully coalesced loads and stores tests the root bounds (the first test of
// every walk). Rays that miss it are finished here; the others are appended
// to a queue with warp-ballot compaction for the persistent walker.
template <bool ANY_HIT, int BOUNDS>
__global__ void __launch_bounds__(256) k_trace_root_filter(
    DevScene s, const float* __restrict__ ox, const float* __restrict__ oy, const float* __restrict__ oz,
    const float* __restrict__ dx, const float* __restrict__ dy, const float* __restrict__ dz,
    const float* __restrict__ tmax, uint64_t n, int32_t* __restrict__ slot, float* __restrict__ t,
    float* __restrict__ u, float* __restrict__ v, uint8_t* __restrict__ occluded, uint32_t* __restrict__ queue,
    unsigned long long* counters) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool pass = false;
    if (i < n) {
        const float3 o = make_float3(__ldg(ox + i), __ldg(oy + i), __ldg(oz + i));
        const float3 d = make_float3(__ldg(dx + i), __ldg(dy + i), __ldg(dz + i));
        const float len = __ldg(tmax + i);
        const float4 a = __ldg(s.nodes), b = __ldg(s.nodes + 1);
        float firstHit;
        bool hit;
        if (BOUNDS == 0) hit = intersect_box(o, make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z)), a, b, firstHit);
        else hit = intersect_ellipsoid(o, d, a, b, firstHit);
        pass = hit && firstHit <= len;
        if (!pass) {
            if (ANY_HIT) {
                occluded[i] = 0;
            } else {
                slot[i] = -1;
                t[i] = len;
                u[i] = 0.0f;
                v[i] = 0.0f;
            }
        }
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned ballot = __ballot_sync(0xffffffffu, pass);
    unsigned long long base = 0;
    if (lane == 0 && ballot) base = atomicAdd(counters + 1, (unsigned long long)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (pass) queue[base + __popc(ballot & ((1u << lane) - 1u))] = (uint32_t)i;
}

// Second launch: the persistent walker over the queued ray indices.
template <bool ANY_HIT, int BOUNDS>
__global__ void __launch_bounds__(128) k_trace_queue(
    DevScene s, const float* __restrict__ ox, const float* __restrict__ oy, const float* __restrict__ oz,
    const float* __restrict__ dx, const float* __restrict__ dy, const float* __restrict__ dz,
    const float* __restrict__ tmax, int32_t* __restrict__ slot, float* __restrict__ t, float* __restrict__ u,
    float* __restrict__ v, uint8_t* __restrict__ occluded, const uint32_t* __restrict__ queue,
    unsigned long long* counters, uint32_t* err, uint32_t stage) {
    extern __shared__ float4 s_top[];
    stage_top_nodes(s, s_top, stage);
    const uint64_t n = counters[1];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanesBelow = (1u << lane) - 1u;
    WalkState w;
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    while (true) {
        const bool need = !active && !exhausted;
        const unsigned needMask = __ballot_sync(0xffffffffu, need);
        if (needMask) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(counters + 2, (unsigned long long)__popc(needMask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need) {
                const uint64_t my = base + (uint64_t)__popc(needMask & lanesBelow);
                if (my < n) {
                    ray = __ldg(queue + my);
                    walk_begin(w, s, make_float3(__ldg(ox + ray), __ldg(oy + ray), __ldg(oz + ray)),
                               make_float3(__ldg(dx + ray), __ldg(dy + ray), __ldg(dz + ray)), __ldg(tmax + ray));
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active && walk_step<ANY_HIT, BOUNDS>(w, s, err, s_top, stage)) {
            if (ANY_HIT) {
                occluded[ray] = w.slot >= 0 ? 1 : 0;
            } else {
                slot[ray] = w.slot;
                t[ray] = w.len;
                u[ray] = w.u;
                v[ray] = w.v;
            }
            active = false;
        }
    }
}

// Group walker (modes 3 and 4), second launch after the root prefilter: G
// lanes walk one ray together. A node round tests the G consecutive nodes
// [node, node + G) of the preorder array (one coalesced 32G-byte load), then
// resolves which of them the sequential walk visits by pointer jumping over
// the in-window successors (log2 G shuffles): the walk leaves the window at
// a node outside it, at the end of the escape chain, or at a hit leaf. A leaf
// round tests G slots of the leaf block at once and applies the sequential
// acceptance rule (a slot is accepted when hit < rayLength, so the result is
// the first slot reaching the minimum; any hit: the first accepted slot).
// Every node decision uses the same arithmetic and the same rayLength as in
// trace_ray, so results are identical; tests of nodes the walk skips are
// discarded. A round advances one ray by several of trace_ray's steps, which
// shortens the dependent fetch chain of the longest walks.
template <bool ANY_HIT, int BOUNDS, int G>
__global__ void __launch_bounds__(128) k_trace_group(
    DevScene s, const float* __restrict__ ox, const float* __restrict__ oy, const float* __restrict__ oz,
    const float* __restrict__ dx, const float* __restrict__ dy, const float* __restrict__ dz,
    const float* __restrict__ tmax, int32_t* __restrict__ slot, float* __restrict__ t, float* __restrict__ u,
    float* __restrict__ v, uint8_t* __restrict__ occluded, const uint32_t* __restrict__ queue,
    unsigned long long* counters, uint32_t* err) {
    static_assert(G == 4 || G == 8 || G == 16, "group size");
    constexpr uint32_t kDone = 0xFFFFFFFFu, kLeafMark = 0x80000000u;
    const uint64_t n = counters[1];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned gl = lane & (G - 1), gbase = lane & ~(unsigned)(G - 1);
    const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << gbase;
    float3 o = make_float3(0.0f, 0.0f, 0.0f), d = o, inv = o;
    float len = 0.0f, bu = 0.0f, bv = 0.0f;
    int32_t best = -1;
    uint32_t node = 0, cur = 0, end = 0, resume = kDone, budget = 0, ray = 0;
    bool active = false, exhausted = false;
    while (true) {
        // refill: one atomic per warp for all groups that need a ray
        const bool need = !active && !exhausted;
        const unsigned needMask = __ballot_sync(0xffffffffu, need && gl == 0);
        if (needMask) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(counters + 2, (unsigned long long)__popc(needMask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (need) {
                const uint64_t my = base + (uint64_t)__popc(needMask & ((1u << gbase) - 1u));
                if (my < n) {
                    ray = __ldg(queue + my);
                    o = make_float3(__ldg(ox + ray), __ldg(oy + ray), __ldg(oz + ray));
                    d = make_float3(__ldg(dx + ray), __ldg(dy + ray), __ldg(dz + ray));
                    inv = make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z));
                    len = __ldg(tmax + ray);
                    best = -1;
                    bu = bv = 0.0f;
                    node = 0;
                    cur = end = 0;
                    resume = kDone;
                    budget = s.numNodes;
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (!active) continue;
        bool finished = false;
        if (cur < end) {
            // leaf round: slots [cur, min(cur + G, end))
            const uint32_t k = cur + gl;
            float h = 0.0f, by = 0.0f, bz = 0.0f;
            bool ok = false;
            if (k < end) ok = intersect_triangle(o, d, s.tris + 3 * (size_t)k, h, by, bz) && h < len;
            if (ANY_HIT) {
                uint32_t key = ok ? k : kDone;
#pragma unroll
                for (int off = G / 2; off > 0; off >>= 1) key = min(key, __shfl_xor_sync(gmask, key, off));
                if (key != kDone) {
                    best = (int32_t)key;
                    finished = true;
                }
            } else {
                unsigned long long key = ok ? ((unsigned long long)__float_as_uint(h) << 32) | k : ~0ull;
#pragma unroll
                for (int off = G / 2; off > 0; off >>= 1) {
                    const unsigned long long other = __shfl_xor_sync(gmask, key, off);
                    key = other < key ? other : key;
                }
                const uint32_t win = (uint32_t)key;
                const unsigned src = gbase + ((key != ~0ull) ? (win - cur) : 0u);
                const float wu = __shfl_sync(gmask, by, src), wv = __shfl_sync(gmask, bz, src);
                if (key != ~0ull) {
                    best = (int32_t)win;
                    len = __uint_as_float((uint32_t)(key >> 32));
                    bu = wu;
                    bv = wv;
                }
            }
            cur = min(cur + G, end);
            if (!finished && cur >= end) {
                node = resume;
                if (node == kDone) finished = true;
            }
        } else {
            // node round: nodes [node, node + G)
            if (budget-- == 0) {
                raise_error(err, DEVERR_TRAVERSAL_CAP);
                finished = true;
            } else {
                const uint32_t p = node + gl;
                uint32_t next = kDone, child = 0, escape = 0;
                if (p < s.numNodes) {
                    const float4 a = __ldg(s.nodes + 2 * (size_t)p), b = __ldg(s.nodes + 2 * (size_t)p + 1);
                    child = __float_as_uint(a.w);
                    escape = __float_as_uint(b.w);
                    float firstHit;
                    bool hit;
                    if (BOUNDS == 0) hit = intersect_box(o, inv, a, b, firstHit);
                    else hit = intersect_ellipsoid(o, d, a, b, firstHit);
                    if (hit && firstHit <= len) next = (child & LEAF_FLAG) ? (kLeafMark | gl) : child;
                    else next = escape ? escape : kDone;
                }
                // pointer jumping over successors inside the window
#pragma unroll
                for (int r = 1; r < G; r <<= 1) {
                    const bool chase = next < kLeafMark && next - node < (uint32_t)G;
                    const uint32_t w = __shfl_sync(gmask, next, gbase + (chase ? next - node : gl));
                    next = chase ? w : next;
                }
                const uint32_t r0 = __shfl_sync(gmask, next, gbase);
                if (r0 == kDone) {
                    finished = true;
                } else if (r0 & kLeafMark) {
                    const unsigned src = gbase + (r0 & (kLeafMark - 1u));
                    const uint32_t lc = __shfl_sync(gmask, child, src), le = __shfl_sync(gmask, escape, src);
                    cur = (lc & LEAF_BLOCK_MASK) * s.leafSize;
                    end = cur + ((lc >> LEAF_COUNT_SHIFT) & LEAF_COUNT_MASK);
                    resume = le ? le : kDone;
                    if (cur >= end) {  // empty leaf block
                        node = resume;
                        if (node == kDone) finished = true;
                    }
                } else {
                    node = r0;
                }
            }
        }
        if (finished) {
            if (gl == 0) {
                if (ANY_HIT) {
                    occluded[ray] = best >= 0 ? 1 : 0;
                } else {
                    slot[ray] = best;
                    t[ray] = len;
                    u[ray] = bu;
                    v[ray] = bv;
                }
            }
            active = false;
        }
    }
}

gpugi_status launch_trace_filtered(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                   const float* oy, const float* oz, const float* dx, const float* dy,
                                   const float* dz, const float* tmax, uint64_t n, int32_t* slot, float* t,
                                   float* u, float* v, uint8_t* occluded) {
    if (n == 0) return GPUGI_OK;
    if (n > 0xFFFFFFFFull) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "mode 2 handles at most 2^32-1 rays per call");
    gpugi_status st = ensure_queue(ctx, n);
    if (st) return st;
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(ctx->scratch);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    return launch_trace_filtered_on(ctx, sc, anyHit, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, occluded,
                                    ctx->queue, counters);
}

// The same two launches as launch_trace_filtered, on scratch memory the
// caller provides (queue of n entries, 4 zeroed counters); allocates nothing.
gpugi_status launch_trace_filtered_on(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                      const float* oy, const float* oz, const float* dx, const float* dy,
                                      const float* dz, const float* tmax, uint64_t n, int32_t* slot, float* t,
                                      float* u, float* v, uint8_t* occluded, uint32_t* queue,
                                      unsigned long long* counters) {
    if (n == 0) return GPUGI_OK;
    const bool ell = sc->dev.boundsKind == GPUGI_BOUNDS_ELLIPSOID;
    const unsigned grid1 = (unsigned)((n + 255) / 256);
#define GPUGI_FILTER_ON(A, B)                                                                                       \
    k_trace_root_filter<A, B><<<grid1, 256, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, \
                                                              v, occluded, queue, counters)
    if (!ell) {
        if (anyHit) GPUGI_FILTER_ON(true, 0);
        else GPUGI_FILTER_ON(false, 0);
    } else {
        if (anyHit) GPUGI_FILTER_ON(true, 1);
        else GPUGI_FILTER_ON(false, 1);
    }
#undef GPUGI_FILTER_ON
    if (ctx->traceMode == 3 || ctx->traceMode == 4) {
        void (*kg)(DevScene, const float*, const float*, const float*, const float*, const float*, const float*,
                   const float*, int32_t*, float*, float*, float*, uint8_t*, const uint32_t*, unsigned long long*,
                   uint32_t*);
        if (ctx->traceMode == 3) {
            if (!ell) kg = anyHit ? k_trace_group<true, 0, 8> : k_trace_group<false, 0, 8>;
            else kg = anyHit ? k_trace_group<true, 1, 8> : k_trace_group<false, 1, 8>;
        } else {
            if (!ell) kg = anyHit ? k_trace_group<true, 0, 4> : k_trace_group<false, 0, 4>;
            else kg = anyHit ? k_trace_group<true, 1, 4> : k_trace_group<false, 1, 4>;
        }
        WalkerLaunch L;
        gpugi_status st = walker_launch_config(ctx, sc, (const void*)kg, 1ull << 40, 0, L);
        if (st) return st;
        kg<<<L.grid, 128, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, slot, t, u, v, occluded, queue,
                                           counters, ctx->errWord);
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        return GPUGI_OK;
    }
    void (*k)(DevScene, const float*, const float*, const float*, const float*, const float*, const float*,
              const float*, int32_t*, float*, float*, float*, uint8_t*, const uint32_t*, unsigned long long*,
              uint32_t*, uint32_t);
    if (!ell) k = anyHit ? k_trace_queue<true, 0> : k_trace_queue<false, 0>;
    else k = anyHit ? k_trace_queue<true, 1> : k_trace_queue<false, 1>;
    WalkerLaunch L;
    gpugi_status st = walker_launch_config(ctx, sc, (const void*)k, n, ctx->sharedNodes, L);
    if (st) return st;
    k<<<L.grid, 128, L.smem, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, slot, t, u, v, occluded, queue,
                                            counters, ctx->errWord, L.stage);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

template <int BOUNDS, bool ANY>
__global__ void __launch_bounds__(256) k_trace_stats(DevScene s, const float* __restrict__ ox,
                                                     const float* __restrict__ oy, const float* __restrict__ oz,
                                                     const float* __restrict__ dx, const float* __restrict__ dy,
                                                     const float* __restrict__ dz, const float* __restrict__ tmax,
                                                     uint64_t n, unsigned long long* sums, uint32_t* err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    WalkCounters c;
    if (i < n) {
        const float3 o = make_float3(ox[i], oy[i], oz[i]);
        const float3 d = make_float3(dx[i], dy[i], dz[i]);
        trace_ray<ANY, BOUNDS, true>(s, o, d, tmax[i], err, &c);
    }
    unsigned long long a = c.nodes, b = c.slots, t = c.tris;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
        t += __shfl_down_sync(0xffffffffu, t, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sums, a);
        atomicAdd(sums + 1, b);
        atomicAdd(sums + 2, t);
    }
}

gpugi_status launch_trace_stats(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                const float* oz, const float* dx, const float* dy, const float* dz,
                                const float* tmax, uint64_t n, uint32_t anyHit, unsigned long long* sums) {
    if (n == 0) return GPUGI_OK;
    const unsigned grid = (unsigned)((n + 255) / 256);
    const bool ell = sc->dev.boundsKind == GPUGI_BOUNDS_ELLIPSOID;
    if (!ell && !anyHit)
        k_trace_stats<0, false><<<grid, 256, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, sums, ctx->errWord);
    else if (!ell)
        k_trace_stats<0, true><<<grid, 256, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, sums, ctx->errWord);
    else if (!anyHit)
        k_trace_stats<1, false><<<grid, 256, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, sums, ctx->errWord);
    else
        k_trace_stats<1, true><<<grid, 256, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, sums, ctx->errWord);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

static unsigned grid_for(uint64_t n, uint32_t block) { return (unsigned)((n + block - 1) / block); }

gpugi_status launch_trace_closest(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                  const float* oz, const float* dx, const float* dy, const float* dz,
                                  const float* tmax, uint64_t n, int32_t* slot, float* t, float* u, float* v) {
    if (n == 0) return GPUGI_OK;
    if (n > (uint64_t)0xFFFFFFFFu * 256u) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "too many rays");
    if (ctx->traceMode >= 2)
        return launch_trace_filtered(ctx, sc, false, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, nullptr);
    if (ctx->traceMode == 1)
        return launch_trace_persistent(ctx, sc, false, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, nullptr);
    const uint32_t block = ctx->traceBlock;
    if (sc->dev.boundsKind == GPUGI_BOUNDS_AABB)
        k_trace_closest<0><<<grid_for(n, block), block, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n,
                                                                           slot, t, u, v, ctx->errWord);
    else
        k_trace_closest<1><<<grid_for(n, block), block, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n,
                                                                           slot, t, u, v, ctx->errWord);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

gpugi_status launch_trace_any(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                              const float* oz, const float* dx, const float* dy, const float* dz,
                              const float* tmax, uint64_t n, uint8_t* occluded) {
    if (n == 0) return GPUGI_OK;
    if (n > (uint64_t)0xFFFFFFFFu * 256u) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "too many rays");
    if (ctx->traceMode >= 2)
        return launch_trace_filtered(ctx, sc, true, ox, oy, oz, dx, dy, dz, tmax, n, nullptr, nullptr, nullptr,
                                     nullptr, occluded);
    if (ctx->traceMode == 1)
        return launch_trace_persistent(ctx, sc, true, ox, oy, oz, dx, dy, dz, tmax, n, nullptr, nullptr, nullptr,
                                       nullptr, occluded);
    const uint32_t block = ctx->traceBlock;
    if (sc->dev.boundsKind == GPUGI_BOUNDS_AABB)
        k_trace_any<0><<<grid_for(n, block), block, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n,
                                                                       occluded, ctx->errWord);
    else
        k_trace_any<1><<<grid_for(n, block), block, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n,
                                                                       occluded, ctx->errWord);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

}  // namespace gpugi
