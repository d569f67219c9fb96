// Ray-query kernels behind gpugi_trace_closest / gpugi_trace_any.
//
// One ray per thread; rays and results are structure-of-arrays so every
// load and store of a warp is a single coalesced 128-B transaction. The
// walk itself reads 32-B nodes and 48-B triangle records through the
// read-only (non-coherent) path with 16-B vector loads.
#include <type_traits>

#include "ctx.cuh"
#include "trace.cuh"

// Resident blocks per SM the group walker is compiled for (registers).
#ifndef GPUGI_GROUP_MIN_BLOCKS
#define GPUGI_GROUP_MIN_BLOCKS 10
#endif

namespace gpugi {

// Picks a kernel instantiation at run time: f receives (any hit, bounds kind
// 0/1/2, triangle test) as integral constants and returns the kernel's address.
template <typename A, typename F>
static auto pick_bounds(A a, int bounds, bool wt, F f) {
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    if (bounds == GPUGI_BOUNDS_ELLIPSOID) return wt ? f(a, I1{}, I1{}) : f(a, I1{}, I0{});
    if (bounds == GPUGI_BOUNDS_OBOX) return wt ? f(a, I2{}, I1{}) : f(a, I2{}, I0{});
    return wt ? f(a, I0{}, I1{}) : f(a, I0{}, I0{});
}
template <typename F>
static auto pick_variant(bool anyHit, int bounds, bool wt, F f) {
    return anyHit ? pick_bounds(std::true_type{}, bounds, wt, f) : pick_bounds(std::false_type{}, bounds, wt, f);
}

template <int BOUNDS, int TRI>
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
    TraceResult r = trace_ray<false, BOUNDS, false, TRI>(s, o, d, __ldg(tmax + i), err);
    slot[i] = r.slot;
    t[i] = r.t;
    u[i] = r.u;
    v[i] = r.v;
}

template <int BOUNDS, int TRI>
__global__ void __launch_bounds__(256) k_trace_any(DevScene s, const float* __restrict__ ox,
                                                   const float* __restrict__ oy, const float* __restrict__ oz,
                                                   const float* __restrict__ dx, const float* __restrict__ dy,
                                                   const float* __restrict__ dz, const float* __restrict__ tmax,
                                                   uint64_t n, uint8_t* __restrict__ occluded, uint32_t* err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 o = make_float3(__ldg(ox + i), __ldg(oy + i), __ldg(oz + i));
    const float3 d = make_float3(__ldg(dx + i), __ldg(dy + i), __ldg(dz + i));
    TraceResult r = trace_ray<true, BOUNDS, false, TRI>(s, o, d, __ldg(tmax + i), err);
    occluded[i] = r.slot >= 0 ? 1 : 0;
}

gpugi_status walker_launch_config(gpugi_ctx* ctx, const gpugi_scene* sc, const void* kernel, uint64_t n,
                                  uint32_t maxStage, WalkerLaunch& out) {
    out.stage = sc->dev.topNodes < maxStage ? sc->dev.topNodes : maxStage;
    out.smem = (size_t)out.stage * 32;
    if (out.smem > 48 * 1024)
        GPUGI_CUDA_TRY(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)out.smem));
    int perSM = -1;
    for (const auto& e : ctx->occupancy)
        if (e.first.first == kernel && e.first.second == out.smem) perSM = e.second;
    if (perSM < 0) {
        GPUGI_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, 128, out.smem));
        ctx->occupancy.push_back({{kernel, out.smem}, perSM});
    }
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
template <bool ANY_HIT, int BOUNDS, int TRI>
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
        if (active && walk_step<ANY_HIT, BOUNDS, TRI>(w, s, err, s_top, stage)) {
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
    auto k = pick_variant(anyHit, (int)sc->dev.boundsKind, sc->dev.triangleTest != 0, [](auto A, auto B, auto T) {
        return &k_trace_persistent<decltype(A)::value, decltype(B)::value, decltype(T)::value>;
    });
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
template <bool ANY_HIT, int BOUNDS, int TRI>
__global__ void __launch_bounds__(256) k_trace_root_filter(
    DevScene s, const float* __restrict__ ox, const float* __restrict__ oy, const float* __restrict__ oz,
    const float* __restrict__ dx, const float* __restrict__ dy, const float* __restrict__ dz,
    const float* __restrict__ tmax, uint64_t n, int32_t* __restrict__ slot, float* __restrict__ t,
    float* __restrict__ u, float* __restrict__ v, uint8_t* __restrict__ occluded, uint32_t* __restrict__ queue,
    unsigned long long* counters, uint32_t rayBase) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool pass = false;
    if (i < n) {
        const float3 o = make_float3(__ldg(ox + i), __ldg(oy + i), __ldg(oz + i));
        const float3 d = make_float3(__ldg(dx + i), __ldg(dy + i), __ldg(dz + i));
        const float len = __ldg(tmax + i);
        const float4 a = __ldg(s.nodes), b = __ldg(s.nodes + 1);
        const float4 c = BOUNDS == 2 ? __ldg(s.nodes + 2) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float firstHit;
        const bool hit = bounds_test<BOUNDS, TRI != 0>(o, d, make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z)), a,
                                                       b, c, firstHit);
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
    if (pass) queue[base + __popc(ballot & ((1u << lane) - 1u))] = rayBase + (uint32_t)i;
}

// The same prefilter for four consecutive rays per thread with 16-B loads
// and stores (all ray and result arrays 16-B aligned; rays [0, 4 n4)). Rays
// that pass are appended with one atomic per warp (warp prefix sum of the
// per-thread counts). Results of passing rays are written too and later
// overwritten by the walker.
template <bool ANY_HIT, int BOUNDS, int TRI>
__global__ void __launch_bounds__(256) k_trace_root_filter4(
    DevScene s, const float4* __restrict__ ox, const float4* __restrict__ oy, const float4* __restrict__ oz,
    const float4* __restrict__ dx, const float4* __restrict__ dy, const float4* __restrict__ dz,
    const float4* __restrict__ tmax, uint64_t n4, int4* __restrict__ slot, float4* __restrict__ t,
    float4* __restrict__ u, float4* __restrict__ v, uchar4* __restrict__ occluded, uint32_t* __restrict__ queue,
    unsigned long long* counters) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned pass = 0;
    if (i < n4) {
        const float4 X = __ldg(ox + i), Y = __ldg(oy + i), Z = __ldg(oz + i);
        const float4 DX = __ldg(dx + i), DY = __ldg(dy + i), DZ = __ldg(dz + i), L = __ldg(tmax + i);
        const float4 a = __ldg(s.nodes), b = __ldg(s.nodes + 1);
        const float4 c = BOUNDS == 2 ? __ldg(s.nodes + 2) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float xs[4] = {X.x, X.y, X.z, X.w}, ys[4] = {Y.x, Y.y, Y.z, Y.w}, zs[4] = {Z.x, Z.y, Z.z, Z.w};
        const float dxs[4] = {DX.x, DX.y, DX.z, DX.w}, dys[4] = {DY.x, DY.y, DY.z, DY.w},
                    dzs[4] = {DZ.x, DZ.y, DZ.z, DZ.w}, ls[4] = {L.x, L.y, L.z, L.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float3 o = make_float3(xs[k], ys[k], zs[k]), d = make_float3(dxs[k], dys[k], dzs[k]);
            float firstHit;
            const bool hit = bounds_test<BOUNDS, TRI != 0>(o, d, make_float3(X::rcp(d.x), X::rcp(d.y), X::rcp(d.z)),
                                                           a, b, c, firstHit);
            if (hit && firstHit <= ls[k]) pass |= 1u << k;
        }
        if (ANY_HIT) {
            occluded[i] = make_uchar4(0, 0, 0, 0);
        } else {
            slot[i] = make_int4(-1, -1, -1, -1);
            t[i] = L;
            u[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            v[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned cnt = __popc(pass);
    unsigned incl = cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned up = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= (unsigned)off) incl += up;
    }
    // one queue reservation per block: warp totals, their exclusive prefix
    // sum, one atomic (instead of one per warp on the same counter)
    __shared__ unsigned s_warp[32];
    __shared__ unsigned long long s_base;
    const unsigned warp = threadIdx.x >> 5;
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned total = 0;
        for (unsigned w = 0; w < (blockDim.x + 31u) >> 5; ++w) {
            const unsigned c = s_warp[w];
            s_warp[w] = total;
            total += c;
        }
        s_base = total ? atomicAdd(counters + 1, (unsigned long long)total) : 0ull;
    }
    __syncthreads();
    uint64_t at = s_base + s_warp[warp] + (incl - cnt);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (pass & (1u << k)) queue[at++] = (uint32_t)(4 * i + k);
}

// Second launch: the persistent walker over the queued ray indices.
template <bool ANY_HIT, int BOUNDS, int TRI>
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
        if (active && walk_step<ANY_HIT, BOUNDS, TRI>(w, s, err, s_top, stage)) {
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
// lanes walk each queued ray together (group_step), which shortens the
// dependent fetch chain of the longest walks.
template <bool ANY_HIT, int BOUNDS, int G, int TRI>
__global__ void __launch_bounds__(128, GPUGI_GROUP_MIN_BLOCKS) k_trace_group(
    DevScene s, const float* __restrict__ ox, const float* __restrict__ oy, const float* __restrict__ oz,
    const float* __restrict__ dx, const float* __restrict__ dy, const float* __restrict__ dz,
    const float* __restrict__ tmax, int32_t* __restrict__ slot, float* __restrict__ t, float* __restrict__ u,
    float* __restrict__ v, uint8_t* __restrict__ occluded, const uint32_t* __restrict__ queue,
    unsigned long long* counters, uint32_t* err) {
    group_walks<ANY_HIT, BOUNDS, G, TRI>(
        s, counters[1], counters + 2, err,
        [&](uint64_t i, float3& o, float3& d, float& len) {
            const uint32_t ray = __ldg(queue + i);
            o = make_float3(__ldg(ox + ray), __ldg(oy + ray), __ldg(oz + ray));
            d = make_float3(__ldg(dx + ray), __ldg(dy + ray), __ldg(dz + ray));
            len = __ldg(tmax + ray);
        },
        [&](uint64_t i, const GroupWalk& g) {
            const uint32_t ray = __ldg(queue + i);
            if (ANY_HIT) {
                occluded[ray] = g.slot >= 0 ? 1 : 0;
            } else {
                slot[ray] = g.slot;
                t[ray] = g.len;
                u[ray] = g.u;
                v[ray] = g.v;
            }
        });
}

// walkerShare percent of a persistent walker grid (at least one block).
static unsigned share_of_grid(unsigned grid, uint32_t walkerShare) {
    if (walkerShare >= 100) return grid;
    const uint64_t g = (uint64_t)grid * (walkerShare ? walkerShare : 1) / 100;
    return g ? (unsigned)g : 1u;
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
                                      unsigned long long* counters, cudaStream_t stream, uint32_t walkerShare) {
    if (n == 0) return GPUGI_OK;
    cudaStream_t cs = stream ? stream : ctx->stream;
    const int ell = (int)sc->dev.boundsKind;  // bounds kind: 0 box, 1 ellipsoid, 2 oriented box
    const bool wt = sc->dev.triangleTest != 0;
    // four rays per thread with 16-B accesses when every array allows it
    auto al = [](const void* p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; };
    const bool vec = al(ox) && al(oy) && al(oz) && al(dx) && al(dy) && al(dz) && al(tmax) && al(slot) && al(t) &&
                     al(u) && al(v) && (occluded == nullptr || ((uintptr_t)occluded & 3u) == 0);
    const uint64_t n4 = vec ? n / 4 : 0, head = 4 * n4;
    if (n4) {
        const unsigned grid4 = (unsigned)((n4 + 255) / 256);
        auto f4 = [](const float* p) { return reinterpret_cast<const float4*>(p); };
        auto kf = pick_variant(anyHit, ell, wt, [](auto A, auto B, auto T) {
            return &k_trace_root_filter4<decltype(A)::value, decltype(B)::value, decltype(T)::value>;
        });
        kf<<<grid4, 256, 0, cs>>>(sc->dev, f4(ox), f4(oy), f4(oz), f4(dx), f4(dy), f4(dz), f4(tmax), n4,
                                  reinterpret_cast<int4*>(slot), reinterpret_cast<float4*>(t),
                                  reinterpret_cast<float4*>(u), reinterpret_cast<float4*>(v),
                                  reinterpret_cast<uchar4*>(occluded), queue, counters);
    }
    if (head < n) {
        const uint64_t m = n - head;
        const unsigned grid1 = (unsigned)((m + 255) / 256);
        auto sh = [&](const float* p) { return p + head; };
        auto kf = pick_variant(anyHit, ell, wt, [](auto A, auto B, auto T) {
            return &k_trace_root_filter<decltype(A)::value, decltype(B)::value, decltype(T)::value>;
        });
        kf<<<grid1, 256, 0, cs>>>(sc->dev, sh(ox), sh(oy), sh(oz), sh(dx), sh(dy), sh(dz), sh(tmax), m,
                                  slot ? slot + head : nullptr, t ? t + head : nullptr, u ? u + head : nullptr,
                                  v ? v + head : nullptr, occluded ? occluded + head : nullptr, queue, counters,
                                  (uint32_t)head);
    }
    if (ctx->traceMode >= 3) {
        auto kg = ctx->traceMode == 3
                      ? pick_variant(anyHit, ell, wt, [](auto A, auto B, auto T) {
                            return &k_trace_group<decltype(A)::value, decltype(B)::value, 8, decltype(T)::value>;
                        })
                  : ctx->traceMode == 4
                      ? pick_variant(anyHit, ell, wt, [](auto A, auto B, auto T) {
                            return &k_trace_group<decltype(A)::value, decltype(B)::value, 4, decltype(T)::value>;
                        })
                      : pick_variant(anyHit, ell, wt, [](auto A, auto B, auto T) {
                            return &k_trace_group<decltype(A)::value, decltype(B)::value, 16, decltype(T)::value>;
                        });
        WalkerLaunch L;
        gpugi_status st = walker_launch_config(ctx, sc, (const void*)kg, 1ull << 40, 0, L);
        if (st) return st;
        L.grid = share_of_grid(L.grid, walkerShare);
        kg<<<L.grid, 128, 0, cs>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, slot, t, u, v, occluded, queue,
                                           counters, ctx->errWord);
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        return GPUGI_OK;
    }
    auto k = pick_variant(anyHit, ell, wt, [](auto A, auto B, auto T) {
        return &k_trace_queue<decltype(A)::value, decltype(B)::value, decltype(T)::value>;
    });
    WalkerLaunch L;
    gpugi_status st = walker_launch_config(ctx, sc, (const void*)k, n, ctx->sharedNodes, L);
    if (st) return st;
    L.grid = share_of_grid(L.grid, walkerShare);
    k<<<L.grid, 128, L.smem, cs>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, slot, t, u, v, occluded, queue,
                                            counters, ctx->errWord, L.stage);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

template <int BOUNDS, bool ANY, int TRI>
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
        trace_ray<ANY, BOUNDS, true, TRI>(s, o, d, tmax[i], err, &c);
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
    auto k = pick_variant(anyHit != 0, (int)sc->dev.boundsKind, sc->dev.triangleTest != 0, [](auto A, auto B, auto T) {
        return &k_trace_stats<decltype(B)::value, decltype(A)::value, decltype(T)::value>;
    });
    k<<<grid, 256, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, sums, ctx->errWord);
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
    auto k = pick_variant(false, (int)sc->dev.boundsKind, sc->dev.triangleTest != 0,
                          [](auto, auto B, auto T) { return &k_trace_closest<decltype(B)::value, decltype(T)::value>; });
    k<<<grid_for(n, block), block, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v,
                                                     ctx->errWord);
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
    auto k = pick_variant(true, (int)sc->dev.boundsKind, sc->dev.triangleTest != 0,
                          [](auto, auto B, auto T) { return &k_trace_any<decltype(B)::value, decltype(T)::value>; });
    k<<<grid_for(n, block), block, 0, ctx->stream>>>(sc->dev, ox, oy, oz, dx, dy, dz, tmax, n, occluded,
                                                     ctx->errWord);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

}  // namespace gpugi
