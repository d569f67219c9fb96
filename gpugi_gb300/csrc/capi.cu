// Context lifetime, error reporting and the ray-query entry points of the C ABI.
#include <algorithm>
#include <cstring>

#include "ctx.cuh"

namespace gpugi {

gpugi_status fail(gpugi_ctx* ctx, gpugi_status st, const std::string& msg) {
    if (ctx) ctx->lastError = msg;
    return st;
}

gpugi_status cuda_fail(gpugi_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, GPUGI_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

gpugi_status ensure_stage(gpugi_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->stageDevBytes) return GPUGI_OK;
    if (ctx->stageDev) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->stageDev);
        ctx->stageDev = nullptr;
        ctx->stageDevBytes = 0;
    }
    size_t want = bytes + bytes / 4;
    if (cudaMalloc(&ctx->stageDev, want) != cudaSuccess) {
        ctx->stageDev = nullptr;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "staging buffer allocation failed");
    }
    ctx->stageDevBytes = want;
    return GPUGI_OK;
}

gpugi_status ensure_queue(gpugi_ctx* ctx, uint64_t n) {
    if (n <= ctx->queueCap) return GPUGI_OK;
    if (ctx->queue) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->queue);
        ctx->queue = nullptr;
        ctx->queueCap = 0;
    }
    const uint64_t want = n + n / 4;
    if (cudaMalloc(&ctx->queue, want * sizeof(uint32_t)) != cudaSuccess) {
        ctx->queue = nullptr;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "ray queue allocation failed");
    }
    ctx->queueCap = want;
    return GPUGI_OK;
}

static gpugi_status check_device_error(gpugi_ctx* ctx) {
    uint32_t bits = 0;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&bits, ctx->errWord, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (bits) {
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(ctx->errWord, 0, 4, ctx->stream));
        char msg[96];
        std::snprintf(msg, sizeof msg, "device guard fired (error bits 0x%x)", bits);
        return fail(ctx, GPUGI_ERROR_DEVICE, msg);
    }
    return GPUGI_OK;
}

// The error word as copied into ctx->errHost by a call's last copies (the
// caller has synchronised them): no extra round trip.
static gpugi_status check_copied_device_error(gpugi_ctx* ctx) {
    const uint32_t bits = *ctx->errHost;
    if (bits) {
        *ctx->errHost = 0;
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(ctx->errWord, 0, 4, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        char msg[96];
        std::snprintf(msg, sizeof msg, "device guard fired (error bits 0x%x)", bits);
        return fail(ctx, GPUGI_ERROR_DEVICE, msg);
    }
    return GPUGI_OK;
}

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static gpugi_status ensure_pipeline(gpugi_ctx* ctx) {
    if (ctx->copyIn) return GPUGI_OK;
    GPUGI_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copyIn, cudaStreamNonBlocking));
    GPUGI_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copyOut, cudaStreamNonBlocking));
    GPUGI_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->compute2, cudaStreamNonBlocking));
    for (int k = 0; k < 8; ++k) {
        GPUGI_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->evIn[k], cudaEventDisableTiming));
        GPUGI_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->evTraced[k], cudaEventDisableTiming));
    }
    return GPUGI_OK;
}

// Ray queries on host arrays. Rays go through device staging in chunks of at
// most 2^22. With trace modes 2-5 a chunk is split into ctx->hostParts parts
// whose copies in (copyIn stream), traversal (the context stream and a second
// one, alternating by part) and copies out (copyOut stream) overlap: part p+1
// uploads while part p is traced, part p downloads while part p+1 is traced,
// and the traversals of neighbouring parts overlap too. Each part has its own
// queue range and counters. Returns when every result is in host memory.
// Device address of page-locked host memory (cudaHostAlloc / cudaHostRegister),
// or nullptr for any other memory.
static void* mapped_host(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear the error of an unknown pointer
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Copies `count` columns of `width` bytes between host and device. When
// the columns sit at one common spacing on both sides (the rays and results
// of one structure-of-arrays block; the device staging columns always do),
// they travel as one 2D copy, else (or when the runtime refuses the 2D copy
// because the columns belong to different allocations) column by column. A copy over the host
// link has a fixed cost of a few microseconds: a 2^20-ray batch moved as
// 7 + 4 separate columns takes ~35 us longer than as one block each way.
static size_t column_spacing(const void* const p[], int count, size_t width) {
    if (count < 2) return 0;
    const uintptr_t b = reinterpret_cast<uintptr_t>(p[0]), c = reinterpret_cast<uintptr_t>(p[1]);
    if (c <= b || c - b < width || c - b > (uintptr_t)INT32_MAX) return 0;
    const uintptr_t pitch = c - b;
    for (int k = 2; k < count; ++k)
        if (reinterpret_cast<uintptr_t>(p[k]) != b + (uintptr_t)k * pitch) return 0;
    return (size_t)pitch;
}
static gpugi_status copy_columns(gpugi_ctx* ctx, void* const dst[], const void* const src[], int count, size_t width,
                                 cudaMemcpyKind kind, cudaStream_t s) {
    const size_t dp = column_spacing(dst, count, width), sp = column_spacing(src, count, width);
    if (dp && sp) {
        const cudaError_t e = cudaMemcpy2DAsync(dst[0], dp, src[0], sp, width, (size_t)count, kind, s);
        if (e == cudaSuccess) return GPUGI_OK;
        if (e != cudaErrorInvalidValue) return cuda_fail(ctx, e, "cudaMemcpy2DAsync");
        // evenly spaced columns of different page-locked allocations: the
        // runtime refuses one copy across them (nothing was enqueued)
        cudaGetLastError();
    }
    for (int k = 0; k < count; ++k) GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dst[k], src[k], width, kind, s));
    return GPUGI_OK;
}
// The rays of [off, off + m) into the staging columns d (at +dOff), and the
// results back: slot, t, u, v (closest hit) or the occlusion bytes (any hit).
static gpugi_status copy_rays_in(gpugi_ctx* ctx, float* const d[7], uint64_t dOff, const float* const src[7],
                                 uint64_t off, uint64_t m, cudaStream_t s) {
    void* dst[7];
    const void* from[7];
    for (int k = 0; k < 7; ++k) {
        dst[k] = d[k] + dOff;
        from[k] = src[k] + off;
    }
    return copy_columns(ctx, dst, from, 7, m * 4, cudaMemcpyHostToDevice, s);
}
static gpugi_status copy_results_out(gpugi_ctx* ctx, bool anyHit, char* const dRes[4], uint64_t dOff,
                                     int32_t* slot, float* t, float* u, float* v, uint8_t* occ, uint64_t off,
                                     uint64_t m, cudaStream_t s) {
    if (anyHit) {
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(occ + off, dRes[0] + dOff, m, cudaMemcpyDeviceToHost, s));
        return GPUGI_OK;
    }
    void* dst[4] = {slot + off, t + off, u + off, v + off};
    const void* from[4];
    for (int k = 0; k < 4; ++k) from[k] = dRes[k] + 4 * dOff;
    return copy_columns(ctx, dst, from, 4, m * 4, cudaMemcpyDeviceToHost, s);
}

static gpugi_status trace_host(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* const src[7],
                               uint64_t n, int32_t* slot, float* t, float* u, float* v, uint8_t* occ) {
    // Page-locked arrays: the kernels read the rays and write the results
    // over the host link themselves (zero copy), with no staging round trip.
    if (ctx->hostZeroCopy) {
        const float* dsrc[7];
        bool ok = true;
        for (int k = 0; k < 7 && ok; ++k) ok = (dsrc[k] = static_cast<const float*>(mapped_host(src[k]))) != nullptr;
        void* dout[4] = {nullptr, nullptr, nullptr, nullptr};
        if (ok && anyHit) ok = (dout[0] = mapped_host(occ)) != nullptr;
        if (ok && !anyHit) {
            void* outs[4] = {slot, t, u, v};
            for (int k = 0; k < 4 && ok; ++k) ok = (dout[k] = mapped_host(outs[k])) != nullptr;
        }
        if (ok) {
            gpugi_status st = anyHit ? launch_trace_any(ctx, sc, dsrc[0], dsrc[1], dsrc[2], dsrc[3], dsrc[4], dsrc[5],
                                                        dsrc[6], n, static_cast<uint8_t*>(dout[0]))
                                     : launch_trace_closest(ctx, sc, dsrc[0], dsrc[1], dsrc[2], dsrc[3], dsrc[4],
                                                            dsrc[5], dsrc[6], n, static_cast<int32_t*>(dout[0]),
                                                            static_cast<float*>(dout[1]), static_cast<float*>(dout[2]),
                                                            static_cast<float*>(dout[3]));
            if (st) return st;
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->errHost, ctx->errWord, 4, cudaMemcpyDeviceToHost, ctx->stream));
            GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            return GPUGI_OK;
        }
    }
    const uint64_t chunk = n < (1ull << 22) ? n : (1ull << 22);
    const size_t col = align256(chunk * 4);
    gpugi_status st = ensure_stage(ctx, 11 * col);
    if (st) return st;
    char* base = static_cast<char*>(ctx->stageDev);
    float* d[7];
    for (int k = 0; k < 7; ++k) d[k] = reinterpret_cast<float*>(base + k * col);
    int32_t* dSlot = reinterpret_cast<int32_t*>(base + 7 * col);
    float* dT = reinterpret_cast<float*>(base + 8 * col);
    float* dU = reinterpret_cast<float*>(base + 9 * col);
    float* dV = reinterpret_cast<float*>(base + 10 * col);
    uint8_t* dOcc = reinterpret_cast<uint8_t*>(base + 7 * col);
    char* const dRes[4] = {base + 7 * col, base + 8 * col, base + 9 * col, base + 10 * col};
    const uint32_t parts = std::min<uint32_t>(std::max<uint32_t>(ctx->hostParts, 1u), 8u);
    const bool pipe = ctx->traceMode >= 2 && parts > 1 && chunk >= (1ull << 16);
    if (pipe) {
        if ((st = ensure_pipeline(ctx)) || (st = ensure_queue(ctx, chunk))) return st;
    }
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        if (!pipe) {
            if ((st = copy_rays_in(ctx, d, 0, src, off, m, ctx->stream))) return st;
            if (anyHit) st = launch_trace_any(ctx, sc, d[0], d[1], d[2], d[3], d[4], d[5], d[6], m, dOcc);
            else st = launch_trace_closest(ctx, sc, d[0], d[1], d[2], d[3], d[4], d[5], d[6], m, dSlot, dT, dU, dV);
            if (st) return st;
            if ((st = copy_results_out(ctx, anyHit, dRes, 0, slot, t, u, v, occ, off, m, ctx->stream))) return st;
            if (off + m >= n)  // the error word after the call's last traversal
                GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->errHost, ctx->errWord, 4, cudaMemcpyDeviceToHost, ctx->stream));
            continue;
        }
        // parts of whole float4 groups, so every part starts 16-B aligned
        const uint64_t per = ((m + parts - 1) / parts + 3) / 4 * 4;
        unsigned long long* counters = reinterpret_cast<unsigned long long*>(ctx->scratch);
        for (uint32_t p = 0; p < parts; ++p) {
            const uint64_t p0 = p * per;
            if (p0 >= m) break;
            const uint64_t mp = std::min(per, m - p0);
            if ((st = copy_rays_in(ctx, d, p0, src, off + p0, mp, ctx->copyIn))) return st;
            GPUGI_CUDA_TRY(ctx, cudaEventRecord(ctx->evIn[p], ctx->copyIn));
        }
        // parts alternate between two traversal streams: the walker of part
        // p+1 starts on the SMs that part p's walker frees in its tail
        for (uint32_t p = 0; p < parts; ++p) {
            const uint64_t p0 = p * per;
            if (p0 >= m) break;
            const uint64_t mp = std::min(per, m - p0);
            cudaStream_t cs = (p & 1u) ? ctx->compute2 : ctx->stream;
            GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(cs, ctx->evIn[p], 0));
            GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(counters + 4 * p, 0, 4 * sizeof(unsigned long long), cs));
            if ((st = launch_trace_filtered_on(ctx, sc, anyHit, d[0] + p0, d[1] + p0, d[2] + p0, d[3] + p0, d[4] + p0,
                                               d[5] + p0, d[6] + p0, mp, anyHit ? nullptr : dSlot + p0,
                                               anyHit ? nullptr : dT + p0, anyHit ? nullptr : dU + p0,
                                               anyHit ? nullptr : dV + p0, anyHit ? dOcc + p0 : nullptr,
                                               ctx->queue + p0, counters + 4 * p, cs)))
                return st;
            GPUGI_CUDA_TRY(ctx, cudaEventRecord(ctx->evTraced[p], cs));
        }
        for (uint32_t p = 0; p < parts; ++p) {
            const uint64_t p0 = p * per;
            if (p0 >= m) break;
            const uint64_t mp = std::min(per, m - p0);
            GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copyOut, ctx->evTraced[p], 0));
            if ((st = copy_results_out(ctx, anyHit, dRes, p0, slot, t, u, v, occ, off + p0, mp, ctx->copyOut)))
                return st;
        }
        // the next chunk reuses the staging columns; the last chunk also
        // brings back the error word (copyOut has waited for every traversal)
        if (off + m >= n)
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->errHost, ctx->errWord, 4, cudaMemcpyDeviceToHost, ctx->copyOut));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->copyOut));
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->compute2) GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->compute2));
    return GPUGI_OK;
}

}  // namespace gpugi

using namespace gpugi;

extern "C" {

const char* gpugi_version(void) {
    return gpugi::kChecked ? "gpugi_gb300 0.1 (sm_103a) checked" : "gpugi_gb300 0.1 (sm_103a)";
}

gpugi_status gpugi_create(gpugi_ctx** out, const gpugi_opts* opts) {
    if (!out) return GPUGI_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    gpugi_ctx* ctx = new gpugi_ctx();
    ctx->device = opts ? opts->device : 0;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        delete ctx;
        return GPUGI_ERROR_CUDA;
    }
    if (ctx->device < 0 || ctx->device >= count) {
        delete ctx;
        return GPUGI_ERROR_INVALID_ARGUMENT;
    }
    if ((e = cudaSetDevice(ctx->device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->errWord, 16)) != cudaSuccess || (e = cudaMemset(ctx->errWord, 0, 16)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->scratch, 256)) != cudaSuccess || (e = cudaMemset(ctx->scratch, 0, 256)) != cudaSuccess ||
        (e = cudaMallocHost(&ctx->errHost, 4)) != cudaSuccess) {
        if (ctx->errWord) cudaFree(ctx->errWord);
        if (ctx->scratch) cudaFree(ctx->scratch);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return GPUGI_ERROR_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->numSMs, cudaDevAttrMultiProcessorCount, ctx->device);
    *out = ctx;
    return GPUGI_OK;
}

void gpugi_destroy(gpugi_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->renderFree) ctx->renderFree(ctx);
    if (ctx->stageDev) cudaFree(ctx->stageDev);
    if (ctx->errWord) cudaFree(ctx->errWord);
    if (ctx->errHost) cudaFreeHost(ctx->errHost);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->queue) cudaFree(ctx->queue);
    for (auto& ss : ctx->streamScratch) {
        if (ss.lastUse) {
            cudaEventSynchronize(ss.lastUse);
            cudaEventDestroy(ss.lastUse);
        }
        if (ss.queue) cudaFree(ss.queue);
        if (ss.counters) cudaFree(ss.counters);
        if (ss.stage) cudaFree(ss.stage);
    }
    if (ctx->copyIn) {
        cudaStreamSynchronize(ctx->copyIn);
        cudaStreamSynchronize(ctx->copyOut);
        cudaStreamSynchronize(ctx->compute2);
        cudaStreamDestroy(ctx->copyIn);
        cudaStreamDestroy(ctx->copyOut);
        cudaStreamDestroy(ctx->compute2);
        for (int k = 0; k < 8; ++k) {
            cudaEventDestroy(ctx->evIn[k]);
            cudaEventDestroy(ctx->evTraced[k]);
        }
    }
    cudaStreamDestroy(ctx->stream);
    for (gpugi_ctx** ref : ctx->children) *ref = nullptr;
    delete ctx;
}

const char* gpugi_last_error(const gpugi_ctx* ctx) { return ctx ? ctx->lastError.c_str() : "null context"; }

void* gpugi_stream(gpugi_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

gpugi_status gpugi_sync(gpugi_ctx* ctx) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

gpugi_status gpugi_debug_raise_device_error(gpugi_ctx* ctx, uint32_t bits) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t cur = 0;
    GPUGI_CUDA_TRY(ctx, cudaMemcpy(&cur, ctx->errWord, 4, cudaMemcpyDeviceToHost));
    cur |= bits;
    GPUGI_CUDA_TRY(ctx, cudaMemcpy(ctx->errWord, &cur, 4, cudaMemcpyHostToDevice));
    return GPUGI_OK;
}

gpugi_status gpugi_device_error_bits(gpugi_ctx* ctx, uint32_t* bits) {
    if (!ctx || !bits) return GPUGI_ERROR_INVALID_ARGUMENT;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(bits, ctx->errWord, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(ctx->errWord, 0, 4, ctx->stream));
    return GPUGI_OK;
}

gpugi_status gpugi_set_trace_config(gpugi_ctx* ctx, uint32_t mode, uint32_t blockSize) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (mode > 5)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT,
                    "mode must be 0 (thread per ray), 1 (persistent), 2 (root prefilter + persistent) or "
                    "3/4/5 (root prefilter + 8/4/16-lane group walker)");
    if (blockSize == 0 || blockSize > 256 || blockSize % 32 != 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "blockSize must be a multiple of 32 in [32, 256]");
    ctx->traceMode = mode;
    ctx->traceBlock = blockSize;
    return GPUGI_OK;
}

gpugi_status gpugi_set_host_pipeline(gpugi_ctx* ctx, uint32_t parts, uint32_t zeroCopy) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (parts < 1 || parts > 8) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "parts must be in [1, 8]");
    ctx->hostParts = parts;
    ctx->hostZeroCopy = zeroCopy ? 1u : 0u;
    return GPUGI_OK;
}

gpugi_status gpugi_set_async_walker_share(gpugi_ctx* ctx, uint32_t percent) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (percent < 1 || percent > 100) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "percent must be in [1, 100]");
    ctx->asyncWalkerShare = percent;
    return GPUGI_OK;
}

gpugi_status gpugi_set_scene_layout(gpugi_ctx* ctx, uint32_t sharedNodes, uint32_t renderSharedNodes) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    // 227 KB of shared memory per block at most: 7,000 nodes of 32 B
    if (sharedNodes > 7000 || renderSharedNodes > 7000)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "at most 7000 staged nodes (227 KB of shared memory)");
    ctx->sharedNodes = sharedNodes;
    ctx->renderSharedNodes = renderSharedNodes;
    return GPUGI_OK;
}

gpugi_status gpugi_trace_closest_device(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                        const float* oz, const float* dx, const float* dy, const float* dz,
                                        const float* tmax, uint64_t n, int32_t* slot, float* t, float* u,
                                        float* v) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !slot || !t || !u || !v)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    return launch_trace_closest(ctx, sc, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v);
}

gpugi_status gpugi_trace_any_device(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                    const float* oz, const float* dx, const float* dy, const float* dz,
                                    const float* tmax, uint64_t n, uint8_t* occluded) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !occluded)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    return launch_trace_any(ctx, sc, ox, oy, oz, dx, dy, dz, tmax, n, occluded);
}

}  // extern "C"

namespace gpugi {

// Scratch of a caller stream: found by stream; a new stream takes a free set
// or, with GPUGI_MAX_QUERY_STREAMS sets in use, the least recently used one
// once the work that last used it has finished (its lastUse event; callers
// create and destroy streams freely). Before a set is used the stream also
// waits for that event, so a set never serves two streams at once even when
// a destroyed stream's handle comes back for a new one. Grown when a call
// needs more queue entries (after its last use has finished).
static gpugi_status stream_scratch(gpugi_ctx* ctx, cudaStream_t s, uint64_t n, gpugi_ctx::StreamScratch** out) {
    gpugi_ctx::StreamScratch* ss = nullptr;
    for (auto& e : ctx->streamScratch)
        if (e.stream == s) ss = &e;
    if (!ss && ctx->streamScratch.size() < kMaxQueryStreams) {
        ctx->streamScratch.push_back({});
        ss = &ctx->streamScratch.back();
        if (cudaMalloc(&ss->counters, 4 * sizeof(unsigned long long)) != cudaSuccess ||
            cudaEventCreateWithFlags(&ss->lastUse, cudaEventDisableTiming) != cudaSuccess) {
            if (ss->counters) cudaFree(ss->counters);
            ctx->streamScratch.pop_back();
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "query counters");
        }
        ss->stream = s;
    }
    if (!ss) {  // reuse the least recently used set
        ss = &ctx->streamScratch[0];
        for (auto& e : ctx->streamScratch)
            if (e.tick < ss->tick) ss = &e;
        GPUGI_CUDA_TRY(ctx, cudaEventSynchronize(ss->lastUse));
        ss->stream = s;
    }
    if (n > ss->cap) {
        if (ss->queue) {
            GPUGI_CUDA_TRY(ctx, cudaEventSynchronize(ss->lastUse));
            cudaFree(ss->queue);
            ss->queue = nullptr;
            ss->cap = 0;
        }
        const uint64_t want = n + n / 4;
        if (cudaMalloc(&ss->queue, want * sizeof(uint32_t)) != cudaSuccess) {
            ss->queue = nullptr;
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "ray queue allocation failed");
        }
        ss->cap = want;
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamWaitEvent(s, ss->lastUse, 0));
    ss->tick = ++ctx->streamTick;
    *out = ss;
    return GPUGI_OK;
}

static gpugi_status trace_async(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                const float* oy, const float* oz, const float* dx, const float* dy, const float* dz,
                                const float* tmax, uint64_t n, int32_t* slot, float* t, float* u, float* v,
                                uint8_t* occluded, void* stream) {
    if (n == 0) return GPUGI_OK;
    if (n > 0xFFFFFFFFull) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "at most 2^32-1 rays per call");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    gpugi_ctx::StreamScratch* ss = nullptr;
    gpugi_status st = stream_scratch(ctx, s, n, &ss);
    if (st) return st;
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(ss->counters, 0, 4 * sizeof(unsigned long long), s));
    st = launch_trace_filtered_on(ctx, sc, anyHit, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, occluded,
                                  ss->queue, ss->counters, s, ctx->asyncWalkerShare);
    if (st) return st;
    GPUGI_CUDA_TRY(ctx, cudaEventRecord(ss->lastUse, s));
    return GPUGI_OK;
}

// Host-pointer query on a caller stream: rays copied in, the two launches,
// results copied out, all enqueued on `stream` with no wait. The stream's
// staging columns grow with n (after the stream's earlier work has finished).
static gpugi_status trace_host_async(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* const src[7],
                                     uint64_t n, int32_t* slot, float* t, float* u, float* v, uint8_t* occ,
                                     void* stream) {
    if (n == 0) return GPUGI_OK;
    if (n > 0xFFFFFFFFull) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "at most 2^32-1 rays per call");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    gpugi_ctx::StreamScratch* ss = nullptr;
    gpugi_status st = stream_scratch(ctx, s, n, &ss);
    if (st) return st;
    const size_t col = align256(n * 4);
    if (ss->stageBytes < 11 * col) {
        if (ss->stage) {
            GPUGI_CUDA_TRY(ctx, cudaEventSynchronize(ss->lastUse));
            cudaFree(ss->stage);
            ss->stage = nullptr;
            ss->stageBytes = 0;
        }
        if (cudaMalloc(&ss->stage, 11 * col) != cudaSuccess) {
            ss->stage = nullptr;
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "query staging allocation failed");
        }
        ss->stageBytes = 11 * col;
    }
    char* base = static_cast<char*>(ss->stage);
    float* d[7];
    for (int k = 0; k < 7; ++k) d[k] = reinterpret_cast<float*>(base + k * col);
    if ((st = copy_rays_in(ctx, d, 0, src, 0, n, s))) return st;
    char* const dRes[4] = {base + 7 * col, base + 8 * col, base + 9 * col, base + 10 * col};
    int32_t* dSlot = reinterpret_cast<int32_t*>(base + 7 * col);
    float* dT = reinterpret_cast<float*>(base + 8 * col);
    float* dU = reinterpret_cast<float*>(base + 9 * col);
    float* dV = reinterpret_cast<float*>(base + 10 * col);
    uint8_t* dOcc = reinterpret_cast<uint8_t*>(base + 7 * col);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(ss->counters, 0, 4 * sizeof(unsigned long long), s));
    st = launch_trace_filtered_on(ctx, sc, anyHit, d[0], d[1], d[2], d[3], d[4], d[5], d[6], n,
                                  anyHit ? nullptr : dSlot, anyHit ? nullptr : dT, anyHit ? nullptr : dU,
                                  anyHit ? nullptr : dV, anyHit ? dOcc : nullptr, ss->queue, ss->counters, s);
    // (the full walker grid: host-array queries are paced by their copies,
    // and a shorter walk keeps each stream's copy-trace-copy cycle short)
    if (st) return st;
    if ((st = copy_results_out(ctx, anyHit, dRes, 0, slot, t, u, v, occ, 0, n, s))) return st;
    GPUGI_CUDA_TRY(ctx, cudaEventRecord(ss->lastUse, s));
    return GPUGI_OK;
}

}  // namespace gpugi

extern "C" {

gpugi_status gpugi_trace_closest_async(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                       const float* oz, const float* dx, const float* dy, const float* dz,
                                       const float* tmax, uint64_t n, int32_t* slot, float* t, float* u, float* v,
                                       void* stream) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !slot || !t || !u || !v)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    const float* const src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    return trace_host_async(ctx, sc, false, src, n, slot, t, u, v, nullptr, stream);
}

gpugi_status gpugi_trace_any_async(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                   const float* oz, const float* dx, const float* dy, const float* dz,
                                   const float* tmax, uint64_t n, uint8_t* occluded, void* stream) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !occluded)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    const float* const src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    return trace_host_async(ctx, sc, true, src, n, nullptr, nullptr, nullptr, nullptr, occluded, stream);
}

gpugi_status gpugi_trace_closest_device_async(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox,
                                              const float* oy, const float* oz, const float* dx, const float* dy,
                                              const float* dz, const float* tmax, uint64_t n, int32_t* slot,
                                              float* t, float* u, float* v, void* stream) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !slot || !t || !u || !v)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    return trace_async(ctx, sc, false, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, nullptr, stream);
}

gpugi_status gpugi_trace_any_device_async(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                          const float* oz, const float* dx, const float* dy, const float* dz,
                                          const float* tmax, uint64_t n, uint8_t* occluded, void* stream) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !occluded)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    return trace_async(ctx, sc, true, ox, oy, oz, dx, dy, dz, tmax, n, nullptr, nullptr, nullptr, nullptr, occluded,
                       stream);
}

gpugi_status gpugi_trace_stats_device(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                      const float* oz, const float* dx, const float* dy, const float* dz,
                                      const float* tmax, uint64_t n, uint32_t anyHit, uint64_t sums[3]) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || !sums || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    gpugi_status st = ensure_stage(ctx, 256);
    if (st) return st;
    unsigned long long* d = static_cast<unsigned long long*>(ctx->stageDev);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(d, 0, 24, ctx->stream));
    if ((st = launch_trace_stats(ctx, sc, ox, oy, oz, dx, dy, dz, tmax, n, anyHit, d))) return st;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(sums, d, 24, cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

// Host-pointer variants: rays are copied into the context's staging buffer
// in chunks; each chunk's upload, walk and download are enqueued in order on
// the context stream.
gpugi_status gpugi_trace_closest(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                 const float* oz, const float* dx, const float* dy, const float* dz,
                                 const float* tmax, uint64_t n, int32_t* slot, float* t, float* u, float* v) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !slot || !t || !u || !v)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return GPUGI_OK;
    const float* const src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    gpugi_status st = trace_host(ctx, sc, false, src, n, slot, t, u, v, nullptr);
    if (st) return st;
    return check_copied_device_error(ctx);
}

gpugi_status gpugi_trace_any(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                             const float* oz, const float* dx, const float* dy, const float* dz, const float* tmax,
                             uint64_t n, uint8_t* occluded) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !occluded)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return GPUGI_OK;
    const float* const src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    gpugi_status st = trace_host(ctx, sc, true, src, n, nullptr, nullptr, nullptr, nullptr, occluded);
    if (st) return st;
    return check_copied_device_error(ctx);
}

}  // extern "C"
