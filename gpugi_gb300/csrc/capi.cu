// Context lifetime, error reporting and the ray-query entry points of the C ABI.
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

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace gpugi

using namespace gpugi;

extern "C" {

const char* gpugi_version(void) { return "gpugi_gb300 0.1 (sm_103a)"; }

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
        (e = cudaMalloc(&ctx->scratch, 256)) != cudaSuccess || (e = cudaMemset(ctx->scratch, 0, 256)) != cudaSuccess) {
        if (ctx->errWord) cudaFree(ctx->errWord);
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
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->queue) cudaFree(ctx->queue);
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
    const float* src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        for (int k = 0; k < 7; ++k)
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(d[k], src[k] + off, m * 4, cudaMemcpyHostToDevice, ctx->stream));
        if ((st = launch_trace_closest(ctx, sc, d[0], d[1], d[2], d[3], d[4], d[5], d[6], m, dSlot, dT, dU, dV)))
            return st;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(slot + off, dSlot, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(t + off, dT, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(u + off, dU, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(v + off, dV, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

gpugi_status gpugi_trace_any(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                             const float* oz, const float* dx, const float* dy, const float* dz, const float* tmax,
                             uint64_t n, uint8_t* occluded) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !occluded)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return GPUGI_OK;
    const uint64_t chunk = n < (1ull << 22) ? n : (1ull << 22);
    const size_t col = align256(chunk * 4);
    gpugi_status st = ensure_stage(ctx, 8 * col);
    if (st) return st;
    char* base = static_cast<char*>(ctx->stageDev);
    float* d[7];
    for (int k = 0; k < 7; ++k) d[k] = reinterpret_cast<float*>(base + k * col);
    uint8_t* dOcc = reinterpret_cast<uint8_t*>(base + 7 * col);
    const float* src[7] = {ox, oy, oz, dx, dy, dz, tmax};
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        for (int k = 0; k < 7; ++k)
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(d[k], src[k] + off, m * 4, cudaMemcpyHostToDevice, ctx->stream));
        if ((st = launch_trace_any(ctx, sc, d[0], d[1], d[2], d[3], d[4], d[5], d[6], m, dOcc))) return st;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(occluded + off, dOcc, m, cudaMemcpyDeviceToHost, ctx->stream));
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

}  // extern "C"
