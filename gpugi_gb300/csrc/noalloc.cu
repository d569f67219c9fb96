// Closest-hit queries without any device allocation in the call.
//
// gpugi_trace_closest_device draws its scratch memory (the ray-index queue
// of the root prefilter and four work counters) from buffers the context
// grows with cudaMalloc on demand. Some callers cannot allow that: a renderer
// or engine that owns all device memory through its own pool, or a frame
// loop where a cudaMalloc would synchronise the device and stall the frame.
// gpugi_trace_closest_noalloc serves them: its scratch lives in the file-scope
// device arrays below, which every GPU that loads this library holds until
// the process exits (4 MiB + 32 B per device).
#include <mutex>

#include "ctx.cuh"

namespace gpugi {

constexpr uint64_t kNoAllocMaxRays = 1ull << 20;  // GPUGI_NOALLOC_MAX_RAYS

static __device__ __align__(256) uint32_t g_noallocQueue[kNoAllocMaxRays];
static __device__ __align__(256) unsigned long long g_noallocCounters[4];

// Host-side device addresses of the arrays above, resolved once per device.
// The array names are only host stand-ins in host code; a kernel must be
// given the address from cudaGetSymbolAddress.
struct NoAllocScratch {
    uint32_t* queue = nullptr;
    unsigned long long* counters = nullptr;
    bool ready = false;
};
constexpr int kMaxDevices = 64;
static NoAllocScratch g_scratch[kMaxDevices];
static std::mutex g_scratchMutex;

static gpugi_status resolve_scratch(gpugi_ctx* ctx, NoAllocScratch& out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return fail(ctx, GPUGI_ERROR_UNSUPPORTED, "device ordinal beyond the no-allocation table");
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    NoAllocScratch& s = g_scratch[ctx->device];
    if (!s.ready) {
        int prev = 0;
        cudaError_t e = cudaGetDevice(&prev);
        if (e == cudaSuccess) e = cudaSetDevice(ctx->device);
        void* q = nullptr;
        void* c = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_noallocQueue);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&c, g_noallocCounters);
        cudaSetDevice(prev);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress (no-allocation scratch)");
        s.queue = static_cast<uint32_t*>(q);
        s.counters = static_cast<unsigned long long*>(c);
        s.ready = true;
    }
    out = s;
    return GPUGI_OK;
}

}  // namespace gpugi

using namespace gpugi;

extern "C" gpugi_status gpugi_trace_closest_noalloc(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox,
                                                   const float* oy, const float* oz, const float* dx,
                                                   const float* dy, const float* dz, const float* tmax, uint64_t n,
                                                   int32_t* slot, float* t, float* u, float* v) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || (n && (!ox || !oy || !oz || !dx || !dy || !dz || !tmax || !slot || !t || !u || !v)))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (n > kNoAllocMaxRays)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT,
                    "gpugi_trace_closest_noalloc takes at most GPUGI_NOALLOC_MAX_RAYS (2^20) rays per call; "
                    "split the batch or use gpugi_trace_closest_device");
    if (n == 0) return GPUGI_OK;
    NoAllocScratch s;
    gpugi_status st = resolve_scratch(ctx, s);
    if (st) return st;
    // The counters keep the previous call's values: clear them on the stream.
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(s.counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    return launch_trace_filtered_on(ctx, sc, false, ox, oy, oz, dx, dy, dz, tmax, n, slot, t, u, v, nullptr, s.queue,
                                    s.counters);
}
