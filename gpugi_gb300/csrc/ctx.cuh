// Host-side objects behind the opaque handles of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gpugi_cuda.h"
#include "scene.cuh"

struct gpugi_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t* errWord = nullptr;  // device error word (GPUGI_DEVERR_*)
    std::string lastError;
    // staging for the host-pointer entry points (grown on demand)
    void* stageDev = nullptr;
    size_t stageDevBytes = 0;
    // trace tuning
    uint32_t traceMode = 1;  // 0 = one thread per ray, 1 = persistent lane refill
    uint32_t traceBlock = 128;
    void* scratch = nullptr;  // 256 B of device counters (work distribution)
    int numSMs = 0;
};

struct gpugi_scene {
    gpugi_ctx* ctx = nullptr;
    gpugi::DevScene dev;
    // owned device allocations
    std::vector<void*> allocations;
    // host copies needed by the renderers (light extraction etc.)
    std::vector<float> hostPositions;
    std::vector<int32_t> hostSlots;
    std::vector<float> hostMaterials;
    uint32_t numLeafBlocks = 0;
};

namespace gpugi {

// Set ctx->lastError and return the status.
gpugi_status fail(gpugi_ctx* ctx, gpugi_status st, const std::string& msg);
// Map a CUDA error to GPUGI_ERROR_CUDA with context.
gpugi_status cuda_fail(gpugi_ctx* ctx, cudaError_t e, const char* what);
// Grow the context's device staging buffer to at least `bytes`.
gpugi_status ensure_stage(gpugi_ctx* ctx, size_t bytes);
// Launch the traversal kernels (device pointers, async on ctx->stream).
gpugi_status launch_trace_closest(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                  const float* oz, const float* dx, const float* dy, const float* dz,
                                  const float* tmax, uint64_t n, int32_t* slot, float* t, float* u, float* v);
gpugi_status launch_trace_any(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                              const float* oz, const float* dx, const float* dy, const float* dz,
                              const float* tmax, uint64_t n, uint8_t* occluded);

gpugi_status launch_trace_persistent(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                     const float* oy, const float* oz, const float* dx, const float* dy,
                                     const float* dz, const float* tmax, uint64_t n, int32_t* slot, float* t,
                                     float* u, float* v, uint8_t* occluded);
gpugi_status launch_trace_stats(gpugi_ctx* ctx, const gpugi_scene* sc, const float* ox, const float* oy,
                                const float* oz, const float* dx, const float* dy, const float* dz,
                                const float* tmax, uint64_t n, uint32_t anyHit, unsigned long long* sums);

}  // namespace gpugi

#define GPUGI_CUDA_TRY(ctx, call)                                    \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return gpugi::cuda_fail(ctx, e_, #call); \
    } while (0)
