// Host-side objects behind the opaque handles of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gpugi_cuda.h"
#include "scene.cuh"

struct gpugi_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t* errWord = nullptr;  // device error word (GPUGI_DEVERR_*)
    uint32_t* errHost = nullptr;  // page-locked copy of it, read back with a call's last copies
    // occupancy of the walker kernels (kernel, dynamic shared bytes) -> blocks per SM
    std::vector<std::pair<std::pair<const void*, size_t>, int>> occupancy;
    std::string lastError;
    // staging for the host-pointer entry points (grown on demand)
    void* stageDev = nullptr;
    size_t stageDevBytes = 0;
    // trace tuning
    uint32_t traceMode = 3;  // 0 thread per ray, 1 persistent lane refill, 2 root prefilter + 1, 3/4 + 8/4-lane groups
    uint32_t traceBlock = 128;
    // photon mapper (PhotonMapper's pm_nphotons, pm_r, pm_progressive; photonmapper.cpp:17-45)
    uint32_t pmPhotonsPerSample = 1u << 11;
    float pmQueryRadius = 0.01f;
    uint32_t pmProgressive = 0;
    // importon map light tracer (PixelMapLighttracer's im_nphotons, im_r, im_progressive;
    // pixelmaplighttracer.cpp:19-41)
    uint32_t imPhotonsPerSample = 1u << 11;
    float imQueryRadius = 0.005f;
    uint32_t imProgressive = 0;
    uint32_t sharedNodes = 0;        // top-of-tree nodes laid out first and staged by ray-query walkers
    uint32_t renderSharedNodes = 0;  // nodes staged by the renderer's walkers
    void* scratch = nullptr;  // 256 B of device counters (work distribution)
    uint32_t* queue = nullptr;  // ray-index queue of the root prefilter (mode 2)
    uint64_t queueCap = 0;
    int numSMs = 0;
    // host-pointer ray queries: copies in, traversal and copies out of
    // hostParts parts of a call overlap on three streams (trace modes 2-5)
    uint32_t hostParts = 2;
    // percent of the persistent walker grid a stream-ordered query on device
    // arrays launches:
    // queries on several streams then run two or more walks side by side,
    // each one's tail overlapping the others' bulk (gpugi_set_async_walker_share)
    uint32_t asyncWalkerShare = 50;
    uint32_t hostZeroCopy = 0;  // 1: page-locked host arrays are read and written by the kernels directly
    cudaStream_t copyIn = nullptr, copyOut = nullptr;
    cudaStream_t compute2 = nullptr;  // second traversal stream of the host-pointer pipeline
    cudaEvent_t evIn[8] = {}, evTraced[8] = {};
    // scratch of the stream-ordered queries (gpugi_trace_*_device_async), one
    // set per caller stream: ray-index queue + four counters
    struct StreamScratch {
        cudaStream_t stream = nullptr;
        uint32_t* queue = nullptr;
        uint64_t cap = 0;
        unsigned long long* counters = nullptr;
        void* stage = nullptr;  // host-pointer queries: device copies of the rays and results
        size_t stageBytes = 0;
        cudaEvent_t lastUse = nullptr;  // recorded after the last work that used this set
        uint64_t tick = 0;              // call counter at the last use (least recently used is reused)
    };
    uint64_t streamTick = 0;
    std::vector<StreamScratch> streamScratch;
    // batched rendering
    uint32_t batchPaths = 16u << 20;  // path-queue capacity of one round
    uint32_t batchGraph = 1;          // replay rounds as a CUDA graph
    // wavefront renderer buffers (owned by render.cu)
    void* render = nullptr;
    void (*renderFree)(gpugi_ctx*) = nullptr;
    // back references (the `ctx` fields) of live scenes, images and caches:
    // gpugi_destroy clears them, so objects released after their context
    // only free their own device memory
    std::vector<gpugi_ctx**> children;
};

namespace gpugi {
struct LightTriangle {
    float v[3][3];
    float lum[3];
};
struct PointLight {
    float position[3], intensity[3];
};
struct DirLight {
    float dir[3], irradiance[3];  // dir points towards the light
};
struct HierBuffers;  // hierarchy.cu
}  // namespace gpugi

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
    uint32_t numNodesUploaded = 0;  // dev.numNodes before gpugi_debug_limit_nodes
    // light tables (Scene::LoadLightSources / ComputePointLightTable)
    bool lightsReady = false;
    std::vector<gpugi::LightTriangle> lightTris;
    std::vector<float> lightSummedArea;
    float lightAreaSum = 0.0f, totalAreaLightFlux = 0.0f, totalPointLightFlux = 0.0f;
    std::vector<gpugi::PointLight> pointLights;
    std::vector<float> pointLightSummedFlux;
    std::vector<gpugi::DirLight> dirLights;
    // Node order on the device: uploaded (preorder) index -> device index;
    // empty when the two are the same.
    std::vector<uint32_t> nodeMap;
    // Ellipsoid scenes: the radii as uploaded (3 floats per node, device
    // order); the device nodes hold their reciprocals.
    std::vector<float> hostRadii;
    // material textures (texels, per-texture table, per-material map indices), one allocation
    void* texBlock = nullptr;
    // hierarchy-importance renderer (hierarchy.cu), device node order
    gpugi::HierBuffers* hier = nullptr;
};

// Accumulation image (RGBA32F sum, optional FP64 RGB sum).
struct gpugi_image {
    gpugi_ctx* ctx = nullptr;
    uint32_t width = 0, height = 0, flags = 0;
    float4* rgba = nullptr;
    double* rgb64 = nullptr;
};

namespace gpugi {

inline void attach_child(gpugi_ctx* ctx, gpugi_ctx** ref) {
    *ref = ctx;
    ctx->children.push_back(ref);
}
inline void detach_child(gpugi_ctx** ref) {
    gpugi_ctx* ctx = *ref;
    if (!ctx) return;
    for (size_t i = 0; i < ctx->children.size(); ++i)
        if (ctx->children[i] == ref) {
            ctx->children[i] = ctx->children.back();
            ctx->children.pop_back();
            break;
        }
    *ref = nullptr;
}

// Set ctx->lastError and return the status.
gpugi_status fail(gpugi_ctx* ctx, gpugi_status st, const std::string& msg);
// Map a CUDA error to GPUGI_ERROR_CUDA with context.
gpugi_status cuda_fail(gpugi_ctx* ctx, cudaError_t e, const char* what);
// Grow the context's device staging buffer to at least `bytes`.
gpugi_status ensure_stage(gpugi_ctx* ctx, size_t bytes);
// Grow the context's ray-index queue to at least n entries.
gpugi_status ensure_queue(gpugi_ctx* ctx, uint64_t n);
constexpr size_t kMaxQueryStreams = 8;  // GPUGI_MAX_QUERY_STREAMS
gpugi_status launch_trace_filtered(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                   const float* oy, const float* oz, const float* dx, const float* dy,
                                   const float* dz, const float* tmax, uint64_t n, int32_t* slot, float* t,
                                   float* u, float* v, uint8_t* occluded);
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
gpugi_status launch_trace_filtered_on(gpugi_ctx* ctx, const gpugi_scene* sc, bool anyHit, const float* ox,
                                      const float* oy, const float* oz, const float* dx, const float* dy,
                                      const float* dz, const float* tmax, uint64_t n, int32_t* slot, float* t,
                                      float* u, float* v, uint8_t* occluded, uint32_t* queue,
                                      unsigned long long* counters, cudaStream_t stream = nullptr,
                                      uint32_t walkerShare = 100);
// Launch shape of a persistent walker: grid, dynamic shared memory and the
// number of top-of-tree nodes it stages (at most maxStage).
struct WalkerLaunch {
    unsigned grid = 1;
    size_t smem = 0;
    uint32_t stage = 0;
};
gpugi_status walker_launch_config(gpugi_ctx* ctx, const gpugi_scene* sc, const void* kernel, uint64_t n,
                                  uint32_t maxStage, WalkerLaunch& out);
// Radiance cache with element counts in device memory (nrc.cu): inference
// of min(n, *count) queries, one Adam step on min(cap, *count) samples.
gpugi_status nrc_infer_counted(gpugi_ctx* ctx, const gpugi_nrc* nn, const float* queries, uint64_t n,
                               const uint32_t* count, float* out);
gpugi_status nrc_train_counted(gpugi_ctx* ctx, gpugi_nrc* nn, const float* samples, uint64_t cap,
                               const uint32_t* count);
// Per-slot triangle records {p0, e0, e1, n} of a device slot array (scene.cu).
void prepare_triangles(cudaStream_t stream, const int4* slots, uint32_t numSlots, const float* positions,
                       float4* tris);
// Light tables and the host light sampler (host.cu).
void build_light_tables(gpugi_scene* sc);
void generate_light_samples(gpugi_scene* sc, uint64_t& rng, uint32_t numSamples, float* out);
// Hierarchy-importance renderer (hierarchy.cu): the GPUGI_PASS_HIERARCHY
// branch of gpugi_render, and the release of a scene's buffers.
gpugi_status render_hierarchy(gpugi_ctx* ctx, gpugi_scene* sc, const gpugi_camera* cam,
                              const gpugi_render_params* p, const float* lightSamples, uint64_t* rngState,
                              gpugi_image* im);
void free_hierarchy(gpugi_scene* sc);

}  // namespace gpugi

#define GPUGI_CUDA_TRY(ctx, call)                                    \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return gpugi::cuda_fail(ctx, e_, #call); \
    } while (0)
