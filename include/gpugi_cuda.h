/* gpugi_cuda.h — C ABI of the GB300 (sm_103a) hot path of gpugi.
 *
 * This is the drop-in boundary: plain pointers and sizes, opaque handles,
 * status codes. It replaces the GL objects and dispatches through which
 * gpugi's renderers reach its compute shaders:
 *
 *   gpugi_create / gpugi_destroy     RendererSystem::RendererSystem (gpugi/renderer/renderersystem.cpp:23-48)
 *   gpugi_scene_upload               Scene::UploadGeometry / UploadHierarchy + RendererSystem::SetScene
 *                                    (gpugi/scene/scene.cpp:75-130, gpugi/renderer/renderersystem.cpp:132-171)
 *   gpugi_trace_closest[_device]     TraceRay            (gpugi/shader/traceray.glsl:25-180)
 *   gpugi_trace_any[_device]         TraceRayAnyHit      (gpugi/shader/traceray.glsl:18-23, stdheader.glsl:26-28)
 *
 * Conventions
 *  - Every call returns gpugi_status; 0 is success. gpugi_last_error(ctx)
 *    gives a message for the last failure on that context.
 *  - The caller owns every host array passed in; the library owns all device
 *    memory behind a handle. Handles are opaque.
 *  - Calls on one context are not thread safe (gpugi's renderers are driven
 *    from the single thread that owns the GL context, the same rule applies).
 *  - `*_device` entry points take device pointers and enqueue asynchronously
 *    on the context's stream; the others take host pointers, copy through the
 *    context's staging buffers and return when the results are in host memory.
 *  - Device-side guards (iteration caps, queue capacity) never trap: they set
 *    bits of an error word that the next synchronising call turns into
 *    GPUGI_ERROR_DEVICE.
 */
#ifndef GPUGI_CUDA_H
#define GPUGI_CUDA_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gpugi_status {
    GPUGI_OK = 0,
    GPUGI_ERROR_INVALID_ARGUMENT = 1,
    GPUGI_ERROR_INVALID_SCENE = 2,   /* malformed hierarchy / leaf blocks / indices */
    GPUGI_ERROR_OUT_OF_MEMORY = 3,
    GPUGI_ERROR_CUDA = 4,            /* a CUDA runtime call failed */
    GPUGI_ERROR_DEVICE = 5,          /* a device-side guard fired, see gpugi_device_error_bits */
    GPUGI_ERROR_UNSUPPORTED = 6
} gpugi_status;

/* Bits of the device error word. */
#define GPUGI_DEVERR_TRAVERSAL_CAP 0x1u   /* a walk exceeded numNodes visits */
#define GPUGI_DEVERR_QUEUE_OVERFLOW 0x2u  /* a wavefront queue or light cache overflowed */
#define GPUGI_DEVERR_WAIT_TIMEOUT 0x4u    /* a bounded device wait ran out */

enum gpugi_bounds_kind { GPUGI_BOUNDS_AABB = 0, GPUGI_BOUNDS_ELLIPSOID = 1 };

typedef struct gpugi_ctx gpugi_ctx;
typedef struct gpugi_scene gpugi_scene;

typedef struct gpugi_opts {
    int device;        /* CUDA device ordinal */
    uint32_t flags;    /* reserved, 0 */
} gpugi_opts;

/* Material record, 6 x float4 = 96 bytes. The constant-valued form of
 * gpugi's Material + MaterialData (gpugi/scene/scene.hpp:79-89,
 * gpugi/shader/materials.glsl:9-30): the four bindless textures are replaced
 * by their values. */
typedef struct gpugi_material {
    float diffuse[3];         float refractionIndexAvg;
    float opacity[3];         float pad0;
    float reflectiveness[4];  /* xyz = reflectiveness, w = Phong exponent */
    float emissivity[3];      float pad1;
    float fresnel0[3];        float pad2;
    float fresnel1[3];        float pad3;
} gpugi_material;

gpugi_status gpugi_create(gpugi_ctx** ctx, const gpugi_opts* opts);
void gpugi_destroy(gpugi_ctx* ctx);
const char* gpugi_last_error(const gpugi_ctx* ctx);
/* Wait for all work on the context's stream; reports device guard bits. */
gpugi_status gpugi_sync(gpugi_ctx* ctx);
/* Read and clear the device error word (synchronises). */
gpugi_status gpugi_device_error_bits(gpugi_ctx* ctx, uint32_t* bits);
/* The cudaStream_t the context enqueues on (returned as void*). */
void* gpugi_stream(gpugi_ctx* ctx);
/* Library version string. */
const char* gpugi_version(void);

/* Upload a scene in the layout of gpugi's GPU buffers.
 *   hierarchy   8 floats per node: {min.xyz, firstChild bits, max.xyz, escape bits}
 *               (Scene::TreeNode<Box>, gpugi/scene/scene.hpp:30-38); for
 *               GPUGI_BOUNDS_ELLIPSOID {center.xyz, firstChild, radii.xyz, escape}
 *   slots       4 int32 per leaf slot {v0, v1, v2, material}; leafSize slots
 *               per block; {0,0,0,0} (v0 == v1) ends a block early
 *   positions   3 floats per vertex (RGB32F, gpugi/scene/scene.cpp:87)
 *   vertexInfo  4 floats per vertex {atan2(n.y,n.x), n.z, u, v} or NULL
 *               (gpugi/scene/scene.cpp:79-84)
 *   materials   numMaterials records (may be NULL when numMaterials == 0)
 * The hierarchy is validated (preorder escape tree, indices in range) and
 * rejected with GPUGI_ERROR_INVALID_SCENE otherwise. leafSize <= 32. */
gpugi_status gpugi_scene_upload(gpugi_ctx* ctx, const float* hierarchy, uint32_t numNodes,
                                uint32_t boundsKind, const int32_t* slots, uint32_t numSlots,
                                uint32_t leafSize, const float* positions, const float* vertexInfo,
                                uint32_t numVertices, const gpugi_material* materials,
                                uint32_t numMaterials, gpugi_scene** out);
void gpugi_scene_destroy(gpugi_scene* scene);

/* Closest hit for n rays in SoA layout. tmax is the initial rayLength
 * (gpugi uses RAY_MAX = 3.402823466e38, stdheader.glsl:6). Outputs per ray:
 * slot = leaf slot index of the hit triangle or -1, t = final rayLength,
 * u = barycentric y, v = barycentric z (x = 1 - (v + u)). */
gpugi_status gpugi_trace_closest(gpugi_ctx* ctx, const gpugi_scene* scene,
                                 const float* ox, const float* oy, const float* oz,
                                 const float* dx, const float* dy, const float* dz,
                                 const float* tmax, uint64_t n,
                                 int32_t* slot, float* t, float* u, float* v);
gpugi_status gpugi_trace_closest_device(gpugi_ctx* ctx, const gpugi_scene* scene,
                                        const float* ox, const float* oy, const float* oz,
                                        const float* dx, const float* dy, const float* dz,
                                        const float* tmax, uint64_t n,
                                        int32_t* slot, float* t, float* u, float* v);
/* Any hit: occluded[i] = 1 if some triangle has hit > 1e-4 and hit < tmax[i]. */
gpugi_status gpugi_trace_any(gpugi_ctx* ctx, const gpugi_scene* scene,
                             const float* ox, const float* oy, const float* oz,
                             const float* dx, const float* dy, const float* dz,
                             const float* tmax, uint64_t n, uint8_t* occluded);
gpugi_status gpugi_trace_any_device(gpugi_ctx* ctx, const gpugi_scene* scene,
                                    const float* ox, const float* oy, const float* oz,
                                    const float* dx, const float* dy, const float* dz,
                                    const float* tmax, uint64_t n, uint8_t* occluded);

/* Fetch statistics of the walk for n device rays: sums over all rays of
 * {nodes visited, leaf slots fetched, valid triangles tested}, the analogue
 * of TRACERAY_DEBUG_VARS (gpugi/shader/traceray.glsl:59-61,131-133). Used to
 * compute the algorithmic bytes of a launch. Synchronous. */
gpugi_status gpugi_trace_stats_device(gpugi_ctx* ctx, const gpugi_scene* scene,
                                      const float* ox, const float* oy, const float* oz,
                                      const float* dx, const float* dy, const float* dz,
                                      const float* tmax, uint64_t n, uint32_t anyHit, uint64_t sums[3]);

/* Traversal tuning (set by the autotuner). mode 0: one thread per ray, grid
 * of ceil(n / blockSize) blocks; mode 1 (default): persistent warps that
 * refill finished lanes from a device ray counter. Both perform the same
 * tests per ray and return identical results. */
gpugi_status gpugi_set_trace_config(gpugi_ctx* ctx, uint32_t mode, uint32_t blockSize);

#ifdef __cplusplus
}
#endif
#endif
