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

/* Closest hit without any device allocation in the call. No counterpart in
 * the reference: it exists for callers that cannot let the library call
 * cudaMalloc, such as an engine that owns all device memory through its own
 * pool, or a frame loop where an allocation would synchronise the device.
 * Same arguments (device pointers) and results as gpugi_trace_closest_device.
 * Scratch memory is a static device array in the library, held by every GPU
 * that loads it until the process exits; it bounds n to
 * GPUGI_NOALLOC_MAX_RAYS (larger n returns GPUGI_ERROR_INVALID_ARGUMENT).
 * The first call on a device looks the array's address up
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the one array: calls that overlap on the GPU (other
 * streams, other contexts on the same device) race and must be serialised
 * by the caller. Asynchronous on the context stream. */
#define GPUGI_NOALLOC_MAX_RAYS (1u << 20)
gpugi_status gpugi_trace_closest_noalloc(gpugi_ctx* ctx, const gpugi_scene* scene,
                                         const float* ox, const float* oy, const float* oz,
                                         const float* dx, const float* dy, const float* dz,
                                         const float* tmax, uint64_t n,
                                         int32_t* slot, float* t, float* u, float* v);

/* Fetch statistics of the walk for n device rays: sums over all rays of
 * {nodes visited, leaf slots fetched, valid triangles tested}, the analogue
 * of TRACERAY_DEBUG_VARS (gpugi/shader/traceray.glsl:59-61,131-133). Used to
 * compute the algorithmic bytes of a launch. Synchronous. */
gpugi_status gpugi_trace_stats_device(gpugi_ctx* ctx, const gpugi_scene* scene,
                                      const float* ox, const float* oy, const float* oz,
                                      const float* dx, const float* dy, const float* dz,
                                      const float* tmax, uint64_t n, uint32_t anyHit, uint64_t sums[3]);

/* Traversal tuning (set by the autotuner). mode 0: one thread per ray, grid
 * of ceil(n / blockSize) blocks; mode 1: persistent warps that refill
 * finished lanes from a device ray counter; mode 2 (default): a coalesced
 * root-bounds prefilter that finishes rays missing the scene and queues the
 * rest (warp-ballot compaction) for the persistent walker. All modes perform
 * the same tests per ray and return identical results. */
gpugi_status gpugi_set_trace_config(gpugi_ctx* ctx, uint32_t mode, uint32_t blockSize);

/* ------------------------------------------------------------------------
 * Rendering passes (wavefront): PT, LT and BPT.
 *
 *   gpugi_render(pass = PT)   Pathtracer::Draw + pathtracer.comp
 *                             (gpugi/renderer/pathtracer.cpp:47-53, gpugi/shader/pathtracer.comp)
 *   gpugi_render(pass = LT)   LightPathtracer::Draw + lighttracer.comp + showlightcaches.comp
 *                             (gpugi/renderer/lightpathtracer.cpp:45-49)
 *   gpugi_render(pass = BPT)  BidirectionalPathtracer::Draw: reset counter, light
 *                             trace into the light cache, eye pass
 *                             (gpugi/renderer/bidirectionalpathtracer.cpp:182-203)
 * ------------------------------------------------------------------------ */
typedef struct gpugi_image gpugi_image;

enum gpugi_pass { GPUGI_PASS_PT = 0, GPUGI_PASS_LT = 1, GPUGI_PASS_BPT = 2 };

/* Camera UBO (gpugi/shader/globaluniforms.glsl:7-15): U, V scaled by
 * tan(fov/2)*aspect and tan(fov/2), W unit view direction. */
typedef struct gpugi_camera {
    float U[3], V[3], W[3], position[3];
    float pixelArea;
} gpugi_camera;

typedef struct gpugi_render_params {
    uint32_t pass;             /* gpugi_pass */
    uint32_t width, height;    /* must match the image */
    uint32_t maxPathLength;    /* MAX_PATHLENGTH */
    uint32_t rrStartDepth;     /* Russian roulette from this bounce on; 0 = the reference */
    uint32_t iteration;        /* first iteration: FrameSeed(s) = WangHash(iteration + s) */
    uint32_t samples;          /* iterations (samples per pixel) rendered by this call */
    uint32_t numLightSamples;  /* initial light samples per iteration (PT/BPT 128, LT 256) */
    float sky[3];              /* constant radiance on a miss (addition; 0 = the reference's black) */
    uint32_t flags;            /* reserved, 0 */
} gpugi_render_params;

/* Camera::ComputeCameraParams (gpugi/camera/camera.cpp:76-85) and the pixel
 * area of RendererSystem::SetCamera (gpugi/renderer/renderersystem.cpp:208). */
gpugi_status gpugi_camera_lookat(const float position[3], const float lookat[3], const float up[3],
                                 float yFovDegrees, uint32_t width, uint32_t height, gpugi_camera* out);

/* Accumulation image: RGBA32F (the backbuffer) plus, with flags & 1, an FP64
 * RGB accumulation used only for converged oracle images and error sums. */
gpugi_status gpugi_image_create(gpugi_ctx* ctx, uint32_t width, uint32_t height, uint32_t flags,
                                gpugi_image** out);
void gpugi_image_destroy(gpugi_image* image);
gpugi_status gpugi_image_clear(gpugi_ctx* ctx, gpugi_image* image);
/* Copy the accumulation to host memory (either pointer may be NULL). */
gpugi_status gpugi_image_read(gpugi_ctx* ctx, const gpugi_image* image, float* rgba, double* rgb64);
/* TextureMSE (gpugi/imageut/texturemse.cpp:39-65, utils/sqerror.frag):
 * mean over pixels of |rgb / divisor - reference|^2 (the RGB sum, not the
 * channel mean), reduced in FP64 on the device. reference: host, 3 floats per
 * pixel. useFp64 selects the FP64 accumulation as the source. */
gpugi_status gpugi_image_mse(gpugi_ctx* ctx, const gpugi_image* image, double divisor, const float* reference,
                             uint32_t useFp64, double* mse);

/* Light sources of a scene (Scene::LoadLightSources, gpugi/scene/scene.cpp:244-293,
 * and point lights, :295-307) and the host light sampler
 * (LightSampler::GenerateRandomSamples, gpugi/scene/lightsampler.cpp:18-95).
 * Emissive triangles are found from the materials at upload. A directional
 * light (direction towards the light, irradiance) is an addition; its
 * samples carry normalThetaCos = 3. Samples: 8 floats each
 * {position.xyz, normalPhi, intensity.xyz, normalThetaCos}. */
gpugi_status gpugi_scene_add_point_light(gpugi_scene* scene, const float position[3], const float intensity[3]);
gpugi_status gpugi_scene_add_directional_light(gpugi_scene* scene, const float towardsLight[3],
                                               const float irradiance[3]);
gpugi_status gpugi_generate_light_samples(const gpugi_scene* scene, uint64_t* rngState, uint32_t numSamples,
                                          float* out);

/* Render `samples` iterations of one pass into the image. lightSamples:
 * host, samples * numLightSamples * 8 floats (one light-sample set per
 * iteration, as RendererSystem::PerIterationBufferUpdate regenerates them);
 * NULL generates them on the host with rngState (required then). Asynchronous
 * on the context stream. */
gpugi_status gpugi_render(gpugi_ctx* ctx, const gpugi_scene* scene, const gpugi_camera* camera,
                          const gpugi_render_params* params, const float* lightSamples, uint64_t* rngState,
                          gpugi_image* image);

/* Rays traced by the last gpugi_render call, by kind: {camera/extension
 * (closest hit), shadow/connection (any hit)}. Synchronises. */
gpugi_status gpugi_render_ray_counts(gpugi_ctx* ctx, uint64_t counts[2]);

#ifdef __cplusplus
}
#endif
#endif
