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
 *    Host ray columns (ox, oy, oz, dx, dy, dz, tmax) at one common spacing,
 *    as in one structure-of-arrays block, travel as a single 2D copy; so do
 *    the result columns (slot, t, u, v). Each separate copy over the host
 *    link adds a fixed cost of a few microseconds.
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
#define GPUGI_DEVERR_BUILD 0x8u           /* the GPU hierarchy build found an inconsistent tree */
#define GPUGI_DEVERR_HIERARCHY 0x10u      /* a hierarchy-importance walk to the root exceeded the node count */
#define GPUGI_DEVERR_BOUNDS 0x20u         /* checked library only: an index outside its array (fetch skipped) */

enum gpugi_bounds_kind { GPUGI_BOUNDS_AABB = 0, GPUGI_BOUNDS_ELLIPSOID = 1, GPUGI_BOUNDS_OBOX = 2 };

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
/* Test support: set bits in the device error word, as a device guard would,
 * so that the reporting of the next synchronising call can be tested. */
gpugi_status gpugi_debug_raise_device_error(gpugi_ctx* ctx, uint32_t bits);
/* The cudaStream_t the context enqueues on (returned as void*). */
void* gpugi_stream(gpugi_ctx* ctx);
/* Library version string ("... checked" for the bounds-checked library). */
const char* gpugi_version(void);

/* Upload a scene in the layout of gpugi's GPU buffers.
 *   hierarchy   8 floats per node: {min.xyz, firstChild bits, max.xyz, escape bits}
 *               (Scene::TreeNode<Box>, gpugi/scene/scene.hpp:30-38); for
 *               GPUGI_BOUNDS_ELLIPSOID {center.xyz, firstChild, radii.xyz, escape};
 *               for GPUGI_BOUNDS_OBOX 12 floats per node, Scene::TreeNode<OBox>
 *               (scene.hpp:40-49): {center.xyz, firstChild, sidesHalf.xyz,
 *               escape, rotationInv quaternion x, y, z, w}, walked as the
 *               reference's OBOX_BVH path (FetchIntersectOBoxNode,
 *               intersectiontests.glsl:114-128). The hierarchy-importance
 *               pass takes AABB hierarchies only.
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
/* Test support: the node count the device code checks indexes against is
 * lowered to numNodes (at most the scene's own; 0 restores it). The node
 * array itself is unchanged, so every fetch stays inside it; walks that
 * reach a node at or past the limit end, and the checked library
 * (libgpugi_cuda_checked.so) reports GPUGI_DEVERR_BOUNDS for them. */
gpugi_status gpugi_debug_limit_nodes(gpugi_scene* scene, uint32_t numNodes);

/* Build the hierarchy on the GPU and create the scene. Replaces a host
 * build with bvhmake (BVHBuilder::BuildBVH + FitBox + ExportBVH/
 * ExportTriangles, bvhmake/bvhbuilder.cpp:526-612,710-722) followed by
 * gpugi_scene_upload: same node and leaf-block layout (preorder escape tree,
 * root at 0, AABB nodes, leaves of at most leafSize triangles padded with
 * {0,0,0,0}), but a linear BVH: triangles sorted by the 63-bit Morton code
 * of their box centre, split where the codes' common prefix ends.
 *   triangles   4 uint32 per triangle {v0, v1, v2, material}; v0 != v1
 * Other arguments as gpugi_scene_upload. Synchronous. */
gpugi_status gpugi_scene_build(gpugi_ctx* ctx, const float* positions, uint32_t numVertices,
                               const uint32_t* triangles, uint32_t numTriangles, const float* vertexInfo,
                               const gpugi_material* materials, uint32_t numMaterials, uint32_t leafSize,
                               gpugi_scene** out);

/* The scene's hierarchy (8 floats per node, 12 for oriented boxes; leaf words {0x80000000 | block})
 * in device node order and its leaf slots (4 int32 each). Call with
 * hierarchy and slots NULL for the sizes. */
gpugi_status gpugi_scene_export(gpugi_ctx* ctx, const gpugi_scene* scene, uint32_t* numNodes, uint32_t* numSlots,
                                float* hierarchy, int32_t* slots);

/* Material textures: the bindless textures of gpugi's materials
 * (Material's four handles, gpugi/shader/scenedata.glsl:60-71, sampled by
 * SampleMaterialData, materials.glsl:19-30; created by Scene::LoadMaterial,
 * gpugi/scene/scene.cpp:132-187, for every map a material JSON names a file
 * for). textures: RGBA32F texels, row-major, row 0 at t in [0, 1/height)
 * (decoded by the caller: the image loader of the reference is not part of
 * this path). materialTextures: 4 int32 per material (the scene's
 * numMaterials) giving the texture of its {reflectiveness (w = Phong
 * exponent), opacity, diffuse, emissivity} map, -1 for the material
 * record's constant value. A pass samples them at the hit's texture
 * coordinate as the reference's sampler does (bilinear, REPEAT; level 0).
 * Emission for next-event estimation still comes from the records'
 * constants (as LoadLightSources takes it); the hierarchy-importance pass
 * uses the constants. A later call replaces the textures; numTextures 0
 * removes them. Synchronous. */
typedef struct gpugi_texture {
    uint32_t width, height;
    const float* rgba;  /* width * height * 4 floats */
} gpugi_texture;
gpugi_status gpugi_scene_set_textures(gpugi_ctx* ctx, gpugi_scene* scene, const gpugi_texture* textures,
                                      uint32_t numTextures, const int32_t* materialTextures);

/* Triangle test of the ray queries on a scene (gpugi_trace_closest / _any,
 * their _device forms, gpugi_trace_closest_noalloc and gpugi_trace_stats_device).
 *   GPUGI_TRIANGLE_REFERENCE   the reference's IntersectTriangle (OptiX-style
 *                              Moeller-Trumbore, gpugi/shader/intersectiontests.glsl:63-79;
 *                              the default): not watertight, a ray through a
 *                              shared edge or vertex can miss both triangles
 *   GPUGI_TRIANGLE_WATERTIGHT  an addition: the watertight test of Woop, Benthin
 *                              and Wald (JCGT 2013) with the reference's hit
 *                              rule (t > 1e-4, accepted when t < rayLength)
 *                              and barycentrics; the first switch builds its
 *                              48-B vertex records on the device (synchronous)
 * The walk, its order and the acceptance rule are the same in both. The
 * rendering passes always use the reference test. */
#define GPUGI_TRIANGLE_REFERENCE 0u
#define GPUGI_TRIANGLE_WATERTIGHT 1u
gpugi_status gpugi_scene_set_triangle_test(gpugi_ctx* ctx, gpugi_scene* scene, uint32_t test);

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

/* Stream-ordered ray queries: as gpugi_trace_closest_device /
 * gpugi_trace_any_device, but enqueued on the caller's stream (a
 * cudaStream_t passed as void*; NULL = the context stream) and ordered only
 * by it. Calls on different streams may run concurrently: a renderer with
 * several independent ray batches in flight issues them on two or more
 * streams, and the tail of one batch's walk (the few deepest rays, while
 * most SMs are idle) overlaps the next batch's walk. The caller orders each
 * call after the work that writes its rays (and before the work that reads
 * its results) on that stream, as for any CUDA library call that takes a
 * stream. The library keeps one scratch set (ray-index queue and counters)
 * per stream, allocated at the first call on a stream and grown when n grows
 * (which waits for the set's previous work). Up to GPUGI_MAX_QUERY_STREAMS
 * sets exist per context; a call on a further stream takes over the least
 * recently used set once that set's last work has finished (streams may be
 * created and destroyed freely; only as many as there are sets overlap). The context's trace mode selects the walker (modes 0 and 1 run
 * the mode-2 launches). No counterpart in the reference (its queries are
 * shader calls inside a dispatch). */
#define GPUGI_MAX_QUERY_STREAMS 8
gpugi_status gpugi_trace_closest_device_async(gpugi_ctx* ctx, const gpugi_scene* scene,
                                              const float* ox, const float* oy, const float* oz,
                                              const float* dx, const float* dy, const float* dz,
                                              const float* tmax, uint64_t n,
                                              int32_t* slot, float* t, float* u, float* v, void* stream);
gpugi_status gpugi_trace_any_device_async(gpugi_ctx* ctx, const gpugi_scene* scene,
                                          const float* ox, const float* oy, const float* oz,
                                          const float* dx, const float* dy, const float* dz,
                                          const float* tmax, uint64_t n, uint8_t* occluded, void* stream);

/* Stream-ordered queries over HOST arrays: the rays are copied in, traced
 * and the results copied back, all enqueued on the caller's stream
 * (cudaStream_t as void*; NULL = the context stream); the call returns at
 * once and the results are in the host arrays when the stream has finished
 * (cudaStreamSynchronize, or an event). Use page-locked host arrays: the
 * copies from pageable memory are not asynchronous. Calls on different
 * streams overlap: while one batch's results travel back, the next batch's
 * rays travel in and a third is traced. The device error word is not read
 * back by these calls: once the stream has finished, gpugi_device_error_bits
 * reports it.
 * Scratch and device staging (44 B per ray) are kept per stream, as for
 * gpugi_trace_closest_device_async. No counterpart in the reference. */
gpugi_status gpugi_trace_closest_async(gpugi_ctx* ctx, const gpugi_scene* scene,
                                       const float* ox, const float* oy, const float* oz,
                                       const float* dx, const float* dy, const float* dz,
                                       const float* tmax, uint64_t n,
                                       int32_t* slot, float* t, float* u, float* v, void* stream);
gpugi_status gpugi_trace_any_async(gpugi_ctx* ctx, const gpugi_scene* scene,
                                   const float* ox, const float* oy, const float* oz,
                                   const float* dx, const float* dy, const float* dz,
                                   const float* tmax, uint64_t n, uint8_t* occluded, void* stream);

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
 * by the caller. Asynchronous on the context stream. It always runs the
 * root prefilter and a queue walker (trace mode 2 when the context is set to
 * mode 0, 1 or 2, the context's group walker for modes 3-5): modes 0 and 1
 * need no queue and have no allocation-free form, and every mode returns the
 * same results. */
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
 * finished lanes from a device ray counter; mode 2: a coalesced
 * root-bounds prefilter that finishes rays missing the scene and queues the
 * rest (warp-ballot compaction) for the persistent walker; modes 3
 * (default), 4 and 5: the same prefilter, then groups of 8 (mode 3), 4
 * (mode 4) or 16 (mode 5) lanes walk one ray together, testing a window of
 * consecutive preorder nodes or leaf slots per round. All modes make the same decisions per ray as TraceRay and
 * return identical results. blockSize applies to mode 0. */
gpugi_status gpugi_set_trace_config(gpugi_ctx* ctx, uint32_t mode, uint32_t blockSize);

/* Host-pointer ray queries (gpugi_trace_closest / gpugi_trace_any). The
 * arrays go through device staging, and each call is split into `parts`
 * parts (1-8, default 2) whose copies to the device, traversal and copies
 * back overlap on separate streams (trace modes 2-5; neighbouring parts are
 * traversed on two streams, so one part's walker tail overlaps the next
 * part's walk; 1 disables the overlap). With zeroCopy (default 0) and every
 * array page-locked (cudaHostAlloc, cudaHostRegister), the kernels instead
 * read the rays and write the results over the host link directly, in one
 * part. Results are the same on every path. */
gpugi_status gpugi_set_host_pipeline(gpugi_ctx* ctx, uint32_t parts, uint32_t zeroCopy);
/* Share (percent, 1-100, default 50) of the persistent walker grid that a
 * stream-ordered query on device arrays (gpugi_trace_*_device_async)
 * launches. Queries on several streams then walk side by side, each one's
 * tail of deep walks overlapping the others' bulk: on the 2^20-ray
 * closest-hit workload over 4 streams, 50 % gives ~7 % more rays/s than the
 * full grid. Synchronous calls and host-array queries (paced by their
 * copies) use the full grid; results do not depend on the share. */
gpugi_status gpugi_set_async_walker_share(gpugi_ctx* ctx, uint32_t percent);

/* Scene layout tuning (set by the autotuner), applied to scenes uploaded
 * afterwards: the top tree levels (up to sharedNodes nodes, whole levels) are
 * stored first, breadth first, and the persistent walkers stage them in
 * shared memory: the ray queries stage up to sharedNodes, the renderers'
 * walkers up to renderSharedNodes. 0 disables staging. The logical walk and
 * every result are unchanged. */
gpugi_status gpugi_set_scene_layout(gpugi_ctx* ctx, uint32_t sharedNodes, uint32_t renderSharedNodes);

/* ------------------------------------------------------------------------
 * Rendering passes (wavefront): PT, LT, BPT and the Whitted ray tracer.
 *
 *   gpugi_render(pass = PT)   Pathtracer::Draw + pathtracer.comp
 *                             (gpugi/renderer/pathtracer.cpp:47-53, gpugi/shader/pathtracer.comp)
 *   gpugi_render(pass = LT)   LightPathtracer::Draw + lighttracer.comp + showlightcaches.comp
 *                             (gpugi/renderer/lightpathtracer.cpp:45-49)
 *   gpugi_render(pass = BPT)  BidirectionalPathtracer::Draw: reset counter, light
 *                             trace into the light cache, eye pass
 *                             (gpugi/renderer/bidirectionalpathtracer.cpp:182-203)
 *   gpugi_render(pass = WHITTED)  WhittedRayTracer::Draw + whittedraytracer.comp with
 *                             STOP_ON_DIFFUSE_BOUNCE (gpugi/renderer/whittedraytracer.cpp:32-38)
 *   gpugi_render(pass = PM)   PhotonMapper::Draw: clear the hash grid, photon
 *                             distribution, gather (gpugi/renderer/photonmapper.cpp:79-114,
 *                             gpugi/shader/photonmapper/{photondistribution,gather}.comp);
 *                             one photon map per iteration, see gpugi_set_photon_config
 *   gpugi_render(pass = HIERARCHY)  HierarchyImportance::Draw (gpugi/renderer/
 *                             hierarchyimportance.cpp:83-114): at iteration 0 the importance
 *                             pass (see gpugi_hierarchy_importance) with the call's first
 *                             light-sample set at the image size, then per sample
 *                             hierarchy/hierarchypathtracer.comp; needs an AABB hierarchy and
 *                             the node NDFs (gpugi_scene_set_hierarchy_ndf); maxPathLength is
 *                             the shader's MAX_PATHLENGTH (4 in the reference)
 *   gpugi_render(pass = IM)   PixelMapLighttracer::Draw (gpugi/renderer/pixelmaplighttracer.cpp:
 *                             76-116) as compiled there (lossless hash grid,
 *                             DEPTH_BUFFER_OCCLUSION_TEST): the eye pass stores one importon
 *                             per pixel in the hash grid and the first hits in a G-buffer
 *                             (pixelmaplt/importondistribution.comp), then the photons splat
 *                             into the importons' pixels and reproject against the G-buffer
 *                             (pixelmaplt/photontracing.comp); one importon map per iteration,
 *                             see gpugi_set_importon_config. The G-buffer is cleared at
 *                             iteration 0 and carries a missed pixel's previous first hit, as
 *                             the reference's position texture does
 * ------------------------------------------------------------------------ */
typedef struct gpugi_image gpugi_image;

enum gpugi_pass {
    GPUGI_PASS_PT = 0,
    GPUGI_PASS_LT = 1,
    GPUGI_PASS_BPT = 2,
    GPUGI_PASS_WHITTED = 3,
    GPUGI_PASS_PM = 4,
    GPUGI_PASS_HIERARCHY = 5,
    GPUGI_PASS_IM = 6
};

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
    uint32_t numLightSamples;  /* initial light samples per iteration (PT/BPT/Whitted/PM 128, LT 256) */
    float sky[3];              /* constant radiance on a miss (addition; 0 = the reference's black) */
    uint32_t flags;            /* GPUGI_RENDER_* bits; other bits must be 0 */
} gpugi_render_params;

/* Random streams of a pass. Default (flags 0): per-pixel PCG, the
 * PCG-RXS-M-XS-32 generator (an addition; the path seed of pixel p in
 * iteration i is pcg(pcg(i) + p)). With GPUGI_RENDER_REFERENCE_RNG the passes
 * draw gpugi's own streams (gpugi/shader/random.glsl:1-43: seed
 * wanghash(WangHash(i) + p), xorshift32 draws), the parity mode in which the
 * images follow the reference's random decisions. */
#define GPUGI_RENDER_REFERENCE_RNG 1u
#define GPUGI_RENDER_KNOWN_FLAGS GPUGI_RENDER_REFERENCE_RNG

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
/* Replace the accumulation with host sums (the inverse of gpugi_image_read;
 * resuming a checkpointed render, an addition: the reference only writes
 * PFM, gpugi/imageut/hdrimage.cpp:6-33). rgba is required; rgb64 NULL
 * zeroes an FP64 accumulation. Synchronous. */
gpugi_status gpugi_image_write(gpugi_ctx* ctx, gpugi_image* image, const float* rgba, const double* rgb64);
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

/* ------------------------------------------------------------------------
 * Neural radiance cache (NRC). No counterpart in the reference: a project
 * addition. A 64-64-64-64-64-3 ReLU MLP (no biases; one input is a constant
 * 1), FP16 weights and activations, FP32 accumulation on the tensor cores,
 * trained online with Adam on a relative L2 loss.
 * Query records: 12 floats {position, outgoing direction, normal, albedo};
 * training samples: 15 floats {query, target radiance rgb}. Positions are
 * normalised to the box given at creation.
 * ------------------------------------------------------------------------ */
typedef struct gpugi_nrc gpugi_nrc;
#define GPUGI_NRC_PARAMS 17408  /* 4 x 64 x 64 + 64 x 16 (output padded to 16) */

gpugi_status gpugi_nrc_create(gpugi_ctx* ctx, const float boxMin[3], const float boxMax[3], uint64_t seed,
                              float learningRate, gpugi_nrc** out);
void gpugi_nrc_destroy(gpugi_nrc* nrc);
/* FP32 master weights, layer l at l*4096, row-major [in][out] (out = 16 for l = 4). */
gpugi_status gpugi_nrc_get_weights(gpugi_ctx* ctx, const gpugi_nrc* nrc, float* weights);
gpugi_status gpugi_nrc_set_weights(gpugi_ctx* ctx, gpugi_nrc* nrc, const float* weights);
/* MLP kernels of the cache. GPUGI_NRC_KERNELS_TCGEN05 (the default): the
 * fifth-generation tensor cores (tcgen05.mma, f16 operands in shared
 * memory, f32 accumulators in tensor memory) on 128-sample tiles: one fused
 * kernel per training step (forward, backward and the weight gradients,
 * summed per CTA in tensor memory) and one for inference.
 * GPUGI_NRC_KERNELS_MMA_SYNC: the warp-level mma.sync kernels (inference;
 * forward + backward, then the weight-gradient GEMM), kept for comparison.
 * Waits for the queued work first. */
#define GPUGI_NRC_KERNELS_TCGEN05 0u
#define GPUGI_NRC_KERNELS_MMA_SYNC 1u
gpugi_status gpugi_nrc_set_kernels(gpugi_ctx* ctx, gpugi_nrc* nrc, uint32_t kernels);
/* Every mbarrier wait of the tcgen05 kernels is bounded (1 s of the global
 * timer by default); a wait that runs out sets GPUGI_DEVERR_WAIT_TIMEOUT, the
 * kernel frees its tensor memory and ends, and the context stays usable.
 * Test support: with stall = 1 those kernels issue no MMA and no commit, so
 * their first wait runs out after waitNs nanoseconds (0 = the default 1 s);
 * stall = 0 restores normal work. Waits for the queued work first. */
gpugi_status gpugi_nrc_debug_stall(gpugi_ctx* ctx, gpugi_nrc* nrc, uint32_t stall, uint64_t waitNs);
/* Inference (and the render pass) use an exponential moving average of the
 * trained weights, bias-corrected (decay 0.99 by default; 0 = the trained
 * weights themselves). Setting it, or the weights, restarts the average. */
gpugi_status gpugi_nrc_set_ema(gpugi_ctx* ctx, gpugi_nrc* nrc, float decay);
/* radiance[3 i + c] = max(network(query i)_c, 0). Device pointers, asynchronous. */
gpugi_status gpugi_nrc_infer_device(gpugi_ctx* ctx, const gpugi_nrc* nrc, const float* queries, uint64_t n,
                                    float* radiance);
/* One Adam step on n device samples; *loss (host, may be NULL) receives the
 * mean relative L2 loss before the step (synchronises when non-NULL). */
gpugi_status gpugi_nrc_train_device(gpugi_ctx* ctx, gpugi_nrc* nrc, const float* samples, uint64_t n, float* loss);
/* The loss gradient without a weight update (host outputs: predictions
 * n*3 may be NULL, gradient GPUGI_NRC_PARAMS floats). For checking. */
gpugi_status gpugi_nrc_gradient_device(gpugi_ctx* ctx, gpugi_nrc* nrc, const float* samples, uint64_t n,
                                       float* predictions, float* gradient, float* loss);
/* The 64-half input encoding of n queries (device output, n * 64 halves). */
gpugi_status gpugi_nrc_encode_device(gpugi_ctx* ctx, const gpugi_nrc* nrc, const float* queries, uint64_t n,
                                     void* encodedHalf);

/* Path tracing (params->pass PT) or bidirectional path tracing (BPT) with
 * the radiance cache. params->samples iterations run as frames of
 * samplesPerFrame iterations (one wavefront each).
 * PT: camera paths stop at vertex terminateDepth (or earlier, by path
 * spread, with terminateSpread > 0) and add throughput x
 * cache(vertex), except a trainFraction of the paths (chosen by a hash of
 * pixel and iteration) that trace full PT paths whose vertices become
 * training samples {query, radiance reflected towards the previous vertex}.
 * Both kinds of path splat into image.
 * BPT: the light pass (light cache and camera splats) runs
 * min(maxPathLength, terminateDepth) bounces; eye paths run
 * pathtracer_bidir.comp's bounce with light-cache connections limited to
 * paths of terminateDepth bounces and stop at vertex terminateDepth, adding
 * (eye throughput without its MIS factors) x cache(vertex): paths of at
 * most terminateDepth bounces keep BPT's estimator, longer ones come from
 * the cache. trainFraction x pixels x samplesPerFrame extra PT training
 * paths per frame only feed the cache (train != 0).
 * After the frame's lookups, trainSteps Adam steps run on the training
 * samples (at most maxTrainSamples, drawn in a shuffled path order) when
 * train != 0. Asynchronous: element counts stay in device memory; the call
 * returns once every frame is queued (it waits only when the light-sample
 * staging buffer is reused). */
typedef struct gpugi_nrc_params {
    uint32_t terminateDepth;  /* vertex index (0 = first hit) where render paths query the cache */
    float trainFraction;      /* share of pixels tracing training paths, in [0, 1] */
    uint32_t maxTrainSamples; /* cap on samples per frame (0: 65536) */
    uint32_t trainSteps;      /* Adam steps per frame on all of the frame's samples (0 counts as 1) */
    uint32_t train;           /* 0: use the cache without updating it */
    uint32_t samplesPerFrame; /* samples (iterations) traced per frame, one wavefront (0 counts as 1) */
    /* Self-training (Mueller et al. 2021, "Real-time Neural Radiance Caching
     * for Path Tracing", section 5): with trainLength >= 1 a training path
     * stops at vertex trainLength and takes the cache's radiance there, times
     * its throughput, as the rest of its path; unbiasedFraction of the
     * training paths (a hash of path and iteration) run to the path's end
     * instead. trainLength 0: every training path runs to its end. */
    uint32_t trainLength;
    float unbiasedFraction;   /* in [0, 1]; read when trainLength >= 1 */
    /* PT only: > 0 stops a render path at the first vertex n >= 1 whose path
     * spread a(x1..xn) = (sum of |x_{i-1} - x_i| / sqrt(p(w_i) |cos theta_i|))^2
     * exceeds terminateSpread x a0, a0 = |x0 - x1|^2 / (4 pi cos theta_1)
     * (the same paper, section 3.4, c = 0.01 there), and at vertex
     * terminateDepth at the latest. 0: at vertex terminateDepth. */
    float terminateSpread;
    /* Frames in flight: frames alternate over this many wavefront lanes
     * (buffer sets and streams; 0 = 4, at most 4), so a frame's walker tails
     * overlap the next frames' bounces; the network's inference and training
     * stay in frame order. */
    uint32_t lanes;
} gpugi_nrc_params;

gpugi_status gpugi_render_nrc(gpugi_ctx* ctx, const gpugi_scene* scene, const gpugi_camera* camera,
                              const gpugi_render_params* params, const float* lightSamples, uint64_t* rngState,
                              gpugi_nrc* nrc, const gpugi_nrc_params* nrcParams, gpugi_image* image);

/* Batched rendering: many jobs, each with its own scene, camera, image,
 * resolution, sample count and path length, in one wavefront. No single
 * counterpart in the reference (RendererSystem::Draw renders one scene per
 * call, gpugi/renderer/renderersystem.cpp:235-258); per job the result is
 * gpugi_render's with the same arguments (same seeds and light samples).
 * PT, LT and BPT jobs share the queues: each stage (generate, then per
 * bounce extend, shade, shadow) is one launch over the paths of all jobs.
 * Phase 0 holds the PT eye paths, the LT particles (with the light samples'
 * camera connections) and the BPT light paths, which fill each BPT job's
 * light caches; phase 1 the BPT eye paths. The whole sequence is captured
 * once as a CUDA graph and replayed per round; a round holds at most the
 * context's path-queue capacity (gpugi_set_batch_config) of paths per phase
 * and at most 4 GiB of light caches (at least one sample of the largest BPT
 * job). A job whose single sample needs more paths than the capacity (PT:
 * width x height; LT: its particles plus numLightSamples; BPT: its particles,
 * and width x height) is refused with GPUGI_ERROR_INVALID_ARGUMENT. BPT
 * connections pick light-cache entries whose order follows the device's
 * atomic appends, so a BPT job equals gpugi_render's in distribution (and
 * exactly at maxPathLength 1). Whitted, photon-mapper and importon-map jobs are rendered
 * afterwards, one gpugi_render call each. Jobs that share an rngState draw
 * their light samples in round order. */
typedef struct gpugi_job {
    const gpugi_scene* scene;
    gpugi_camera camera;
    gpugi_render_params params;
    const float* lightSamples;  /* params.samples x numLightSamples x 8 floats, or NULL */
    uint64_t* rngState;         /* host light sampler state when lightSamples is NULL */
    gpugi_image* image;
} gpugi_job;

gpugi_status gpugi_render_batch(gpugi_ctx* ctx, const gpugi_job* jobs, uint32_t numJobs);

/* Path-queue capacity of one batched round (paths in flight per phase;
 * default 16M, in [1024, 64M]) and whether rounds replay a CUDA graph
 * (default 1). */
gpugi_status gpugi_set_batch_config(gpugi_ctx* ctx, uint32_t pathsPerRound, uint32_t useGraph);

/* Photon mapper settings (PhotonMapper's pm_nphotons, pm_r and
 * pm_progressive; gpugi/renderer/photonmapper.cpp:17-45): photons traced per
 * light sample (default 2048), query radius (default 0.01; grid spacing
 * 2.01 x radius) and Knaus-Zwicker radius shrinking per iteration (default 0). */
gpugi_status gpugi_set_photon_config(gpugi_ctx* ctx, uint32_t photonsPerLightSample, float queryRadius,
                                     uint32_t progressive);

/* Importon map light tracer settings (PixelMapLighttracer's im_nphotons,
 * im_r and im_progressive; gpugi/renderer/pixelmaplighttracer.cpp:19-41):
 * photons per light sample (default 2048), query radius (default 0.005; grid
 * spacing 2.01 x radius) and Knaus-Zwicker radius shrinking (default 0). */
gpugi_status gpugi_set_importon_config(gpugi_ctx* ctx, uint32_t photonsPerLightSample, float queryRadius,
                                       uint32_t progressive);

/* Hierarchy-importance renderer (HierarchyImportance, gpugi/renderer/
 * hierarchyimportance.cpp). AABB hierarchies only: the reference's
 * importance shaders test box (or oriented-box) nodes.
 *
 * gpugi_scene_set_hierarchy_ndf  HierarchyImportance::SetScene: the node NDFs
 *     (bvhmake's "approx_sggx" chunk, 6 uint16 per node in the uploaded node
 *     order, see gpugi_bvh_sggx) and the node materials of
 *     ComputeHierarchyMaterials (hierarchyimportance.cpp:136-160): area-
 *     weighted averages of the triangles' materials below each node, stored
 *     as packed halves (sampleleafmaterials.comp, pullmaterials.comp).
 * gpugi_hierarchy_importance  the importance pass of HierarchyImportance::Draw
 *     (hierarchyimportance.cpp:83-109): `iterations` passes of
 *     acquisition2.comp (one path of up to 8 vertices per pixel, each vertex
 *     with one next-event ray; every node entered and every triangle hit adds
 *     the path importance, halved per vertex) numbered 1..iterations, then
 *     the propagation (hierarchypropagation_init.comp, _nodes.comp): per node
 *     x = mean importance, subtree = importance of its children, y =
 *     (x / subtree)^2 x mean face area. The init shader reads the node's
 *     minimum corner from an undeclared variable (hierarchypropagation_init.
 *     comp:59); the node's first texel is used, as in the nodes shader.
 * gpugi_hierarchy_read  copies of the results in the uploaded node order:
 *     importance {x, y} per node then per leaf slot (2 x (numNodes + numSlots)
 *     floats), subtree importance per node, and the node materials (12 uint32
 *     per node: six pairs of halves {Reflectiveness.xy}, {.zw}, {Opacity.xy},
 *     {Opacity.z, area}, {Diffuse.xy}, {Diffuse.z, 0}, {Emissivity.xy},
 *     {Emissivity.z, 0}, {Fresnel0.xy}, {Fresnel0.z, RefractionIndexAvg},
 *     {Fresnel1.xy}, {Fresnel1.z, 0}). Any pointer may be NULL. */
gpugi_status gpugi_scene_set_hierarchy_ndf(gpugi_ctx* ctx, gpugi_scene* scene, const uint16_t* sggx);
gpugi_status gpugi_hierarchy_importance(gpugi_ctx* ctx, gpugi_scene* scene, const gpugi_camera* camera,
                                        uint32_t width, uint32_t height, const float* lightSamples,
                                        uint32_t numLightSamples, uint32_t iterations);
gpugi_status gpugi_hierarchy_read(gpugi_ctx* ctx, const gpugi_scene* scene, float* importance, float* subtree,
                                  uint32_t* materials);

/* L2 read bandwidth of the device, for the second roofline of L2-resident
 * scenes: one launch re-reads a `bytes` buffer (1-64 MiB, L2-resident)
 * `reps` times with 16-B loads cached in L2 only; GB/s of bytes read, CUDA
 * events. No counterpart in the reference. Synchronises; allocates. */
gpugi_status gpugi_measure_l2_bandwidth(gpugi_ctx* ctx, uint64_t bytes, uint32_t reps, double* gbs);

/* Autotuner. No counterpart in the reference (its launch shapes are fixed
 * local sizes, e.g. gpugi/renderer/pathtracer.cpp:11). Times candidates on
 * the scene with CUDA events and applies the fastest to the context:
 * GPUGI_TUNE_TRACE: ray-query kernels (gpugi_set_trace_config mode and block
 * size) on 2^20 synthetic rays over the scene bounds; GPUGI_TUNE_BATCH: the
 * path-queue capacity of batched rounds on a 512 x 512, 64-spp PT job
 * (needs vertex info and materials). The traversal is stackless, so no stack
 * depth is tuned. Synchronises; allocates temporary buffers. */
#define GPUGI_TUNE_TRACE 1u
#define GPUGI_TUNE_BATCH 2u
typedef struct gpugi_tuning {
    uint32_t traceMode, traceBlock; /* chosen ray-query settings */
    uint32_t batchPaths;            /* chosen paths per batched round */
    double traceMraysPerSecond;     /* closest-hit rate of the chosen setting (0 if not tuned) */
    double batchMpathsPerSecond;    /* camera paths per second of the chosen capacity (0 if not tuned) */
} gpugi_tuning;
gpugi_status gpugi_autotune(gpugi_ctx* ctx, const gpugi_scene* scene, uint32_t flags, gpugi_tuning* out);

/* Rays traced by the last gpugi_render call, by kind: {camera/extension
 * (closest hit), shadow/connection (any hit)}. Synchronises. */
gpugi_status gpugi_render_ray_counts(gpugi_ctx* ctx, uint64_t counts[2]);

#ifdef __cplusplus
}
#endif
#endif
