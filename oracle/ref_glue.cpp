// ORACLE — test infrastructure only. Not part of the product.
//
// Glue around the reference's own shader text (rewritten by
// oracle/ref_build.py into oracle/_ref/gen/, compiled against ref_shim.hpp):
// it binds scene arrays to the shaders' buffers and exports C entry points
// that tests/test_ref_pinned.py calls side by side with the oracle's.
//   ref_trace_closest / ref_trace_any   TraceRay / TraceRayAnyHit
//                                       (gpugi/shader/traceray.glsl with AABOX_BVH,
//                                       intersectiontests.glsl), leaf blocks of 8 or 2;
//                                       with OBOX_BVH (oriented boxes), leaf blocks of 8
//   ref_eval                            random.glsl / helper.glsl functions
//   ref_render_pt                       pathtracer.comp's main() per pixel
//   ref_render_lt                       lighttracer.comp + showlightcaches.comp (LightPathtracer::Draw),
//                                       or with bidir the cache-filling light pass + pathtracer_bidir.comp,
//                                       or (bidir = 2) whittedraytracer.comp per pixel,
//                                       (3) the photon mapper, (4) the importon map light tracer
//   ref_render_hier                     hierarchy/hierarchypathtracer.comp per pixel
//   ref_hier_importance                 acquisition2.comp x iterations + the propagation shaders
//   ref_hier_materials                  sampleleafmaterials.comp + pullmaterials.comp per tree level
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "ref_shim.hpp"

namespace glslref {
const vec4* g_textureColours = nullptr;
thread_local uvec3 gl_GlobalInvocationID;
}  // namespace glslref

// ------------------------------------------------ traversal, 8-slot leaves
namespace ref_leaf8 {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#define AABOX_BVH
#include "helper.glsl.h"
#include "scenedata.glsl.h"
#include "intersectiontests.glsl.h"
#include "random.glsl.h"
#include "traceray.glsl.h"
#define ANY_HIT
#include "traceray.glsl.h"
#undef ANY_HIT
#undef TRIANGLES_PER_LEAF
}  // namespace ref_leaf8

// ------------------------------------------------ traversal, 2-slot leaves
namespace ref_leaf2 {
using namespace glslref;
#define TRIANGLES_PER_LEAF 2
#include "helper.glsl.h"
#include "scenedata.glsl.h"
#include "intersectiontests.glsl.h"
#include "random.glsl.h"
#include "traceray.glsl.h"
#define ANY_HIT
#include "traceray.glsl.h"
#undef ANY_HIT
#undef TRIANGLES_PER_LEAF
}  // namespace ref_leaf2

// ------------------------------------------------ oriented-box nodes (OBOX_BVH), 8-slot leaves
namespace ref_obox8 {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#undef AABOX_BVH
#define OBOX_BVH
#include "helper.glsl.h"
#include "scenedata.glsl.h"
#include "intersectiontests.glsl.h"
#include "random.glsl.h"
#include "traceray.glsl.h"
#define ANY_HIT
#include "traceray.glsl.h"
#undef ANY_HIT
#undef OBOX_BVH
#define AABOX_BVH
#undef TRIANGLES_PER_LEAF
}  // namespace ref_obox8

// ------------------------------------------------ the path tracer, 8-slot leaves
namespace ref_pt {
using namespace glslref;
int g_maxPathLength = 8;  // MAX_PATHLENGTH, injected by the application (application.cpp:123)
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define main PathtracerMain
#include "pathtracer.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_pt
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE

// ------------------------------------------------ lighttracer.comp (LightPathtracer's shader)
namespace ref_lt {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define main LighttracerMain
#include "lighttracer.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_lt
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE

// ------------------------------------------------ showlightcaches.comp (RendererSystem::DispatchShowLightCacheShader)
namespace ref_slc {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define main ShowLightCachesMain
#include "showlightcaches.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_slc
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE

// ------------------------------------------------ BidirectionalPathtracer's shaders
// the light pass: lighttracer.comp with SAVE_LIGHT_CACHE (bidirectionalpathtracer.cpp:146-147)
namespace ref_bpl {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define SAVE_LIGHT_CACHE
#define main BidirLightMain
#include "lighttracer.comp.h"
#undef main
#undef SAVE_LIGHT_CACHE
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_bpl
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE

// the eye pass: bidirpathtracer/pathtracer_bidir.comp
namespace ref_bpe {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define main BidirEyeMain
#include "bidirpathtracer/pathtracer_bidir.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_bpe
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE

// ------------------------------------------------ whittedraytracer.comp (WhittedRayTracer's shader)
namespace ref_wh {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define STOP_ON_DIFFUSE_BOUNCE  // whittedraytracer.cpp:40
#define main WhittedMain
#include "whittedraytracer.comp.h"
#undef main
#undef STOP_ON_DIFFUSE_BOUNCE
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_wh
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE

// ------------------------------------------------ PhotonMapper's shaders (lossless hash map)
namespace ref_pmd {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define main PhotonDistributionMain
#include "photonmapper/photondistribution.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_pmd
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace ref_pmg {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define main PhotonGatherMain
#include "photonmapper/gather.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_pmg
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

// ------------------------------------------------ PixelMapLighttracer's shaders (pixelmaplighttracer.cpp:128-142)
namespace ref_imd {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define DEPTH_BUFFER_OCCLUSION_TEST
#define main ImportonDistributionMain
#include "pixelmaplt/importondistribution.comp.h"
#undef main
#undef DEPTH_BUFFER_OCCLUSION_TEST
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_imd
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace ref_imp {
using namespace glslref;
int g_maxPathLength = 8;
#define MAX_PATHLENGTH g_maxPathLength
#define TRIANGLES_PER_LEAF 8
#define DEPTH_BUFFER_OCCLUSION_TEST
#define main ImportonPhotonMain
#include "pixelmaplt/photontracing.comp.h"
#undef main
#undef DEPTH_BUFFER_OCCLUSION_TEST
#undef REPROJECT
#undef USE_PIXEL_CACHE
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
}  // namespace ref_imp
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

// ------------------------------------------------ hierarchypathtracer.comp (HierarchyImportance's renderer)
namespace ref_hpt {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#define main HierarchyPathtracerMain
#include "hierarchy/hierarchypathtracer.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef MAX_PATHLENGTH
#undef IMPORTANCE_THRESHOLD
#undef HIT_INDEX_OUTPUT
#undef TRACERAY_IMPORTANCE_BREAK
}  // namespace ref_hpt
// the shader's own switches end with it
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

// ------------------------------------------------ the hierarchy-importance passes
// acquisition2.comp (+ counthits.glsl), hierarchypropagation_init.comp and
// _nodes.comp, sampleleafmaterials.comp and pullmaterials.comp; each in its
// own namespace, bound to the same arrays by the entry points below.
namespace ref_acq {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#define main AcquisitionMain
#include "hierarchy/acquisition2.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef NEXT_EVENT_IMPORTANCE
#undef HIT_INDEX_OUTPUT
#undef MAX_PATHLENGTH
}  // namespace ref_acq
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace ref_pinit {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
// hierarchypropagation_init.comp reads the node's minimum corner from an
// undeclared `hierarchy0` (the shader does not compile for AABB
// hierarchies as written); it is the node's first texel, as
// hierarchypropagation_nodes.comp declares it.
#define hierarchy0 texelFetch(HierachyBuffer, int(gl_GlobalInvocationID.x) * HierarchyBufferStride)
#define main PropagationInitMain
#include "hierarchy/hierarchypropagation_init.comp.h"
#undef main
#undef hierarchy0
#undef TRIANGLES_PER_LEAF
}  // namespace ref_pinit
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace ref_pnodes {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#define main PropagationNodesMain
#include "hierarchy/hierarchypropagation_nodes.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
#undef TRIINDEX_OUTPUT
}  // namespace ref_pnodes
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace ref_leafm {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#define main SampleLeafMaterialsMain
#include "hierarchy/sampleleafmaterials.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
}  // namespace ref_leafm
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace ref_pullm {
using namespace glslref;
#define TRIANGLES_PER_LEAF 8
#define main PullMaterialsMain
#include "hierarchy/pullmaterials.comp.h"
#undef main
#undef TRIANGLES_PER_LEAF
}  // namespace ref_pullm
#undef TRINORMAL_OUTPUT
#undef SAMPLING_DECISION_OUTPUT
#undef NUM_LIGHT_SAMPLES
#undef LOCAL_SIZE
#undef QUADRATIC_PROBING
#undef HASH_MAP_BINDIDX
#undef HASH_MAP_DATA_BINDIDX

namespace {

template <typename F>
void parallel_for(uint64_t n, int threads, F fn) {
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > n) threads = (int)(n ? n : 1);
    std::vector<std::thread> pool;
    const uint64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const uint64_t b = (uint64_t)t * chunk, e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back([=]() { fn(b, e); });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

#define GPUGI_REF_BIND(NS)                                                         \
    NS::HierachyBuffer = glslref::samplerBuffer{hierarchy, 4};                     \
    NS::TriangleBuffer = glslref::isamplerBuffer{reinterpret_cast<const glslref::ivec4*>(slots)}; \
    NS::VertexPositionBuffer = glslref::samplerBuffer{positions, 3};

extern "C" {

// Closest hit with the reference's TraceRay: the Triangle record it returns
// ({v0, v1, v2, material}, all -1 on a miss), t, u = barycentric.y,
// v = barycentric.z.
int ref_trace_closest(const float* hierarchy, const int32_t* slots, const float* positions, int leafSize,
                      int boundsKind, const float* ox, const float* oy, const float* oz, const float* dx,
                      const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* outTri, float* outT,
                      float* outU, float* outV, int numThreads) {
    using namespace glslref;
    const bool obox = boundsKind == 2;
    if ((leafSize != 8 && leafSize != 2) || (obox && leafSize != 8) || (boundsKind != 0 && !obox)) return 1;
    if (obox) {
        GPUGI_REF_BIND(ref_obox8)
    } else if (leafSize == 8) {
        GPUGI_REF_BIND(ref_leaf8)
    } else {
        GPUGI_REF_BIND(ref_leaf2)
    }
    parallel_for(n, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            ref_leaf8::Ray r8;
            ref_leaf2::Ray r2;
            ref_obox8::Ray ro;
            r8.Origin = r2.Origin = ro.Origin = vec3(ox[i], oy[i], oz[i]);
            r8.Direction = r2.Direction = ro.Direction = vec3(dx[i], dy[i], dz[i]);
            float rayLength = tmax[i];
            vec3 bary(-1.0f);
            ivec4 tri(-1, -1, -1, -1);
            if (obox) ref_obox8::TraceRay(ro, rayLength, bary, tri);
            else if (leafSize == 8) ref_leaf8::TraceRay(r8, rayLength, bary, tri);
            else ref_leaf2::TraceRay(r2, rayLength, bary, tri);
            // the shader leaves its out parameters unwritten on a miss
            const bool hit = rayLength < tmax[i];
            outTri[4 * i] = hit ? tri.x : -1;
            outTri[4 * i + 1] = hit ? tri.y : -1;
            outTri[4 * i + 2] = hit ? tri.z : -1;
            outTri[4 * i + 3] = hit ? tri.w : -1;
            outT[i] = rayLength;
            outU[i] = hit ? bary.y : 0.0f;
            outV[i] = hit ? bary.z : 0.0f;
        }
    });
    return 0;
}

int ref_trace_any(const float* hierarchy, const int32_t* slots, const float* positions, int leafSize,
                  int boundsKind, const float* ox, const float* oy, const float* oz, const float* dx,
                  const float* dy, const float* dz, const float* tmax, uint64_t n, uint8_t* occluded,
                  int numThreads) {
    using namespace glslref;
    const bool obox = boundsKind == 2;
    if ((leafSize != 8 && leafSize != 2) || (obox && leafSize != 8) || (boundsKind != 0 && !obox)) return 1;
    if (obox) {
        GPUGI_REF_BIND(ref_obox8)
    } else if (leafSize == 8) {
        GPUGI_REF_BIND(ref_leaf8)
    } else {
        GPUGI_REF_BIND(ref_leaf2)
    }
    parallel_for(n, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            const vec3 o(ox[i], oy[i], oz[i]), d(dx[i], dy[i], dz[i]);
            bool hit;
            if (obox) {
                ref_obox8::Ray r;
                r.Origin = o;
                r.Direction = d;
                hit = ref_obox8::TraceRayAnyHit(r, tmax[i]);
            } else if (leafSize == 8) {
                ref_leaf8::Ray r;
                r.Origin = o;
                r.Direction = d;
                hit = ref_leaf8::TraceRayAnyHit(r, tmax[i]);
            } else {
                ref_leaf2::Ray r;
                r.Origin = o;
                r.Direction = d;
                hit = ref_leaf2::TraceRayAnyHit(r, tmax[i]);
            }
            occluded[i] = hit ? 1 : 0;
        }
    });
    return 0;
}

// Functions of random.glsl and helper.glsl over arrays (kind selects):
//   0 wanghash(u)                        in: u32        out: u32
//   1 RandomUInt x4 from seed u          in: u32        out: 4 u32 (the stream)
//   2 Random x4 from seed u              in: u32        out: 4 floats
//   3 InitRandomSeed(a, b)               in: 2 u32      out: u32
//   4 SampleDirection(r)                 in: 2 floats   out: 3 floats
//   5 SampleHemisphereCosine(r, ONB(n))  in: 5 floats   out: 3 floats (r, n)
//   6 SamplePhongLobe(r, e, ONB(n))      in: 6 floats   out: 3 floats (r, e, n)
//   7 CreateONB(n)                       in: 3 floats   out: 6 floats (U, V)
//   8 UnpackNormal(vec2)                 in: 2 floats   out: 3 floats
//   9 PackNormal(n)                      in: 3 floats   out: 2 floats
//  10 GetLuminance(c)                    in: 3 floats   out: 1 float
int ref_eval(int kind, uint64_t n, const void* in, void* out) {
    using namespace ref_leaf8;
    const uint32_t* iu = static_cast<const uint32_t*>(in);
    const float* f = static_cast<const float*>(in);
    uint32_t* ou = static_cast<uint32_t*>(out);
    float* of = static_cast<float*>(out);
    for (uint64_t i = 0; i < n; ++i) {
        switch (kind) {
        case 0: ou[i] = wanghash(iu[i]); break;
        case 1: {
            uint s = iu[i];
            for (int k = 0; k < 4; ++k) ou[4 * i + k] = RandomUInt(s);
            break;
        }
        case 2: {
            uint s = iu[i];
            for (int k = 0; k < 4; ++k) of[4 * i + k] = Random(s);
            break;
        }
        case 3: ou[i] = InitRandomSeed(iu[2 * i], iu[2 * i + 1]); break;
        case 4: {
            vec3 d = SampleDirection(vec2(f[2 * i], f[2 * i + 1]));
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 5: {
            const float* p = f + 5 * i;
            vec3 N(p[2], p[3], p[4]), U, V;
            CreateONB(N, U, V);
            vec3 d = SampleHemisphereCosine(vec2(p[0], p[1]), U, V, N);
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 6: {
            const float* p = f + 6 * i;
            vec3 N(p[3], p[4], p[5]), U, V;
            CreateONB(N, U, V);
            vec3 d = SamplePhongLobe(vec2(p[0], p[1]), p[2], U, V, N);
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 7: {
            vec3 N(f[3 * i], f[3 * i + 1], f[3 * i + 2]), U, V;
            CreateONB(N, U, V);
            of[6 * i] = U.x, of[6 * i + 1] = U.y, of[6 * i + 2] = U.z;
            of[6 * i + 3] = V.x, of[6 * i + 4] = V.y, of[6 * i + 5] = V.z;
            break;
        }
        case 8: {
            vec3 d = UnpackNormal(vec2(f[2 * i], f[2 * i + 1]));
            of[3 * i] = d.x, of[3 * i + 1] = d.y, of[3 * i + 2] = d.z;
            break;
        }
        case 9: {
            vec2 p = PackNormal(vec3(f[3 * i], f[3 * i + 1], f[3 * i + 2]));
            of[2 * i] = p.x, of[2 * i + 1] = p.y;
            break;
        }
        case 10: of[i] = GetLuminance(vec3(f[3 * i], f[3 * i + 1], f[3 * i + 2])); break;
        default: return 1;
        }
    }
    return 0;
}

// One iteration of pathtracer.comp over every pixel of a width x height
// image (the reference dispatches whole 8x8 groups only; every pixel here),
// accumulated into accum (RGBA32F). Scene arrays as oracle_render takes
// them; materials: 24 floats per material (the library's record), turned
// into the shader's Material UBO with one constant "texture" per map;
// camera: U, V, W, position, pixelArea (13 floats); sky: the constant
// environment radiance.
int ref_render_pt(const float* hierarchy, const int32_t* slots, const float* positions, const float* vertexInfo,
                  const float* materials, int numMaterials, int width, int height, int maxPathLength,
                  const float* cam, uint32_t frameSeed, const float* lightSamples, int numLightSamples,
                  const float* sky, float* accum, int numThreads) {
    using namespace glslref;
    if (numMaterials > 256) return 1;  // the shader's UBO holds 256 materials (globaluniforms.glsl:23-27)
    namespace P = ref_pt;
    P::HierachyBuffer = samplerBuffer{hierarchy, 4};
    P::TriangleBuffer = isamplerBuffer{reinterpret_cast<const ivec4*>(slots)};
    P::VertexPositionBuffer = samplerBuffer{positions, 3};
    P::VertexInfoBuffer = samplerBuffer{vertexInfo, 4};
    P::InitialLightSampleBuffer = samplerBuffer{lightSamples, 4};
    std::vector<vec4> colours(4 * (size_t)numMaterials);
    for (int m = 0; m < numMaterials; ++m) {
        const float* r = materials + 24 * (size_t)m;
        colours[4 * m + 0] = vec4(r[0], r[1], r[2], 1.0f);     // diffuse
        colours[4 * m + 1] = vec4(r[4], r[5], r[6], 1.0f);     // opacity
        colours[4 * m + 2] = vec4(r[8], r[9], r[10], r[11]);   // reflectiveness, w = Phong exponent
        colours[4 * m + 3] = vec4(r[12], r[13], r[14], 1.0f);  // emissivity
        P::Material& M = P::Materials[m];
        M.diffuseTexHandle = uvec2(4 * m + 0, 0);
        M.opacityTexHandle = uvec2(4 * m + 1, 0);
        M.reflectivenessTexHandle = uvec2(4 * m + 2, 0);
        M.emissivityTexHandle = uvec2(4 * m + 3, 0);
        M.Fresnel0 = vec3(r[16], r[17], r[18]);
        M.RefractionIndexAvg = r[3];
        M.Fresnel1 = vec3(r[20], r[21], r[22]);
    }
    g_textureColours = colours.data();
    P::BackbufferSize = ivec2(width, height);
    P::NumInitialLightSamples = numLightSamples;
    P::CameraU = vec3(cam[0], cam[1], cam[2]);
    P::CameraV = vec3(cam[3], cam[4], cam[5]);
    P::CameraW = vec3(cam[6], cam[7], cam[8]);
    P::CameraPosition = vec3(cam[9], cam[10], cam[11]);
    P::PixelArea = cam[12];
    P::FrameSeed = frameSeed;
    P::IterationCount = 0;
    P::EnvironmentMap.colour = vec3(sky[0], sky[1], sky[2]);
    P::OutputTexture = image2D{reinterpret_cast<vec4*>(accum), width, height};
    P::g_maxPathLength = maxPathLength;
    parallel_for((uint64_t)width * height, numThreads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            gl_GlobalInvocationID = uvec3((uint)(i % width), (uint)(i / width), 0u);
            P::PathtracerMain();
        }
    });
    g_textureColours = nullptr;
    return 0;
}

// One iteration of LightPathtracer::Draw (lightpathtracer.cpp:45-51), or
// with bidir of BidirectionalPathtracer::Draw: the
// light tracer over numLightSamples x raysPerLightSample invocations, then
// showlightcaches.comp over the light samples (the reference dispatches it
// with 64 invocations per light sample, lightpathtracer.cpp:48 via
// renderersystem.cpp:280; the ones past the last sample read zero light
// samples and add nothing). Invocations run in order on one thread, so the
// image sums are in a fixed order.
int ref_render_lt(const float* hierarchy, const int32_t* slots, const float* positions, const float* vertexInfo,
                  const float* materials, int numMaterials, int width, int height, int maxPathLength,
                  const float* cam, uint32_t frameSeed, const float* lightSamples, int numLightSamples,
                  int raysPerLightSample, int bidir, float param, float* accum, float* position) {
    using namespace glslref;
    if (numMaterials > 256) return 1;
    std::vector<vec4> colours(4 * (size_t)numMaterials);
    auto bind = [&](auto& M, int m, const float* r) {
        M.diffuseTexHandle = uvec2(4 * m + 0, 0);
        M.opacityTexHandle = uvec2(4 * m + 1, 0);
        M.reflectivenessTexHandle = uvec2(4 * m + 2, 0);
        M.emissivityTexHandle = uvec2(4 * m + 3, 0);
        M.Fresnel0 = vec3(r[16], r[17], r[18]);
        M.RefractionIndexAvg = r[3];
        M.Fresnel1 = vec3(r[20], r[21], r[22]);
    };
    for (int m = 0; m < numMaterials; ++m) {
        const float* r = materials + 24 * (size_t)m;
        colours[4 * m + 0] = vec4(r[0], r[1], r[2], 1.0f);
        colours[4 * m + 1] = vec4(r[4], r[5], r[6], 1.0f);
        colours[4 * m + 2] = vec4(r[8], r[9], r[10], r[11]);
        colours[4 * m + 3] = vec4(r[12], r[13], r[14], 1.0f);
        bind(ref_lt::Materials[m], m, r);
        bind(ref_slc::Materials[m], m, r);
        bind(ref_bpl::Materials[m], m, r);
        bind(ref_bpe::Materials[m], m, r);
        bind(ref_wh::Materials[m], m, r);
        bind(ref_pmd::Materials[m], m, r);
        bind(ref_pmg::Materials[m], m, r);
        bind(ref_imd::Materials[m], m, r);
        bind(ref_imp::Materials[m], m, r);
    }
    g_textureColours = colours.data();
#define GPUGI_REF_SCENE(NS)                                                           \
    NS::HierachyBuffer = samplerBuffer{hierarchy, 4};                                 \
    NS::TriangleBuffer = isamplerBuffer{reinterpret_cast<const ivec4*>(slots)};       \
    NS::VertexPositionBuffer = samplerBuffer{positions, 3};                           \
    NS::VertexInfoBuffer = samplerBuffer{vertexInfo, 4};                              \
    NS::InitialLightSampleBuffer = samplerBuffer{lightSamples, 4};                    \
    NS::BackbufferSize = ivec2(width, height);                                        \
    NS::NumInitialLightSamples = numLightSamples;                                     \
    NS::CameraU = vec3(cam[0], cam[1], cam[2]);                                       \
    NS::CameraV = vec3(cam[3], cam[4], cam[5]);                                       \
    NS::CameraW = vec3(cam[6], cam[7], cam[8]);                                       \
    NS::CameraPosition = vec3(cam[9], cam[10], cam[11]);                              \
    NS::PixelArea = cam[12];                                                          \
    NS::FrameSeed = frameSeed;                                                        \
    NS::IterationCount = 0;                                                           \
    NS::g_maxPathLength = maxPathLength;
    GPUGI_REF_SCENE(ref_lt)
    GPUGI_REF_SCENE(ref_slc)
    GPUGI_REF_SCENE(ref_bpl)
    GPUGI_REF_SCENE(ref_bpe)
    GPUGI_REF_SCENE(ref_wh)
    GPUGI_REF_SCENE(ref_pmd)
    GPUGI_REF_SCENE(ref_pmg)
    GPUGI_REF_SCENE(ref_imd)
    GPUGI_REF_SCENE(ref_imp)
#undef GPUGI_REF_SCENE
    for (image2D* im : {&ref_lt::OutputTexture, &ref_slc::OutputTexture, &ref_bpl::OutputTexture,
                        &ref_bpe::OutputTexture, &ref_wh::OutputTexture, &ref_pmg::OutputTexture,
                        &ref_imd::OutputTexture, &ref_imp::OutputTexture})
        *im = image2D{reinterpret_cast<vec4*>(accum), width, height};
    const uint64_t n = (uint64_t)numLightSamples * raysPerLightSample;
    if (bidir == 4) {
        // PixelMapLighttracer::Draw (pixelmaplighttracer.cpp:76-125): the map
        // cleared, importondistribution.comp per pixel (importons at index
        // 2 x pixel; the first hit's position and packed normal y into the
        // position texture, its packed normal x into the image's alpha),
        // then photontracing.comp over numLightSamples x photonsPerLightSample
        // invocations; param = the query radius. position: the position
        // texture (H x W x 4), carried between iterations like the image.
        const float radius = param;
        uint32_t size = (uint32_t)std::max<uint64_t>(1031, 4 * (uint64_t)width * height + 1);
        auto prime = [](uint32_t v) {
            if (v < 2) return false;
            for (uint32_t d = 2; (uint64_t)d * d <= v; ++d)
                if (v % d == 0) return false;
            return true;
        };
        while (!prime(size)) ++size;
        std::vector<uvec2> map(size, uvec2(0xffffffffu, 0xffffffffu));
        std::vector<ivec4> data(2 * (size_t)width * height + 2);
        ref_imd::HashMap = ref_imp::HashMap = map.data();
        ref_imd::HashMapData = ref_imp::HashMapData = data.data();
        ref_imd::HashMapSize = ref_imp::HashMapSize = size;
        ref_imd::NumPhotonsPerLightSample = ref_imp::NumPhotonsPerLightSample = raysPerLightSample;
        ref_imd::HashGridSpacing = ref_imp::HashGridSpacing = radius * 2.01f;
        ref_imd::PhotonQueryRadiusSq = ref_imp::PhotonQueryRadiusSq = radius * radius;
        ref_imd::PositionTexture = ref_imp::PositionTexture =
            image2D{reinterpret_cast<vec4*>(position), width, height};
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
                ref_imd::ImportonDistributionMain();
            }
        for (uint64_t i = 0; i < n; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            ref_imp::ImportonPhotonMain();
        }
    } else if (bidir == 3) {
        // PhotonMapper::Draw (photonmapper.cpp:69-112): the hash map cleared to
        // all ones and its data to zero, photondistribution.comp over
        // numLightSamples x photonsPerLightSample (raysPerLightSample)
        // invocations, then gather.comp per pixel; param = the query radius
        // r (HashGridSpacing = 2.01 r, PhotonQueryRadiusSq = r^2). The
        // map's size is a prime above four entries per possible photon
        // (the reference sizes it from its own photon estimate), so probing
        // never fills it; the data holds two texels per photon.
        const float radius = param;
        const uint64_t maxPhotons = n * (uint64_t)maxPathLength;
        uint32_t size = (uint32_t)std::max<uint64_t>(1031, 4 * maxPhotons + 1);
        auto prime = [](uint32_t v) {
            if (v < 2) return false;
            for (uint32_t d = 2; (uint64_t)d * d <= v; ++d)
                if (v % d == 0) return false;
            return true;
        };
        while (!prime(size)) ++size;
        std::vector<uvec2> map(size, uvec2(0xffffffffu, 0xffffffffu));
        std::vector<ivec4> data(2 * maxPhotons + 2);
        ref_pmd::HashMap = ref_pmg::HashMap = map.data();
        ref_pmd::HashMapData = ref_pmg::HashMapData = data.data();
        ref_pmd::HashMapCounter = ref_pmg::HashMapCounter = 0;
        for (auto* u : {&ref_pmd::HashMapSize, &ref_pmg::HashMapSize}) *u = size;
        ref_pmd::NumPhotonsPerLightSample = ref_pmg::NumPhotonsPerLightSample = raysPerLightSample;
        ref_pmd::HashGridSpacing = ref_pmg::HashGridSpacing = radius * 2.01f;
        ref_pmd::PhotonQueryRadiusSq = ref_pmg::PhotonQueryRadiusSq = radius * radius;
        for (uint64_t i = 0; i < n; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            ref_pmd::PhotonDistributionMain();
        }
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
                ref_pmg::PhotonGatherMain();
            }
    } else if (bidir == 2) {  // WhittedRayTracer::Draw: whittedraytracer.comp per pixel
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
                ref_wh::WhittedMain();
            }
    } else if (!bidir) {
        ref_lt::NumRaysPerLightSample = raysPerLightSample;
        for (uint64_t i = 0; i < n; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            ref_lt::LighttracerMain();
        }
        for (int i = 0; i < numLightSamples; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            ref_slc::ShowLightCachesMain();
        }
    } else {
        // BidirectionalPathtracer::Draw: resetcounter.comp, the light pass
        // filling the cache, then the eye pass per pixel. The capacity is the
        // worst case (every light path stores at most maxPathLength + 1
        // entries) instead of the warm-up estimate, so nothing is dropped.
        std::vector<ref_bpl::LightCacheEntry> cache(n * (uint64_t)(maxPathLength + 1));
        ref_bpl::LightCacheEntries = cache.data();
        ref_bpl::NumRaysPerLightSample = raysPerLightSample;
        ref_bpl::LightRayPixelWeight = 2.0f * 3.14159265358979f / (float)raysPerLightSample;
        ref_bpl::LightCacheCapacity = (int)cache.size();
        ref_bpl::AverageLightPathLength = 1;
        ref_bpl::NumLightCacheEntries = raysPerLightSample * numLightSamples;  // resetcounter.comp
        ref_bpl::LightPathLengthSum = 0;
        for (uint64_t i = 0; i < n; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            ref_bpl::BidirLightMain();
        }
        ref_bpe::LightCacheEntries = reinterpret_cast<ref_bpe::LightCacheEntry*>(cache.data());
        ref_bpe::NumLightCacheEntries = std::min<int>(ref_bpl::NumLightCacheEntries, (int)cache.size());
        ref_bpe::NumRaysPerLightSample = raysPerLightSample;
        ref_bpe::LightRayPixelWeight = ref_bpl::LightRayPixelWeight;
        ref_bpe::LightCacheCapacity = (int)cache.size();
        ref_bpe::AverageLightPathLength = 1;
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
                ref_bpe::BidirEyeMain();
            }
    }
    g_textureColours = nullptr;
    return 0;
}

// One iteration of hierarchypathtracer.comp (the shader's own
// MAX_PATHLENGTH 4) per pixel in order: importance (RG32F, two floats per
// node), the hierarchy materials (RGBA16F, six texels per inner node, as
// halves) and the node NDFs (RG16, three texels per inner node) as the
// renderer binds them (hierarchyimportance.cpp:34-68).
int ref_render_hier(const float* hierarchy, const int32_t* slots, const float* positions, const float* vertexInfo,
                    const float* materials, int numMaterials, int width, int height, const float* cam,
                    uint32_t frameSeed, const float* lightSamples, int numLightSamples, const float* sky,
                    const float* importance, const uint16_t* hierMaterialHalves, uint64_t numHierMaterialHalves,
                    const uint16_t* sggx, uint64_t numSggx, float* accum) {
    using namespace glslref;
    if (numMaterials > 256) return 1;
    namespace P = ref_hpt;
    std::vector<vec4> colours(4 * (size_t)numMaterials);
    for (int m = 0; m < numMaterials; ++m) {
        const float* r = materials + 24 * (size_t)m;
        colours[4 * m + 0] = vec4(r[0], r[1], r[2], 1.0f);
        colours[4 * m + 1] = vec4(r[4], r[5], r[6], 1.0f);
        colours[4 * m + 2] = vec4(r[8], r[9], r[10], r[11]);
        colours[4 * m + 3] = vec4(r[12], r[13], r[14], 1.0f);
        P::Material& M = P::Materials[m];
        M.diffuseTexHandle = uvec2(4 * m + 0, 0);
        M.opacityTexHandle = uvec2(4 * m + 1, 0);
        M.reflectivenessTexHandle = uvec2(4 * m + 2, 0);
        M.emissivityTexHandle = uvec2(4 * m + 3, 0);
        M.Fresnel0 = vec3(r[16], r[17], r[18]);
        M.RefractionIndexAvg = r[3];
        M.Fresnel1 = vec3(r[20], r[21], r[22]);
    }
    g_textureColours = colours.data();
    // the texture units' conversions: half to float (exact), unorm16 to float (c / 65535)
    auto half = [](uint16_t h) {
        const uint32_t sign = (uint32_t)(h >> 15) << 31, e = (h >> 10) & 31u, m = h & 1023u;
        uint32_t bits;
        if (e == 0) {
            if (m == 0) {
                bits = sign;
            } else {  // subnormal: normalise
                int k = -1;
                uint32_t mm = m;
                do {
                    ++k;
                    mm <<= 1;
                } while (!(mm & 1024u));
                bits = sign | ((uint32_t)(127 - 15 - k) << 23) | ((mm & 1023u) << 13);
            }
        } else if (e == 31) {
            bits = sign | 0x7F800000u | (m << 13);
        } else {
            bits = sign | ((e + 112u) << 23) | (m << 13);
        }
        float f;
        std::memcpy(&f, &bits, 4);
        return f;
    };
    std::vector<float> matTexels(numHierMaterialHalves), ndf(numSggx);
    for (uint64_t i = 0; i < numHierMaterialHalves; ++i) matTexels[i] = half(hierMaterialHalves[i]);
    for (uint64_t i = 0; i < numSggx; ++i) ndf[i] = (float)sggx[i] / 65535.0f;
    P::HierachyBuffer = samplerBuffer{hierarchy, 4};
    P::TriangleBuffer = isamplerBuffer{reinterpret_cast<const ivec4*>(slots)};
    P::VertexPositionBuffer = samplerBuffer{positions, 3};
    P::VertexInfoBuffer = samplerBuffer{vertexInfo, 4};
    P::InitialLightSampleBuffer = samplerBuffer{lightSamples, 4};
    P::HierarchyImportanceBuffer = samplerBuffer{importance, 2};
    P::HierarchyMaterialBuffer = samplerBuffer{matTexels.data(), 4};
    P::SGGXBuffer = samplerBuffer{ndf.data(), 2};
    P::BackbufferSize = ivec2(width, height);
    P::NumInitialLightSamples = numLightSamples;
    P::CameraU = vec3(cam[0], cam[1], cam[2]);
    P::CameraV = vec3(cam[3], cam[4], cam[5]);
    P::CameraW = vec3(cam[6], cam[7], cam[8]);
    P::CameraPosition = vec3(cam[9], cam[10], cam[11]);
    P::PixelArea = cam[12];
    P::FrameSeed = frameSeed;
    P::IterationCount = 0;
    P::EnvironmentMap.colour = vec3(sky[0], sky[1], sky[2]);
    P::OutputTexture = image2D{reinterpret_cast<vec4*>(accum), width, height};
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
            P::HierarchyPathtracerMain();
        }
    g_textureColours = nullptr;
    return 0;
}

}  // extern "C"

namespace {
// Parent of every inner node (the scene's parent buffer, an R32I texture
// buffer the propagation and material passes read through a float view):
// both children of a binary node point at it; the root points at itself.
std::vector<float> ParentPointers(const float* hierarchy, int numNodes) {
    std::vector<float> parent((size_t)numNodes);
    auto put = [&](int i, int32_t v) { std::memcpy(&parent[(size_t)i], &v, 4); };
    if (numNodes > 0) put(0, 0);
    for (int i = 0; i < numNodes; ++i) {
        uint32_t child;
        std::memcpy(&child, hierarchy + 8 * (size_t)i + 3, 4);
        if (child & 0x80000000u) continue;
        int32_t second;
        std::memcpy(&second, hierarchy + 8 * (size_t)child + 7, 4);
        put((int)child, i);
        if (second > 0 && second < numNodes) put(second, i);
    }
    return parent;
}
// Number of tree levels (ComputeHierarchyMaterials runs pullmaterials.comp
// once per level): one more than the deepest inner node's depth.
int TreeLevels(const float* hierarchy, int numNodes) {
    std::vector<int> depth((size_t)numNodes, 0);
    int levels = numNodes > 0 ? 1 : 0;
    for (int i = 0; i < numNodes; ++i) {  // parents precede their children
        uint32_t child;
        std::memcpy(&child, hierarchy + 8 * (size_t)i + 3, 4);
        if (child & 0x80000000u) continue;
        int32_t second;
        std::memcpy(&second, hierarchy + 8 * (size_t)child + 7, 4);
        depth[child] = depth[i] + 1;
        if (second > 0 && second < numNodes) depth[second] = depth[i] + 1;
        levels = std::max(levels, depth[i] + 2);
    }
    return levels;
}
void BindConstantMaterials(std::vector<glslref::vec4>& colours, const float* materials, int numMaterials) {
    using namespace glslref;
    colours.assign(4 * (size_t)numMaterials, vec4());
    for (int m = 0; m < numMaterials; ++m) {
        const float* r = materials + 24 * (size_t)m;
        colours[4 * m + 0] = vec4(r[0], r[1], r[2], 1.0f);
        colours[4 * m + 1] = vec4(r[4], r[5], r[6], 1.0f);
        colours[4 * m + 2] = vec4(r[8], r[9], r[10], r[11]);
        colours[4 * m + 3] = vec4(r[12], r[13], r[14], 1.0f);
    }
    g_textureColours = colours.data();
}
template <class M>
void BindMaterial(M& mat, int m, const float* materials) {
    using namespace glslref;
    const float* r = materials + 24 * (size_t)m;
    mat.diffuseTexHandle = uvec2(4 * m + 0, 0);
    mat.opacityTexHandle = uvec2(4 * m + 1, 0);
    mat.reflectivenessTexHandle = uvec2(4 * m + 2, 0);
    mat.emissivityTexHandle = uvec2(4 * m + 3, 0);
    mat.Fresnel0 = vec3(r[16], r[17], r[18]);
    mat.RefractionIndexAvg = r[3];
    mat.Fresnel1 = vec3(r[20], r[21], r[22]);
}
}  // namespace

extern "C" {

// HierarchyImportance::Draw's importance pass (hierarchyimportance.cpp:
// 87-108, 119-152): `iterations` runs of acquisition2.comp over every pixel
// (NumImportanceIterations = 1..iterations), then
// hierarchypropagation_init.comp over the inner nodes and
// hierarchypropagation_nodes.comp until no node changes. Invocations run in
// order on one thread. imp: {x, y} per inner node, then per leaf slot;
// subtree: per inner node.
int ref_hier_importance(const float* hierarchy, int numNodes, const int32_t* slots, int numSlots,
                        const float* positions, const float* vertexInfo, const float* materials, int numMaterials,
                        int width, int height, const float* cam, const float* lightSamples, int numLightSamples,
                        int iterations, float* imp, float* subtree) {
    using namespace glslref;
    if (numMaterials > 256 || iterations < 1) return 1;
    std::vector<vec4> colours;
    BindConstantMaterials(colours, materials, numMaterials);
    for (int m = 0; m < numMaterials; ++m) BindMaterial(ref_acq::Materials[m], m, materials);
    std::vector<float> parent = ParentPointers(hierarchy, numNodes);
    std::fill(imp, imp + 2 * ((size_t)numNodes + numSlots), 0.0f);
    std::fill(subtree, subtree + numNodes, 0.0f);
    namespace A = ref_acq;
    A::HierachyBuffer = samplerBuffer{hierarchy, 4};
    A::TriangleBuffer = isamplerBuffer{reinterpret_cast<const ivec4*>(slots)};
    A::VertexPositionBuffer = samplerBuffer{positions, 3};
    A::VertexInfoBuffer = samplerBuffer{vertexInfo, 4};
    A::InitialLightSampleBuffer = samplerBuffer{lightSamples, 4};
    A::BackbufferSize = ivec2(width, height);
    A::NumInitialLightSamples = numLightSamples;
    A::CameraU = vec3(cam[0], cam[1], cam[2]);
    A::CameraV = vec3(cam[3], cam[4], cam[5]);
    A::CameraW = vec3(cam[6], cam[7], cam[8]);
    A::CameraPosition = vec3(cam[9], cam[10], cam[11]);
    A::PixelArea = cam[12];
    A::HierarchyImportance = reinterpret_cast<vec2*>(imp);
    A::NumInnerNodes = numNodes;
    A::NumTriangles = numSlots;
    A::HierarchyBufferStride = 2;
    for (int it = 1; it <= iterations; ++it) {
        A::NumImportanceIterations = it;
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
                A::AcquisitionMain();
            }
    }
    namespace I = ref_pinit;
    namespace N = ref_pnodes;
    I::HierachyBuffer = N::HierachyBuffer = samplerBuffer{hierarchy, 4};
    I::HierarchyImportance = N::HierarchyImportance = reinterpret_cast<vec2*>(imp);
    I::SubtreeImportance = N::SubtreeImportance = subtree;
    I::ParentPointerBuffer = N::ParentPointerBuffer = samplerBuffer{parent.data(), 1};
    I::NumInnerNodes = N::NumInnerNodes = numNodes;
    I::NumTriangles = N::NumTriangles = numSlots;
    I::NumImportanceIterations = N::NumImportanceIterations = iterations;
    I::HierarchyBufferStride = N::HierarchyBufferStride = 2;
    for (int i = 0; i < numNodes; ++i) {
        gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
        I::PropagationInitMain();
    }
    int passes = 0;
    do {
        N::ChangedAnything = 0;
        for (int i = 0; i < numNodes; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            N::PropagationNodesMain();
        }
        if (++passes > numNodes + 1) return 2;  // no convergence: a malformed tree
    } while (N::ChangedAnything != 0);
    g_textureColours = nullptr;
    return 0;
}

// HierarchyImportance::ComputeHierarchyMaterials (hierarchyimportance.cpp:
// 154-181): sampleleafmaterials.comp over the inner nodes, then
// pullmaterials.comp once per tree level. out: six uvec2 per inner node.
int ref_hier_materials(const float* hierarchy, int numNodes, const int32_t* slots, const float* positions,
                       const float* vertexInfo, const float* materials, int numMaterials, uint32_t* out) {
    using namespace glslref;
    if (numMaterials > 256) return 1;
    std::vector<vec4> colours;
    BindConstantMaterials(colours, materials, numMaterials);
    for (int m = 0; m < numMaterials; ++m) BindMaterial(ref_leafm::Materials[m], m, materials);
    std::vector<float> parent = ParentPointers(hierarchy, numNodes);
    std::fill(out, out + 12 * (size_t)numNodes, 0u);
    namespace L = ref_leafm;
    namespace U = ref_pullm;
    L::HierachyBuffer = U::HierachyBuffer = samplerBuffer{hierarchy, 4};
    L::TriangleBuffer = isamplerBuffer{reinterpret_cast<const ivec4*>(slots)};
    L::VertexPositionBuffer = samplerBuffer{positions, 3};
    L::VertexInfoBuffer = samplerBuffer{vertexInfo, 4};
    L::hierarchyMaterial = reinterpret_cast<L::HierarchyMaterial*>(out);
    U::hierarchyMaterial = reinterpret_cast<U::HierarchyMaterial*>(out);
    static_assert(sizeof(L::HierarchyMaterial) == 48 && sizeof(U::HierarchyMaterial) == 48, "six uvec2 per node");
    U::ParentPointerBuffer = samplerBuffer{parent.data(), 1};
    L::NumInnerNodes = U::NumInnerNodes = numNodes;
    L::HierarchyBufferStride = U::HierarchyBufferStride = 2;
    for (int i = 0; i < numNodes; ++i) {
        gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
        L::SampleLeafMaterialsMain();
    }
    const int levels = TreeLevels(hierarchy, numNodes);
    for (int pass = 0; pass < levels; ++pass)
        for (int i = 0; i < numNodes; ++i) {
            gl_GlobalInvocationID = uvec3((uint)i, 0u, 0u);
            U::PullMaterialsMain();
        }
    g_textureColours = nullptr;
    return 0;
}

}  // extern "C"
