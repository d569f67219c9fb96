/* gpugi_bvhmake.h — C ABI of the offline BVH builder (host-only C++).
 *
 * This library stands in for gpugi's `bvhmake` tool: it builds the
 * stackless escape-pointer hierarchy and the fixed-size leaf blocks that the
 * traversal kernels consume, and reads/writes bvhmake's NamedArray file.
 *
 *   gpugi_bvh_build       replaces BVHBuilder::BuildBVH        (bvhmake/bvhbuilder.cpp:526-555)
 *                         with BuildSweep/BuildKdtree/BuildLDS  (bvhmake/buildmethods/sweep.cpp:27-259,
 *                                                                bvhmake/buildmethods/kdtree.cpp:9-157,
 *                                                                bvhmake/buildmethods/lds.cpp:11-164)
 *                         and FitBox/FitEllipsoid               (bvhmake/fitmethods/aaboxfit.cpp:5-33,
 *                                                                bvhmake/fitmethods/aaellipsoidfit.cpp:6-79)
 *   gpugi_bvh_export      replaces BVHBuilder::ExportBVH + ExportTriangles + the
 *                         node repacking of Scene::UploadHierarchy
 *                                                               (bvhmake/bvhbuilder.cpp:569-612,710-722;
 *                                                                gpugi/scene/scene.cpp:92-106)
 *   gpugi_bvh_write_file  replaces the NamedArray export of bvhmake's main
 *   gpugi_bvh_read_file                                         (bvhmake/main.cpp:27-146,
 *                                                                documentation/fileformat.tex)
 *   gpugi_bvh_sggx        replaces ComputeSGGXBases + BVHBuilder::ExportApproximation
 *                                                               (bvhmake/processing/approx_sggx.cpp:88-203,
 *                                                                bvhmake/bvhbuilder.cpp:557-567)
 *
 * Conventions: 0 = OK, negative = error (see gpugi_bvh_last_error). The
 * caller owns every array passed in; the handle owns the built tree.
 */
#ifndef GPUGI_BVHMAKE_H
#define GPUGI_BVHMAKE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gpugi_bvh gpugi_bvh;

enum gpugi_build_method { GPUGI_BUILD_KDTREE = 0, GPUGI_BUILD_SWEEP = 1, GPUGI_BUILD_LDS = 2 };
/* GPUGI_FIT_OBOX (an addition; bvhmake fits boxes and ellipsoids only):
 * oriented boxes, the nodes of the reference's OBOX_BVH walk, fitted bottom
 * up along the principal axes of each node's points. */
enum gpugi_fit_method { GPUGI_FIT_AABOX = 0, GPUGI_FIT_ELLIPSOID = 1, GPUGI_FIT_OBOX = 2 };

/* Build a hierarchy over `numTriangles` triangles, each 4 uint32
 * {v0, v1, v2, material}, indexing `positions` (3 floats per vertex).
 * leafSize is the number of triangle slots per leaf block (bvhmake: 8).
 * seed drives the ellipsoid fit's particle swarm (the reference leaves it
 * uninitialised, bvhmake/fitmethods/optimize.inl:158). */
int gpugi_bvh_build(const float* positions, uint32_t numVertices, const uint32_t* triangles,
                    uint32_t numTriangles, uint32_t buildMethod, uint32_t fitMethod,
                    uint32_t leafSize, uint64_t seed, gpugi_bvh** out);

/* Sizes of the built hierarchy. boundsKind: 0 = AABB, 1 = ellipsoid, 2 = oriented box. */
int gpugi_bvh_info(const gpugi_bvh* bvh, uint32_t* numNodes, uint32_t* numLeafBlocks,
                   uint32_t* leafSize, uint32_t* boundsKind, uint32_t* maxDepth);

/* Export in the GPU layout of Scene::TreeNode<Box> (gpugi/scene/scene.hpp:30-38):
 * 8 floats per node {min.xyz, firstChild bits, max.xyz, escape bits}
 * (ellipsoid: {center.xyz, firstChild, radii.xyz, escape}; oriented box:
 * 12 floats, Scene::TreeNode<OBox> (scene.hpp:40-49) {center.xyz, firstChild,
 * sidesHalf.xyz, escape, rotationInv quaternion x, y, z, w}), leafSize
 * int32x4 slots per leaf block {v0, v1, v2, material}, invalid = {0,0,0,0},
 * and optionally the parent index of every node (may be NULL). */
int gpugi_bvh_export(const gpugi_bvh* bvh, float* hierarchy, int32_t* slots, uint32_t* parents);

/* Write/read bvhmake's NamedArray file ("vertices", "triangles",
 * "hierarchy", "bounding_aabox"/"bounding_ellipsoid"). The reader returns a
 * handle usable with gpugi_bvh_info/gpugi_bvh_export and fills the vertex
 * positions through gpugi_bvh_vertices. */
int gpugi_bvh_write_file(const gpugi_bvh* bvh, const char* path);
int gpugi_bvh_read_file(const char* path, gpugi_bvh** out);
int gpugi_bvh_vertices(const gpugi_bvh* bvh, uint32_t* numVertices, float* positions /* may be NULL */);

/* Per-vertex normal (3 floats) and texture coordinate (2 floats) of the
 * "vertices" chunk's 32-byte records {position, normal, texcoord}
 * (bvhmake/filedef.hpp:15-20). Set before gpugi_bvh_write_file (either
 * array may be NULL: zeros are written); read after gpugi_bvh_read_file. */
int gpugi_bvh_set_vertex_attributes(gpugi_bvh* bvh, const float* normals, const float* texcoords);
int gpugi_bvh_vertex_attributes(const gpugi_bvh* bvh, float* normals, float* texcoords);

/* Node NDFs ("approx_sggx" chunk, FileDecl::SGGX of bvhmake/filedef.hpp:
 * 79-95): 6 uint16 per node {sigma.xyz, r.xyz}; sigma = sqrt(S_ii) as
 * unorm16, r = S_ij / sqrt(S_ii S_jj) mapped to [0, 65534] (S_xy, S_xz,
 * S_yz), S the node's SGGX matrix fitted to the vertex normals below it.
 * Computed from the vertex normals (gpugi_bvh_set_vertex_attributes) on
 * first use, or taken from a file's chunk; gpugi_bvh_write_file writes the
 * chunk whenever normals or NDFs are present, as bvhmake does. */
int gpugi_bvh_sggx(const gpugi_bvh* bvh, uint16_t* out);

/* Material records carried in an extra "gpugi_materials" chunk (24 floats
 * each, the gpugi_material layout of gpugi_cuda.h). No counterpart in the
 * reference, which keeps materials in the scene's JSON next to the file;
 * readers that do not know the chunk skip it, as the format allows. */
int gpugi_bvh_set_materials(gpugi_bvh* bvh, const float* records, uint32_t numMaterials);
int gpugi_bvh_materials(const gpugi_bvh* bvh, uint32_t* numMaterials, float* records /* may be NULL */);

/* Material names of the "materialref" chunk (32-byte names, the order of the
 * triangles' material indices; bvhbuilder.cpp:622-630). Set before writing;
 * after reading, name i is returned (NULL past the end). */
int gpugi_bvh_set_material_names(gpugi_bvh* bvh, const char* const* names, uint32_t numNames);
const char* gpugi_bvh_material_name(const gpugi_bvh* bvh, uint32_t index);
uint32_t gpugi_bvh_num_material_names(const gpugi_bvh* bvh);

/* Material records (24 floats each, the gpugi_material layout) for the named
 * materials of a scene JSON's "materials" object, with the parameter mapping
 * and defaults of Scene::LoadMaterial (gpugi/scene/scene.cpp:132-180).
 * 0 = OK; negative: parse error, missing material or a texture reference
 * (see gpugi_materials_json_error). */
int gpugi_materials_from_json(const char* json, const char* const* names, uint32_t numNames, float* records);
const char* gpugi_materials_json_error(void);

void gpugi_bvh_free(gpugi_bvh* bvh);
const char* gpugi_bvh_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
