// Scene upload: validation of the escape tree, repacking of leaf children,
// and the per-slot triangle precompute (p0, e0, e1, n) on the device.
//
// Replaces Scene::UploadGeometry / UploadHierarchy (gpugi/scene/scene.cpp:
// 75-130) for the CUDA path.
#include <cstring>

#include "ctx.cuh"

namespace gpugi {

// Precompute each valid slot's triangle record with the operation order of
// IntersectTriangle (intersectiontests.glsl:66-68).
__global__ void k_prepare_triangles(const int4* __restrict__ slots, uint32_t numSlots,
                                    const float* __restrict__ pos, float4* __restrict__ tris) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numSlots) return;
    int4 s = slots[i];
    float4 a = make_float4(0, 0, 0, 0), b = a, c = a;
    if (s.x != s.y) {
        float3 p0 = make_float3(pos[3 * (size_t)s.x], pos[3 * (size_t)s.x + 1], pos[3 * (size_t)s.x + 2]);
        float3 p1 = make_float3(pos[3 * (size_t)s.y], pos[3 * (size_t)s.y + 1], pos[3 * (size_t)s.y + 2]);
        float3 p2 = make_float3(pos[3 * (size_t)s.z], pos[3 * (size_t)s.z + 1], pos[3 * (size_t)s.z + 2]);
        float3 e0 = X::sub3(p1, p0);
        float3 e1 = X::sub3(p0, p2);
        float3 n = X::cross(e1, e0);
        a = make_float4(p0.x, p0.y, p0.z, e0.x);
        b = make_float4(e0.y, e0.z, e1.x, e1.y);
        c = make_float4(e1.z, n.x, n.y, n.z);
    }
    tris[3 * (size_t)i] = a;
    tris[3 * (size_t)i + 1] = b;
    tris[3 * (size_t)i + 2] = c;
}

// Records of the watertight test: the exact vertices of each valid slot,
// {p0.xyz p1.x | p1.yz p2.xy | p2.z 0 0 0}; invalid slots stay zero.
__global__ void k_prepare_wt_triangles(const int4* __restrict__ slots, uint32_t numSlots,
                                       const float* __restrict__ pos, float4* __restrict__ tris) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= numSlots) return;
    int4 s = slots[i];
    float4 a = make_float4(0, 0, 0, 0), b = a, c = a;
    if (s.x != s.y) {
        const float* p0 = pos + 3 * (size_t)s.x;
        const float* p1 = pos + 3 * (size_t)s.y;
        const float* p2 = pos + 3 * (size_t)s.z;
        a = make_float4(p0[0], p0[1], p0[2], p1[0]);
        b = make_float4(p1[1], p1[2], p2[0], p2[1]);
        c = make_float4(p2[2], 0.0f, 0.0f, 0.0f);
    }
    tris[3 * (size_t)i] = a;
    tris[3 * (size_t)i + 1] = b;
    tris[3 * (size_t)i + 2] = c;
}

void prepare_triangles(cudaStream_t stream, const int4* slots, uint32_t numSlots, const float* positions,
                       float4* tris) {
    if (numSlots) k_prepare_triangles<<<(numSlots + 255) / 256, 256, 0, stream>>>(slots, numSlots, positions, tris);
}

static uint32_t bits_of(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// Device node order: the nodes of the top tree levels first, breadth first
// (as many whole levels as fit in maxTop), then every other node in its
// original preorder. Child and escape words are renumbered; leaf words are
// kept. The walk visits the same logical nodes in the same order, only their
// addresses change. Returns the number of leading (top) nodes.
static uint32_t relayout_nodes(std::vector<float>& nodes, uint32_t numNodes, uint32_t maxTop,
                               std::vector<uint32_t>& mapOut) {
    std::vector<uint32_t> depth(numNodes, 0);
    uint32_t maxDepth = 0;
    for (uint32_t i = 0; i < numNodes; ++i) {  // preorder: parents precede children
        const uint32_t child = bits_of(nodes[8 * (size_t)i + 3]);
        if (child & LEAF_FLAG) continue;
        const uint32_t right = bits_of(nodes[8 * (size_t)child + 7]);
        depth[child] = depth[right] = depth[i] + 1;
        maxDepth = std::max(maxDepth, depth[i] + 1);
    }
    std::vector<uint32_t> perLevel(maxDepth + 2, 0);
    for (uint32_t d : depth) ++perLevel[d];
    uint32_t levels = 0, top = 0;
    while (levels <= maxDepth && top + perLevel[levels] <= maxTop) top += perLevel[levels++];
    if (top <= 1) return 0;  // nothing worth staging: keep the original order
    std::vector<uint32_t> map(numNodes, UINT32_MAX);
    uint32_t next = 0;
    std::vector<uint32_t> queue{0};
    for (size_t q = 0; q < queue.size(); ++q) {  // breadth first over the top levels, siblings adjacent
        const uint32_t i = queue[q];
        map[i] = next++;
        const uint32_t child = bits_of(nodes[8 * (size_t)i + 3]);
        if ((child & LEAF_FLAG) || depth[i] + 1 >= levels) continue;
        queue.push_back(child);
        queue.push_back(bits_of(nodes[8 * (size_t)child + 7]));
    }
    for (uint32_t i = 0; i < numNodes; ++i)
        if (map[i] == UINT32_MAX) map[i] = next++;
    std::vector<float> out(nodes.size());
    for (uint32_t i = 0; i < numNodes; ++i) {
        float* o = &out[8 * (size_t)map[i]];
        std::memcpy(o, &nodes[8 * (size_t)i], 8 * sizeof(float));
        const uint32_t child = bits_of(nodes[8 * (size_t)i + 3]);
        const uint32_t esc = bits_of(nodes[8 * (size_t)i + 7]);
        const uint32_t nc = (child & LEAF_FLAG) ? child : map[child];
        const uint32_t ne = esc ? map[esc] : 0u;
        std::memcpy(&o[3], &nc, 4);
        std::memcpy(&o[7], &ne, 4);
    }
    nodes.swap(out);
    mapOut.swap(map);
    return top;
}

template <typename T>
static gpugi_status upload(gpugi_ctx* ctx, gpugi_scene* sc, const T* host, size_t count, const T** dst) {
    *dst = nullptr;
    if (count == 0) return GPUGI_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "cudaMalloc failed for scene buffer");
    sc->allocations.push_back(p);
    if (host) {
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    } else {
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(p, 0, count * sizeof(T), ctx->stream));
    }
    *dst = static_cast<const T*>(p);
    return GPUGI_OK;
}

}  // namespace gpugi

using namespace gpugi;

extern "C" gpugi_status gpugi_scene_upload(gpugi_ctx* ctx, const float* hierarchy, uint32_t numNodes,
                                           uint32_t boundsKind, const int32_t* slots, uint32_t numSlots,
                                           uint32_t leafSize, const float* positions, const float* vertexInfo,
                                           uint32_t numVertices, const gpugi_material* materials,
                                           uint32_t numMaterials, gpugi_scene** out) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!out) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!hierarchy || !slots || !positions || numNodes == 0 || numSlots == 0 || numVertices == 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "empty scene: hierarchy, slots and positions are required");
    if (boundsKind > GPUGI_BOUNDS_OBOX) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown bounds kind");
    const size_t nf = boundsKind == GPUGI_BOUNDS_OBOX ? 12 : 8;  // floats per node
    if (leafSize == 0 || leafSize > 32 || numSlots % leafSize != 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "leafSize must be in [1, 32] and divide numSlots");
    if (numNodes >= 0x80000000u) return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "too many nodes");
    if (numMaterials > 0 && !materials) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "materials is NULL");
    const uint32_t numBlocks = numSlots / leafSize;
    if (numBlocks > LEAF_BLOCK_MASK + 1u) return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "too many leaf blocks");

    // Leaf slots: indices in range; count the leading valid slots per block.
    std::vector<uint32_t> counts(numBlocks, 0);
    for (uint32_t blk = 0; blk < numBlocks; ++blk) {
        uint32_t c = 0;
        bool ended = false;
        for (uint32_t k = 0; k < leafSize; ++k) {
            const int32_t* s = slots + 4 * ((size_t)blk * leafSize + k);
            if (s[0] == s[1]) {
                ended = true;
                continue;
            }
            if (s[0] < 0 || s[1] < 0 || s[2] < 0 || (uint32_t)s[0] >= numVertices || (uint32_t)s[1] >= numVertices ||
                (uint32_t)s[2] >= numVertices)
                return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "leaf slot references a vertex out of range");
            if (numMaterials > 0 && (s[3] < 0 || (uint32_t)s[3] >= numMaterials))
                return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "leaf slot references a material out of range");
            if (!ended) ++c;
        }
        counts[blk] = c;
    }
    // Escape tree: children and escapes point strictly forward (preorder), so
    // every walk terminates within numNodes steps and stays in bounds.
    std::vector<float> nodes(hierarchy, hierarchy + nf * (size_t)numNodes);
    for (uint32_t i = 0; i < numNodes; ++i) {
        uint32_t child = bits_of(hierarchy[nf * i + 3]);
        uint32_t esc = bits_of(hierarchy[nf * i + 7]);
        if (child & LEAF_FLAG) {
            uint32_t blk = child & 0x7FFFFFFFu;
            if (blk >= numBlocks) return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "leaf block index out of range");
            uint32_t enc = LEAF_FLAG | (counts[blk] << LEAF_COUNT_SHIFT) | blk;
            std::memcpy(&nodes[nf * i + 3], &enc, 4);
        } else if (child <= i || child >= numNodes) {
            return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "firstChild must point forward to a node (preorder)");
        }
        if (esc != 0 && (esc <= i || esc >= numNodes))
            return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "escape must be 0 or point forward (preorder)");
    }

    std::vector<uint32_t> nodeMap;  // uploaded index -> device index (empty: the same)
    // oriented-box nodes keep the preorder layout (no top-level staging)
    const uint32_t topNodes =
        boundsKind == GPUGI_BOUNDS_OBOX ? 0u : relayout_nodes(nodes, numNodes, ctx->sharedNodes, nodeMap);
    // Ellipsoid nodes travel as {center, firstChild}, {1 / (radii + 1e-15), escape}:
    // the node test then multiplies where the virtual-ellipsoid arithmetic
    // divides (the guard is the shader's, intersectiontests.glsl:29).
    std::vector<float> hostRadii;
    if (boundsKind == GPUGI_BOUNDS_ELLIPSOID) {
        hostRadii.resize(3 * (size_t)numNodes);
        for (size_t i = 0; i < numNodes; ++i)
            for (int c = 0; c < 3; ++c) {
                float& r = nodes[8 * i + 4 + c];
                hostRadii[3 * i + c] = r;
                r = 1.0f / (r + 1e-15f);
            }
    }

    cudaError_t se = cudaSetDevice(ctx->device);
    if (se != cudaSuccess) return cuda_fail(ctx, se, "cudaSetDevice");
    gpugi_scene* sc = new gpugi_scene();
    attach_child(ctx, &sc->ctx);
    sc->numLeafBlocks = numBlocks;
    auto cleanup = [&](gpugi_status st) {
        gpugi_scene_destroy(sc);
        return st;
    };
    gpugi_status st;
    const float4* dNodes;
    if ((st = upload(ctx, sc, reinterpret_cast<const float4*>(nodes.data()), nf / 4 * (size_t)numNodes, &dNodes)))
        return cleanup(st);
    const int4* dSlots;
    if ((st = upload(ctx, sc, reinterpret_cast<const int4*>(slots), numSlots, &dSlots))) return cleanup(st);
    const float* dPos;
    if ((st = upload(ctx, sc, positions, 3 * (size_t)numVertices, &dPos))) return cleanup(st);
    const float4* dInfo;
    if ((st = upload(ctx, sc, reinterpret_cast<const float4*>(vertexInfo), numVertices, &dInfo)))
        return cleanup(st);
    const float4* dMat = nullptr;
    if (numMaterials > 0 &&
        (st = upload(ctx, sc, reinterpret_cast<const float4*>(materials), 6 * (size_t)numMaterials, &dMat)))
        return cleanup(st);
    const float4* dTris;
    if ((st = upload<float4>(ctx, sc, nullptr, 3 * (size_t)numSlots, &dTris))) return cleanup(st);
    k_prepare_triangles<<<(numSlots + 255) / 256, 256, 0, ctx->stream>>>(dSlots, numSlots, dPos,
                                                                         const_cast<float4*>(dTris));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "scene upload"));

    sc->dev.nodes = dNodes;
    sc->dev.tris = dTris;
    sc->dev.slots = dSlots;
    sc->dev.positions = dPos;
    sc->dev.vinfo = dInfo;
    sc->dev.materials = dMat;
    sc->dev.err = ctx->errWord;
    sc->dev.numNodes = numNodes;
    sc->numNodesUploaded = numNodes;
    sc->dev.numSlots = numSlots;
    sc->dev.leafSize = leafSize;
    sc->dev.boundsKind = boundsKind;
    sc->dev.numVertices = numVertices;
    sc->dev.numMaterials = numMaterials;
    sc->dev.topNodes = topNodes;
    sc->nodeMap.swap(nodeMap);
    sc->hostRadii.swap(hostRadii);
    sc->hostPositions.assign(positions, positions + 3 * (size_t)numVertices);
    sc->hostSlots.assign(slots, slots + 4 * (size_t)numSlots);
    if (numMaterials)
        sc->hostMaterials.assign(reinterpret_cast<const float*>(materials),
                                 reinterpret_cast<const float*>(materials) + 24 * (size_t)numMaterials);
    *out = sc;
    return GPUGI_OK;
}

extern "C" gpugi_status gpugi_scene_set_triangle_test(gpugi_ctx* ctx, gpugi_scene* sc, uint32_t test) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene is NULL");
    if (test > GPUGI_TRIANGLE_WATERTIGHT) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "unknown triangle test");
    if (test == GPUGI_TRIANGLE_WATERTIGHT && !sc->dev.wtris) {
        const uint32_t n = sc->dev.numSlots;
        const float4* w = nullptr;
        gpugi_status st = upload<float4>(ctx, sc, nullptr, 3 * (size_t)n, &w);
        if (st) return st;
        k_prepare_wt_triangles<<<(n + 255) / 256, 256, 0, ctx->stream>>>(sc->dev.slots, n, sc->dev.positions,
                                                                         const_cast<float4*>(w));
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        sc->dev.wtris = w;
    }
    sc->dev.triangleTest = test;
    return GPUGI_OK;
}

extern "C" gpugi_status gpugi_scene_set_textures(gpugi_ctx* ctx, gpugi_scene* sc, const gpugi_texture* textures,
                                                 uint32_t numTextures, const int32_t* materialTextures) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "scene is NULL");
    const uint32_t nm = sc->dev.numMaterials;
    if (numTextures && (!textures || !materialTextures))
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "textures and materialTextures are required");
    uint64_t texels = 0;
    for (uint32_t i = 0; i < numTextures; ++i) {
        const gpugi_texture& t = textures[i];
        if (t.width == 0 || t.height == 0 || !t.rgba || t.width > (1u << 16) || t.height > (1u << 16))
            return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "a texture needs RGBA texels and 1..65536 texels a side");
        texels += (uint64_t)t.width * t.height;
    }
    if (texels >= (1ull << 32)) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "more than 2^32 texels");
    for (uint64_t k = 0; numTextures && k < 4ull * nm; ++k)
        if (materialTextures[k] < -1 || materialTextures[k] >= (int64_t)numTextures)
            return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "material texture index out of range");
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // earlier passes may still read the old textures
    if (sc->texBlock) cudaFree(sc->texBlock);
    sc->texBlock = nullptr;
    sc->dev.texels = nullptr;
    sc->dev.texInfo = nullptr;
    sc->dev.matTex = nullptr;
    if (numTextures == 0) return GPUGI_OK;
    const size_t texBytes = 16 * (size_t)texels, infoBytes = 16 * (size_t)numTextures, mapBytes = 16 * (size_t)nm;
    const size_t infoAt = (texBytes + 255) & ~size_t(255), mapAt = (infoAt + infoBytes + 255) & ~size_t(255);
    if (cudaMalloc(&sc->texBlock, mapAt + mapBytes + 16) != cudaSuccess) {
        sc->texBlock = nullptr;
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "texture allocation failed");
    }
    char* base = static_cast<char*>(sc->texBlock);
    std::vector<uint32_t> info(4 * (size_t)numTextures);
    uint64_t at = 0;
    for (uint32_t i = 0; i < numTextures; ++i) {
        const size_t n = (size_t)textures[i].width * textures[i].height;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(base + 16 * at, textures[i].rgba, 16 * n, cudaMemcpyHostToDevice, ctx->stream));
        info[4 * i] = (uint32_t)at;
        info[4 * i + 1] = textures[i].width;
        info[4 * i + 2] = textures[i].height;
        info[4 * i + 3] = 0;
        at += n;
    }
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(base + infoAt, info.data(), infoBytes, cudaMemcpyHostToDevice, ctx->stream));
    if (nm)
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(base + mapAt, materialTextures, mapBytes, cudaMemcpyHostToDevice, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    sc->dev.texels = reinterpret_cast<const float4*>(base);
    sc->dev.texInfo = reinterpret_cast<const uint4*>(base + infoAt);
    sc->dev.matTex = nm ? reinterpret_cast<const int4*>(base + mapAt) : nullptr;
    return GPUGI_OK;
}

extern "C" void gpugi_scene_destroy(gpugi_scene* sc) {
    if (!sc) return;
    if (sc->ctx) cudaStreamSynchronize(sc->ctx->stream);
    detach_child(&sc->ctx);
    free_hierarchy(sc);
    if (sc->texBlock) cudaFree(sc->texBlock);
    for (void* p : sc->allocations) cudaFree(p);
    delete sc;
}

extern "C" gpugi_status gpugi_debug_limit_nodes(gpugi_scene* sc, uint32_t numNodes) {
    if (!sc) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (numNodes > sc->numNodesUploaded)
        return fail(sc->ctx, GPUGI_ERROR_INVALID_ARGUMENT, "the node limit can only be lowered");
    sc->dev.numNodes = numNodes ? numNodes : sc->numNodesUploaded;
    return GPUGI_OK;
}
