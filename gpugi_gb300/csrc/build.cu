// GPU hierarchy builder: a linear BVH (LBVH) in gpugi's escape-pointer layout.
//
// The reference builds its hierarchies on the host (bvhmake's BuildSweep /
// BuildKdtree, bvhmake/bvhbuilder.cpp:526-555); this builder produces the
// same layout on the device, so a scene goes from host triangle arrays to a
// traversable gpugi_scene without a host build:
//   * nodes in preorder with the root at 0, escape(left child) = right child,
//     escape(right child) = escape(parent), escape(root) = 0
//     (RecursiveWriteHierarchy, bvhbuilder.cpp:710-722);
//   * axis-aligned boxes over the triangles below (FitBox,
//     fitmethods/aaboxfit.cpp:5-33);
//   * leaves of at most leafSize triangles, one block of leafSize slots each,
//     padded with {0,0,0,0} (ExportTriangles, bvhbuilder.cpp:569-612).
// The tree is different from bvhmake's (Morton-order splits instead of SAH
// sweeps), so traversal results are compared against the oracle walking this
// same tree, and closest hits against brute force.
//
// Passes (all on the context stream):
//   1. box centres of the triangles, their bounds        k_centre_bounds
//   2. 63-bit Morton codes of the centres, radix sort     k_morton + cub
//      (stable: equal codes keep the input order)
//   3. binary radix tree over the sorted codes            k_radix_tree
//      (Karras, "Maximizing Parallelism in the Construction of BVHs,
//      Octrees, and k-d Trees", HPG 2012; equal codes are ordered by index)
//   4. subtrees of at most leafSize triangles become      k_mark_leaves + scan
//      leaves; leaf blocks are numbered in Morton order
//   5. child boxes and output subtree sizes, bottom up    k_bottom_up
//      (the second child to finish continues to the parent)
//   6. preorder index and escape of every output node     k_emit_nodes
//      from its path to the root
//   7. leaf blocks from the sorted triangles              k_emit_slots
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ctx.cuh"

namespace gpugi {
namespace lbvh {

constexpr uint32_t kLeafRef = 0x80000000u;  // radix-tree child: a sorted triangle position
constexpr uint32_t kRoot = 0xFFFFFFFFu;      // parent of the root
// Depth bound of the radix tree: the common prefix grows by at least one bit
// per level, and a prefix has at most 64 + 32 bits (code, then position).
// Walks towards the root stop there and raise DEVERR_BUILD.
constexpr int kMaxDepth = 100;

// Internal node of the radix tree over sorted positions [first, last].
struct Inner {
    uint32_t left, right, first, last;
};
// Per internal node: the boxes and output subtree sizes of its two children.
struct alignas(16) ChildRec {
    float lo[2][3], hi[2][3];
    uint32_t size[2];
    uint32_t pad[2];
};

GPUGI_D uint32_t ordered_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
GPUGI_D float from_ordered(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u); }

GPUGI_D void tri_box(const float* __restrict__ pos, uint4 t, float lo[3], float hi[3]) {
    const uint32_t v[3] = {t.x, t.y, t.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        lo[c] = hi[c] = pos[3 * (size_t)v[0] + c];
#pragma unroll
        for (int k = 1; k < 3; ++k) {
            const float p = pos[3 * (size_t)v[k] + c];
            lo[c] = fminf(lo[c], p);
            hi[c] = fmaxf(hi[c], p);
        }
    }
}

// bounds: 3 ordered minima then 3 ordered maxima of the triangle box centres.
__global__ void k_centre_bounds(const float* __restrict__ pos, const uint4* __restrict__ tris, uint32_t n,
                                uint32_t* bounds) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float a[3], b[3];
        tri_box(pos, tris[i], a, b);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float m = 0.5f * (a[c] + b[c]);
            lo[c] = fminf(lo[c], m);
            hi[c] = fmaxf(hi[c], m);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], off));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], off));
        }
    }
    if ((threadIdx.x & 31u) == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            atomicMin(bounds + c, ordered_bits(lo[c]));
            atomicMax(bounds + 3 + c, ordered_bits(hi[c]));
        }
    }
}

// bvhmake's input rules, checked before any kernel indexes with the
// triangles: bit 0 = vertex index out of range, bit 1 = v0 == v1 (the
// padding triangle), bit 2 = material out of range.
__global__ void k_validate(const uint4* __restrict__ tris, uint32_t n, uint32_t numVertices, uint32_t numMaterials,
                           uint32_t* bad) {
    uint32_t bits = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 t = tris[i];
        if (t.x >= numVertices || t.y >= numVertices || t.z >= numVertices) bits |= 1u;
        else if (t.x == t.y) bits |= 2u;
        if (numMaterials > 0 && t.w >= numMaterials) bits |= 4u;
    }
    bits = __reduce_or_sync(0xffffffffu, bits);
    if ((threadIdx.x & 31u) == 0 && bits) atomicOr(bad, bits);
}

// Triangles whose material emits (Emissivity, the fourth float4 of a
// gpugi_material record): flags for an order-preserving compaction.
__global__ void k_flag_emissive(const uint4* __restrict__ tris, uint32_t n, const float4* __restrict__ mats,
                                uint32_t* __restrict__ flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 e = __ldg(mats + 6 * (size_t)tris[i].w + 3);
        flag[i] = (e.x != 0.0f || e.y != 0.0f || e.z != 0.0f) ? 1u : 0u;
    }
}

__global__ void k_compact(const uint4* __restrict__ tris, uint32_t n, const uint32_t* __restrict__ flag,
                          const uint32_t* __restrict__ pos, uint4* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flag[i]) out[pos[i]] = tris[i];
}

// Spread the low 21 bits of v to every third bit of a 63-bit word.
GPUGI_D uint64_t spread3(uint32_t v) {
    uint64_t x = v & 0x1FFFFFu;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float* __restrict__ pos, const uint4* __restrict__ tris, uint32_t n,
                         const uint32_t* __restrict__ bounds, uint64_t* __restrict__ keys,
                         uint32_t* __restrict__ vals) {
    float base[3], scale[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        base[c] = from_ordered(bounds[c]);
        const float ext = from_ordered(bounds[3 + c]) - base[c];
        scale[c] = ext > 0.0f ? 2097152.0f / ext : 0.0f;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float a[3], b[3];
        tri_box(pos, tris[i], a, b);
        uint32_t q[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float u = fmaxf(0.0f, (0.5f * (a[c] + b[c]) - base[c]) * scale[c]);  // NaN -> 0
            q[c] = (uint32_t)fminf(u, 2097151.0f);
        }
        keys[i] = spread3(q[0]) << 2 | spread3(q[1]) << 1 | spread3(q[2]);
        vals[i] = i;
    }
}

// Common prefix length of sorted keys i and j (-1 outside [0, n)); equal keys
// continue with the prefix of their positions.
GPUGI_D int prefix(const uint64_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clzll(a ^ b);
}

__global__ void k_radix_tree(const uint64_t* __restrict__ keys, int n, Inner* __restrict__ inner,
                             uint32_t* __restrict__ parent) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n - 1) return;
    const int d = prefix(keys, n, i, i + 1) - prefix(keys, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = prefix(keys, n, i, i - d);
    int lmax = 2;
    while (prefix(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = prefix(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (prefix(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int split = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    Inner in;
    in.first = (uint32_t)first;
    in.last = (uint32_t)last;
    in.left = first == split ? (kLeafRef | (uint32_t)split) : (uint32_t)split;
    in.right = last == split + 1 ? (kLeafRef | (uint32_t)(split + 1)) : (uint32_t)(split + 1);
    inner[i] = in;
    if (!(in.left & kLeafRef)) parent[in.left] = (uint32_t)i;
    if (!(in.right & kLeafRef)) parent[in.right] = (uint32_t)i;
    if (i == 0) parent[0] = kRoot;
}

GPUGI_D void child_range(const Inner* __restrict__ inner, uint32_t c, uint32_t& first, uint32_t& count) {
    if (c & kLeafRef) {
        first = c & ~kLeafRef;
        count = 1;
    } else {
        first = inner[c].first;
        count = inner[c].last - inner[c].first + 1;
    }
}

// Output nodes: internal nodes over more than leafSize triangles (inner
// nodes) and their children over at most leafSize triangles (leaves). A
// leaf is flagged at its first sorted position with its triangle count.
__global__ void k_mark_leaves(const Inner* __restrict__ inner, uint32_t n, uint32_t leafSize,
                              uint32_t* __restrict__ flag, uint32_t* __restrict__ count,
                              uint32_t* __restrict__ numInner) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool isInner = i + 1 < n && inner[i].last - inner[i].first + 1 > leafSize;
    const unsigned mask = __ballot_sync(0xffffffffu, isInner);
    if ((threadIdx.x & 31u) == 0 && mask) atomicAdd(numInner, (uint32_t)__popc(mask));
    if (!isInner) return;
    const Inner in = inner[i];
    for (int side = 0; side < 2; ++side) {
        uint32_t f, c;
        child_range(inner, side ? in.right : in.left, f, c);
        if (c <= leafSize) {
            flag[f] = 1u;
            count[f] = c;
        }
    }
}

// Leaf block b starts at sorted position start[b] with cnt[b] triangles.
__global__ void k_leaf_blocks(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ count,
                              const uint32_t* __restrict__ blockOf, uint32_t n, uint32_t* __restrict__ start,
                              uint32_t* __restrict__ cnt) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n || !flag[t]) return;
    start[blockOf[t]] = t;
    cnt[blockOf[t]] = count[t];
}

// One task per (internal node, side) whose child is a leaf: the leaf's box,
// then up the tree; at each node the second arriving child computes the
// node's box and size and hands them to the parent. The sibling's record is
// read after the arrival counter (acquire side of the __threadfence pair).
__global__ void k_bottom_up(const Inner* __restrict__ inner, const uint32_t* __restrict__ parent,
                            const float* __restrict__ pos, const uint4* __restrict__ tris,
                            const uint32_t* __restrict__ order, uint32_t n, uint32_t leafSize,
                            ChildRec* rec, uint32_t* arrive, float* rootBox, uint32_t* rootSize,
                            uint32_t* err) {
    const uint32_t task = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= 2 * (n - 1)) return;
    uint32_t i = task >> 1;
    const int side = (int)(task & 1u);
    const Inner in = inner[i];
    if (in.last - in.first + 1 <= leafSize) return;
    uint32_t f, c;
    child_range(inner, side ? in.right : in.left, f, c);
    if (c > leafSize) return;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t k = f; k < f + c; ++k) {
        float a[3], b[3];
        tri_box(pos, tris[order[k]], a, b);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            lo[q] = fminf(lo[q], a[q]);
            hi[q] = fmaxf(hi[q], b[q]);
        }
    }
    ChildRec* r = rec + i;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        __stcg(&r->lo[side][q], lo[q]);
        __stcg(&r->hi[side][q], hi[q]);
    }
    __stcg(&r->size[side], 1u);
    for (int level = 0;; ++level) {
        if (level > kMaxDepth) {
            raise_error(err, DEVERR_BUILD);
            return;
        }
        __threadfence();
        if (atomicAdd(arrive + i, 1u) == 0) return;  // the sibling is still on its way
        __threadfence();
        r = rec + i;
        uint32_t sz = 1;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            lo[q] = fminf(__ldcg(&r->lo[0][q]), __ldcg(&r->lo[1][q]));
            hi[q] = fmaxf(__ldcg(&r->hi[0][q]), __ldcg(&r->hi[1][q]));
        }
        sz += __ldcg(&r->size[0]) + __ldcg(&r->size[1]);
        const uint32_t p = parent[i];
        if (p != kRoot && p >= n - 1) {
            raise_error(err, DEVERR_BUILD);
            return;
        }
        if (p == kRoot) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                rootBox[q] = lo[q];
                rootBox[3 + q] = hi[q];
            }
            *rootSize = sz;
            return;
        }
        const int s = inner[p].left == i ? 0 : 1;
        ChildRec* pr = rec + p;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            __stcg(&pr->lo[s][q], lo[q]);
            __stcg(&pr->hi[s][q], hi[q]);
        }
        __stcg(&pr->size[s], sz);
        i = p;
    }
}

GPUGI_D void store_node(float4* nodes, uint32_t idx, const float lo[3], uint32_t child, const float hi[3],
                        uint32_t escape) {
    nodes[2 * (size_t)idx] = make_float4(lo[0], lo[1], lo[2], __uint_as_float(child));
    nodes[2 * (size_t)idx + 1] = make_float4(hi[0], hi[1], hi[2], __uint_as_float(escape));
}

// Every inner output node finds its preorder index from its path to the
// root: an edge from a left child adds 1 (the parent), from a right child
// 1 + the size of the left subtree. Its escape is the right sibling of the
// lowest ancestor edge taken from a left child (0 on the right spine). The
// node writes itself and its leaf children.
__global__ void k_emit_nodes(const Inner* __restrict__ inner, const uint32_t* __restrict__ parent,
                             const ChildRec* __restrict__ rec, const uint32_t* __restrict__ blockOf, uint32_t n,
                             uint32_t leafSize, float4* __restrict__ nodes, uint32_t numNodes, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    const Inner in = inner[i];
    if (in.last - in.first + 1 <= leafSize) return;
    uint32_t total = 0, atLeft = 0, leftParent = kRoot;
    int level = 0;
    for (uint32_t v = i, p = parent[i]; p != kRoot; v = p, p = parent[p]) {
        if (++level > kMaxDepth || p >= n - 1) {
            raise_error(err, DEVERR_BUILD);
            return;
        }
        const bool isLeft = inner[p].left == v;
        total += isLeft ? 1u : 1u + rec[p].size[0];
        if (isLeft && leftParent == kRoot) {
            leftParent = p;
            atLeft = total;
        }
    }
    const uint32_t idx = total;
    const uint32_t esc = leftParent == kRoot ? 0u : (total - atLeft) + 1u + rec[leftParent].size[0];
    const ChildRec r = rec[i];
    float lo[3], hi[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        lo[q] = fminf(r.lo[0][q], r.lo[1][q]);
        hi[q] = fmaxf(r.hi[0][q], r.hi[1][q]);
    }
    const uint32_t rightIdx = idx + 1 + r.size[0];
    if (rightIdx >= numNodes || esc >= numNodes) {  // sizes of an inconsistent tree: write nothing
        raise_error(err, DEVERR_BUILD);
        return;
    }
    store_node(nodes, idx, lo, idx + 1, hi, esc);
    for (int side = 0; side < 2; ++side) {
        uint32_t f, c;
        child_range(inner, side ? in.right : in.left, f, c);
        if (c > leafSize) continue;
        const uint32_t word = LEAF_FLAG | (c << LEAF_COUNT_SHIFT) | blockOf[f];
        store_node(nodes, side ? rightIdx : idx + 1, r.lo[side], word, r.hi[side], side ? esc : rightIdx);
    }
}

__global__ void k_emit_slots(const uint4* __restrict__ tris, const uint32_t* __restrict__ order,
                             const uint32_t* __restrict__ start, const uint32_t* __restrict__ cnt,
                             uint32_t numSlots, uint32_t leafSize, int4* __restrict__ slots) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= numSlots) return;
    const uint32_t b = s / leafSize, k = s % leafSize;
    int4 v = make_int4(0, 0, 0, 0);
    if (k < cnt[b]) {
        const uint4 t = tris[order[start[b] + k]];
        v = make_int4((int)t.x, (int)t.y, (int)t.z, (int)t.w);
    }
    slots[s] = v;
}

}  // namespace lbvh
}  // namespace gpugi

using namespace gpugi;

namespace {

// Device memory of one build, released on every exit path.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    cudaError_t get(T** out, size_t count) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(p);
        *out = static_cast<T*>(p);
        return e;
    }
};

}  // namespace

// Builds into sc (attached to ctx); the caller destroys sc on failure.
static gpugi_status build_into(gpugi_ctx* ctx, gpugi_scene* sc, const float* positions, uint32_t numVertices,
                               const uint32_t* triangles, uint32_t numTriangles, const float* vertexInfo,
                               const gpugi_material* materials, uint32_t numMaterials, uint32_t leafSize) {
    using namespace gpugi::lbvh;
    cudaStream_t st = ctx->stream;
    const uint32_t n = numTriangles;
    auto own = [&](size_t bytes, void** p) -> gpugi_status {
        if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess)
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "cudaMalloc failed for scene buffer");
        sc->allocations.push_back(*p);
        return GPUGI_OK;
    };
    gpugi_status gs;
    float* dPos;
    if ((gs = own(12 * (size_t)numVertices, (void**)&dPos))) return gs;

    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dPos, positions, 12 * (size_t)numVertices, cudaMemcpyHostToDevice, st));
    float4* dInfo;
    if ((gs = own(16 * (size_t)numVertices, (void**)&dInfo))) return gs;
    if (vertexInfo)
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dInfo, vertexInfo, 16 * (size_t)numVertices, cudaMemcpyHostToDevice, st));
    else
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(dInfo, 0, 16 * (size_t)numVertices, st));
    float4* dMat = nullptr;
    if (numMaterials > 0) {
        if ((gs = own(96 * (size_t)numMaterials, (void**)&dMat))) return gs;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dMat, materials, 96 * (size_t)numMaterials, cudaMemcpyHostToDevice, st));
    }

    Scratch S;
    uint4* dTri;
    uint64_t *keys, *keysSorted;
    uint32_t *vals, *order, *bounds, *flag, *count, *blockOf, *counters;
    if (S.get(&dTri, n) || S.get(&keys, n) || S.get(&keysSorted, n) || S.get(&vals, n) || S.get(&order, n) ||
        S.get(&bounds, 8) || S.get(&flag, n) || S.get(&count, n) || S.get(&blockOf, n) || S.get(&counters, 8))
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "builder scratch");
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dTri, triangles, 16 * (size_t)n, cudaMemcpyHostToDevice, st));
    const uint32_t init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(bounds, init, sizeof init, cudaMemcpyHostToDevice, st));
    const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->numSMs * 8);
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(counters, 0, 32, st));
    k_validate<<<grid, 256, 0, st>>>(dTri, n, numVertices, numMaterials, counters);
    uint32_t bad = 0;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&bad, counters, 4, cudaMemcpyDeviceToHost, st));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (bad & 1u) return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "triangle references a vertex out of range");
    if (bad & 2u) return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "triangle with v0 == v1");
    if (bad & 4u) return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "triangle references a material out of range");
    k_centre_bounds<<<grid, 256, 0, st>>>(dPos, dTri, n, bounds);
    k_morton<<<grid, 256, 0, st>>>(dPos, dTri, n, bounds, keys, vals);
    size_t tempBytes = 0, scanBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, keys, keysSorted, vals, order, (int)n, 0, 63, st);
    cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, flag, blockOf, (int)n, st);
    void* temp;
    if (S.get((char**)&temp, std::max(tempBytes, scanBytes)))
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "builder scratch");
    GPUGI_CUDA_TRY(ctx, cub::DeviceRadixSort::SortPairs(temp, tempBytes, keys, keysSorted, vals, order, (int)n, 0,
                                                        63, st));

    uint32_t numInner = 0, numBlocks = 0, numNodes = 0;
    float rootBox[6];
    Inner* inner = nullptr;
    uint32_t* parent = nullptr;
    ChildRec* rec = nullptr;
    if (n > leafSize) {
        uint32_t *arrive, *start, *cnt;
        if (S.get(&inner, n - 1) || S.get(&parent, n - 1) || S.get(&rec, n - 1) || S.get(&arrive, n - 1))
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "builder scratch");
        k_radix_tree<<<(n - 1 + 255) / 256, 256, 0, st>>>(keysSorted, (int)n, inner, parent);
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(flag, 0, 4 * (size_t)n, st));
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(counters, 0, 32, st));
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(arrive, 0, 4 * (size_t)(n - 1), st));
        k_mark_leaves<<<(n + 255) / 256, 256, 0, st>>>(inner, n, leafSize, flag, count, counters);
        GPUGI_CUDA_TRY(ctx, cub::DeviceScan::ExclusiveSum(temp, scanBytes, flag, blockOf, (int)n, st));
        uint32_t last[2], hostInner;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&last[0], flag + n - 1, 4, cudaMemcpyDeviceToHost, st));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&last[1], blockOf + n - 1, 4, cudaMemcpyDeviceToHost, st));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&hostInner, counters, 4, cudaMemcpyDeviceToHost, st));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        numInner = hostInner;
        numBlocks = last[0] + last[1];
        numNodes = 2 * numInner + 1;
        if (numBlocks != numInner + 1 || numBlocks - 1 > LEAF_BLOCK_MASK)
            return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "hierarchy build produced an inconsistent tree");
        if (S.get(&start, numBlocks) || S.get(&cnt, numBlocks))
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "builder scratch");
        k_leaf_blocks<<<(n + 255) / 256, 256, 0, st>>>(flag, count, blockOf, n, start, cnt);
        k_bottom_up<<<(2 * (n - 1) + 255) / 256, 256, 0, st>>>(inner, parent, dPos, dTri, order, n, leafSize, rec,
                                                             arrive, reinterpret_cast<float*>(counters + 2),
                                                             counters + 1, ctx->errWord);
        float4* dNodes;
        int4* dSlots;
        if ((gs = own(32 * (size_t)numNodes, (void**)&dNodes))) return gs;
        if ((gs = own(16 * (size_t)numBlocks * leafSize, (void**)&dSlots))) return gs;
        k_emit_nodes<<<(n - 1 + 255) / 256, 256, 0, st>>>(inner, parent, rec, blockOf, n, leafSize, dNodes,
                                                            numNodes, ctx->errWord);
        const uint32_t numSlots = numBlocks * leafSize;
        k_emit_slots<<<(numSlots + 255) / 256, 256, 0, st>>>(dTri, order, start, cnt, numSlots, leafSize, dSlots);
        sc->dev.nodes = dNodes;
        sc->dev.slots = dSlots;
        uint32_t rootSize = 0;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&rootSize, counters + 1, 4, cudaMemcpyDeviceToHost, st));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        if (gpugi_status es = gpugi_sync(ctx)) return es;
        if (rootSize != numNodes)
            return fail(ctx, GPUGI_ERROR_INVALID_SCENE, "hierarchy build produced an inconsistent tree");
    } else {
        // at most leafSize triangles: the root is the only node, one leaf
        std::vector<float> node(8);
        std::vector<int32_t> slots(4 * (size_t)leafSize, 0);
        for (int c = 0; c < 3; ++c) {
            rootBox[c] = INFINITY;
            rootBox[3 + c] = -INFINITY;
        }
        for (uint32_t t = 0; t < n; ++t) {
            for (int k = 0; k < 3; ++k)
                for (int c = 0; c < 3; ++c) {
                    const float p = positions[3 * (size_t)triangles[4 * t + k] + c];
                    rootBox[c] = std::min(rootBox[c], p);
                    rootBox[3 + c] = std::max(rootBox[3 + c], p);
                }
            for (int k = 0; k < 4; ++k) slots[4 * t + k] = (int32_t)triangles[4 * t + k];
        }
        const uint32_t word = LEAF_FLAG | (n << LEAF_COUNT_SHIFT), zero = 0;
        for (int c = 0; c < 3; ++c) {
            node[c] = rootBox[c];
            node[4 + c] = rootBox[3 + c];
        }
        std::memcpy(&node[3], &word, 4);
        std::memcpy(&node[7], &zero, 4);
        float4* dNodes;
        int4* dSlots;
        if ((gs = own(32, (void**)&dNodes)) || (gs = own(16 * (size_t)leafSize, (void**)&dSlots))) return gs;
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dNodes, node.data(), 32, cudaMemcpyHostToDevice, st));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(dSlots, slots.data(), 16 * (size_t)leafSize, cudaMemcpyHostToDevice, st));
        sc->dev.nodes = dNodes;
        sc->dev.slots = dSlots;
        numNodes = 1;
        numBlocks = 1;
    }
    const uint32_t numSlots = numBlocks * leafSize;
    float4* dTris;
    if ((gs = own(48 * (size_t)numSlots, (void**)&dTris))) return gs;
    prepare_triangles(st, sc->dev.slots, numSlots, dPos, dTris);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    sc->dev.tris = dTris;
    sc->dev.positions = dPos;
    sc->dev.vinfo = dInfo;
    sc->dev.materials = dMat;
    sc->dev.err = ctx->errWord;
    sc->dev.numNodes = numNodes;
    sc->numNodesUploaded = numNodes;
    sc->dev.numSlots = numSlots;
    sc->dev.leafSize = leafSize;
    sc->dev.boundsKind = GPUGI_BOUNDS_AABB;
    sc->dev.numVertices = numVertices;
    sc->dev.numMaterials = numMaterials;
    sc->dev.topNodes = 0;
    sc->numLeafBlocks = numBlocks;
    // Host copies for the light tables (Scene::LoadLightSources): only the
    // emissive triangles, in input order, each with its own three vertices.
    bool anyEmissive = false;
    for (uint32_t m = 0; m < numMaterials; ++m) {
        const float* e = reinterpret_cast<const float*>(materials) + 24 * (size_t)m + 12;
        anyEmissive = anyEmissive || e[0] != 0.0f || e[1] != 0.0f || e[2] != 0.0f;
    }
    if (anyEmissive) {
        // flag and blockOf are free again (the kernels that read them are
        // queued before on the same stream)
        k_flag_emissive<<<grid, 256, 0, st>>>(dTri, n, dMat, flag);
        GPUGI_CUDA_TRY(ctx, cub::DeviceScan::ExclusiveSum(temp, scanBytes, flag, blockOf, (int)n, st));
        uint32_t last[2];
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&last[0], flag + n - 1, 4, cudaMemcpyDeviceToHost, st));
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(&last[1], blockOf + n - 1, 4, cudaMemcpyDeviceToHost, st));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        const uint32_t ne = last[0] + last[1];
        std::vector<uint32_t> list(4 * (size_t)ne);
        if (ne) {
            uint4* emissive;
            if (S.get(&emissive, ne)) return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "builder scratch");
            k_compact<<<grid, 256, 0, st>>>(dTri, n, flag, blockOf, emissive);
            GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(list.data(), emissive, 16 * (size_t)ne, cudaMemcpyDeviceToHost, st));
            GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        }
        sc->hostSlots.resize(4 * (size_t)ne);
        sc->hostPositions.resize(9 * (size_t)ne);
        for (uint32_t k = 0; k < ne; ++k) {
            for (int v = 0; v < 3; ++v) {
                sc->hostSlots[4 * (size_t)k + v] = (int32_t)(3 * k + v);
                for (int c = 0; c < 3; ++c)
                    sc->hostPositions[9 * (size_t)k + 3 * v + c] = positions[3 * (size_t)list[4 * (size_t)k + v] + c];
            }
            sc->hostSlots[4 * (size_t)k + 3] = (int32_t)list[4 * (size_t)k + 3];
        }
    }
    if (numMaterials)
        sc->hostMaterials.assign(reinterpret_cast<const float*>(materials),
                                 reinterpret_cast<const float*>(materials) + 24 * (size_t)numMaterials);
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return GPUGI_OK;
}

extern "C" gpugi_status gpugi_scene_build(gpugi_ctx* ctx, const float* positions, uint32_t numVertices,
                                          const uint32_t* triangles, uint32_t numTriangles, const float* vertexInfo,
                                          const gpugi_material* materials, uint32_t numMaterials, uint32_t leafSize,
                                          gpugi_scene** out) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!out) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!positions || !triangles || numVertices == 0 || numTriangles == 0)
        return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "empty scene: positions and triangles are required");
    if (leafSize == 0 || leafSize > 32) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "leafSize must be in [1, 32]");
    if (numMaterials > 0 && !materials) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "materials is NULL");
    if (numTriangles >= 0x10000000u) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "too many triangles (2^28 at most)");
    cudaError_t se = cudaSetDevice(ctx->device);
    if (se != cudaSuccess) return cuda_fail(ctx, se, "cudaSetDevice");
    gpugi_scene* sc = new gpugi_scene();
    attach_child(ctx, &sc->ctx);
    const gpugi_status st = build_into(ctx, sc, positions, numVertices, triangles, numTriangles, vertexInfo,
                                       materials, numMaterials, leafSize);
    if (st != GPUGI_OK) {
        gpugi_scene_destroy(sc);
        return st;
    }
    *out = sc;
    return GPUGI_OK;
}

// The hierarchy of a scene in the reference layout (leaf words without the
// slot count bits) in device node order, and its leaf slots. Sizes first
// (hierarchy and slots NULL), then the arrays.
extern "C" gpugi_status gpugi_scene_export(gpugi_ctx* ctx, const gpugi_scene* sc, uint32_t* numNodes,
                                           uint32_t* numSlots, float* hierarchy, int32_t* slots) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!sc || !numNodes || !numSlots) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    *numNodes = sc->dev.numNodes;
    *numSlots = sc->dev.numSlots;
    if (slots)
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(slots, sc->dev.slots, 16 * (size_t)sc->dev.numSlots,
                                            cudaMemcpyDeviceToHost, ctx->stream));
    if (hierarchy) {
        const size_t nf = sc->dev.boundsKind == GPUGI_BOUNDS_OBOX ? 12 : 8;  // floats per node
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(hierarchy, sc->dev.nodes, 4 * nf * (size_t)sc->dev.numNodes,
                                            cudaMemcpyDeviceToHost, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < sc->dev.numNodes; ++i) {
            uint32_t w;
            std::memcpy(&w, &hierarchy[nf * i + 3], 4);
            if (w & LEAF_FLAG) w = LEAF_FLAG | (w & LEAF_BLOCK_MASK);
            std::memcpy(&hierarchy[nf * i + 3], &w, 4);
            if (!sc->hostRadii.empty())  // ellipsoid nodes: the radii as uploaded, not their reciprocals
                for (int c = 0; c < 3; ++c) hierarchy[nf * i + 4 + c] = sc->hostRadii[3 * i + c];
        }
    }
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return GPUGI_OK;
}
