// Offline BVH builder: restates gpugi's bvhmake (the producer of the node
// layout the traversal kernels walk). Host-only C++, no CUDA.
//
// Layout produced (bvhmake/filedef.hpp:41-54, documentation/fileformat.tex):
//  * nodes in preorder; node 0 is the root (bvhmake/bvhbuilder.cpp:551);
//  * firstChild = index of the left child, or 0x80000000 | leafBlock when the
//    node's only child is a leaf block (bvhmake/buildmethods/sweep.cpp:210);
//  * escape(left child) = right child, escape(right child) = parent's escape,
//    escape(root) = 0 (RecursiveWriteHierarchy, bvhmake/bvhbuilder.cpp:710-722);
//  * leaf blocks of leafSize slots, padded with the invalid triangle {0,0,0,0}
//    (bvhmake/buildmethods/sweep.cpp:197-207, bvhbuilder.cpp:35).
//
// Differences from the reference, all deliberate:
//  * recursion is replaced by an explicit task stack that allocates nodes in
//    the same preorder (deep SAH trees would overflow the call stack);
//  * sorting is stable, so ties in the Hilbert or centre order resolve by
//    triangle index on every platform (std::sort leaves them unspecified);
//  * the sweep's three scratch bounding volumes live in their own variables
//    instead of the last slots of the node pool (sweep.cpp:214-216);
//  * ellipsoid bounds (FitEllipsoid) are fitted after the topology is built:
//    leaves by the particle-swarm centre search of aaellipsoidfit.cpp:46-79,
//    inner nodes as the ellipsoid around the box of all triangles below. The
//    reference derives inner boxes from the children's ellipsoids divided by
//    sqrt(3) (aaellipsoidfit.cpp:31-44), which does not contain the children,
//    so a traversal over it can miss hits. The point-count factor of
//    fitFromCenter uses the non-zero components of (v - centre), not of v
//    (aaellipsoidfit.cpp:21), for the same reason. Radii get a relative
//    margin of 2^-18 so that fitted vertices lie strictly inside.
#include "../../../include/gpugi_bvhmake.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_lastError;

struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return (&x)[i]; }
    float& operator[](int i) { return (&x)[i]; }
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline V3 vmin(V3 a, V3 b) { return V3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return V3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
inline float lensq(V3 a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }

struct Box {
    V3 min, max;
};
struct Ellipsoid {
    V3 center, radii;
};
// Oriented box: centre, half sides and the inverse orientation (a unit
// quaternion x, y, z, w that takes world directions into the box frame), the
// fields of gpugi's Scene::TreeNode<OBox> (gpugi/scene/scene.hpp:40-49).
struct OBox {
    V3 center, halfSides;
    float qInv[4];
};

inline Box BoxUnion(const Box& a, const Box& b) { return Box{vmin(a.min, b.min), vmax(a.max, b.max)}; }
// Surface of a box (epsilon's surface(Box), restated: 2(wx wy + wx wz + wy wz)).
inline float BoxSurface(const Box& b) {
    V3 w = b.max - b.min;
    return 2.0f * ((w.x * w.y + w.x * w.z) + w.y * w.z);
}
// Ellipsoid surface, Knud Thomsen's approximation with p = 1.6075
// (epsilon's surface(Ellipsoid) is not available; restated from the formula).
inline float EllipsoidSurface(const Ellipsoid& e) {
    const double p = 1.6075;
    double a = std::pow((double)e.radii.x, p), b = std::pow((double)e.radii.y, p),
           c = std::pow((double)e.radii.z, p);
    return (float)(4.0 * M_PI * std::pow((a * b + a * c + b * c) / 3.0, 1.0 / p));
}
// Ellipsoid around a box: radii = half extent * sqrt(3) (epsilon's Ellipsoid(Box)).
inline Ellipsoid EllipsoidOfBox(const Box& b) {
    return Ellipsoid{(b.min + b.max) * 0.5f, (b.max - b.min) * (0.5f * 1.7320508075688772f)};
}
inline bool PointInEllipsoid(V3 p, const Ellipsoid& e) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double off = (double)p[d] - (double)e.center[d];
        if (e.radii[d] == 0.0f) {
            if (off != 0.0) return false;
        } else {
            double q = off / (double)e.radii[d];
            s += q * q;
        }
    }
    return s <= 1.0;
}

// 64-bit xorshift* and its float helpers (gpugi/utilities/random.cpp:26-49).
inline uint64_t Xorshift64(uint64_t s) {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return s * UINT64_C(2685821657736338717);
}
inline float XorshiftRange(uint64_t& s, float lo, float hi) {
    s = Xorshift64(s);
    return (static_cast<float>(s % 8388593) / 8388593.0f) * (hi - lo) + lo;
}

// --- Hilbert-curve comparator (bvhmake/buildmethods/sweep.cpp:72-157) -------
inline uint64_t PartBy2(uint16_t x) {
    uint64_t r = x;
    r = (r | (r << 16)) & 0x0000ff0000ffULL;
    r = (r | (r << 8)) & 0x00f00f00f00fULL;
    r = (r | (r << 4)) & 0x0c30c30c30c3ULL;
    r = (r | (r << 2)) & 0x249249249249ULL;
    return r;
}
inline uint64_t Morton(uint16_t a, uint16_t b, uint16_t c) {
    return PartBy2(a) | (PartBy2(b) << 1) | (PartBy2(c) << 2);
}
inline uint64_t GrayToBinary(uint64_t num) {
    num ^= num >> 32;
    num ^= num >> 16;
    num ^= num >> 8;
    num ^= num >> 4;
    num ^= num >> 2;
    num ^= num >> 1;
    return num;
}
struct HilbertKey {
    uint64_t hi, lo;
};
inline HilbertKey MakeHilbertKey(V3 c) {
    uint32_t a[3];
    for (int d = 0; d < 3; ++d) {
        float v = c[d] * 4096.0f;
        a[d] = v > 0.0f ? (v < 4294967040.0f ? (uint32_t)v : 0xFFFFFF00u) : 0u;
    }
    HilbertKey k;
    k.hi = GrayToBinary(Morton((uint16_t)(a[0] >> 16), (uint16_t)(a[1] >> 16), (uint16_t)(a[2] >> 16)));
    k.lo = GrayToBinary(Morton((uint16_t)(a[0] & 0xffff), (uint16_t)(a[1] & 0xffff), (uint16_t)(a[2] & 0xffff)));
    return k;
}
// hilbertcurvecmp: compare the high 16-bit interleave, then the low one.
inline bool HilbertLess(const HilbertKey& a, const HilbertKey& b) {
    if (a.hi != b.hi) return a.hi < b.hi;
    return a.lo < b.lo;
}

struct Node {
    uint32_t left;   // child index or 0x80000000 | leaf block
    uint32_t right;  // right child (inner nodes)
};

}  // namespace

struct gpugi_bvh {
    std::vector<float> positions;      // 3 per vertex
    std::vector<float> normals;        // 3 per vertex (file attribute; may be empty)
    std::vector<float> texcoords;      // 2 per vertex (file attribute; may be empty)
    std::vector<float> materials;      // 24 per material ("gpugi_materials" chunk; may be empty)
    std::vector<std::string> materialNames;  // "materialref" chunk
    std::vector<uint32_t> triangles;   // 4 per triangle
    uint32_t leafSize = 8;
    uint32_t boundsKind = GPUGI_FIT_AABOX;
    std::vector<Node> nodes;           // preorder
    std::vector<Box> boxes;            // per node: box of all triangles below
    std::vector<Ellipsoid> ellipsoids; // per node when boundsKind == ellipsoid
    std::vector<OBox> oboxes;          // per node when boundsKind == obox
    std::vector<uint32_t> leaves;      // leafSize * 4 uint32 per block
    std::vector<uint32_t> escapes, parents;
    uint32_t maxDepth = 0;
    // "approx_sggx" chunk: 6 uint16 per node (computed from the vertex
    // normals on first use, or read from a file)
    mutable std::vector<uint16_t> sggx;

    V3 Pos(uint32_t v) const { return V3(positions[3 * v], positions[3 * v + 1], positions[3 * v + 2]); }
    Box TriBox(uint32_t t) const {
        V3 a = Pos(triangles[4 * t]), b = Pos(triangles[4 * t + 1]), c = Pos(triangles[4 * t + 2]);
        return Box{vmin(vmin(a, b), c), vmax(vmax(a, b), c)};
    }
    V3 Center(uint32_t t) const {
        V3 a = Pos(triangles[4 * t]), b = Pos(triangles[4 * t + 1]), c = Pos(triangles[4 * t + 2]);
        return ((a + b) + c) / 3.0f;
    }
    uint32_t NewLeaf(const uint32_t* ids, uint32_t lo, uint32_t hi) {
        uint32_t idx = (uint32_t)(leaves.size() / (4 * leafSize));
        for (uint32_t i = lo; i <= hi; ++i)
            for (int k = 0; k < 4; ++k) leaves.push_back(triangles[4 * ids[i] + k]);
        for (uint32_t i = hi - lo + 1; i < leafSize; ++i)
            for (int k = 0; k < 4; ++k) leaves.push_back(0u);
        return idx;
    }
};

namespace {

struct Task {
    uint32_t lo, hi;
    uint32_t parent;  // UINT32_MAX for the root
    bool isRight;
};

// Attach a freshly allocated node to its parent slot.
inline void Link(gpugi_bvh& b, const Task& t, uint32_t idx) {
    if (t.parent == UINT32_MAX) return;
    if (t.isRight) b.nodes[t.parent].right = idx;
    else b.nodes[t.parent].left = idx;
}

// BuildSweep (bvhmake/buildmethods/sweep.cpp:27-259): Hilbert-curve order,
// then at every node a full sweep over the sorted range that evaluates
// SAH(left) + SAH(right) with SAH = surface(child)/surface(parent) * count.
void BuildSweep(gpugi_bvh& b) {
    const uint32_t n = (uint32_t)(b.triangles.size() / 4);
    std::vector<V3> centers(n);
    V3 minCenter = b.Pos(b.triangles[0]);  // sweep.cpp:166 starts from v0 of triangle 0
    for (uint32_t i = 0; i < n; ++i) {
        centers[i] = b.Center(i);
        minCenter = vmin(centers[i], minCenter);
    }
    std::vector<HilbertKey> keys(n);
    for (uint32_t i = 0; i < n; ++i) keys[i] = MakeHilbertKey(centers[i] - minCenter);
    std::vector<uint32_t> sorted(n);
    for (uint32_t i = 0; i < n; ++i) sorted[i] = i;
    std::stable_sort(sorted.begin(), sorted.end(),
                     [&](uint32_t l, uint32_t r) { return HilbertLess(keys[l], keys[r]); });

    std::vector<Box> triBoxes(n);
    for (uint32_t i = 0; i < n; ++i) triBoxes[i] = b.TriBox(i);

    std::vector<float> hx, hy;
    std::vector<Task> stack;
    stack.push_back(Task{0, n - 1, UINT32_MAX, false});
    std::vector<uint32_t> depthOf;  // depth per task entry via parallel stack
    std::vector<uint32_t> depthStack{1};
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        uint32_t depth = depthStack.back();
        depthStack.pop_back();
        b.maxDepth = std::max(b.maxDepth, depth);
        uint32_t idx = (uint32_t)b.nodes.size();
        b.nodes.push_back(Node{0, 0});
        Link(b, t, idx);
        // ComputeBoundingVolume (sweep.cpp:262-274): box of the whole range.
        Box nodeBox = triBoxes[sorted[t.hi]];
        for (uint32_t i = t.lo; i < t.hi; ++i) nodeBox = BoxUnion(nodeBox, triBoxes[sorted[i]]);
        b.boxes.push_back(nodeBox);
        if (t.hi - t.lo < b.leafSize) {
            uint32_t leaf = b.NewLeaf(sorted.data(), t.lo, t.hi);
            b.nodes[idx].left = 0x80000000u | leaf;
            b.nodes[idx].right = 0;
            continue;
        }
        const uint32_t m = t.hi - t.lo;
        hx.assign(m, 0.0f);
        hy.assign(m, 0.0f);
        const float parentSurface = BoxSurface(nodeBox);
        Box left = triBoxes[sorted[t.lo]];
        Box right = triBoxes[sorted[t.hi]];
        for (uint32_t i = t.lo; i < t.hi; ++i) {
            left = BoxUnion(left, triBoxes[sorted[i]]);
            right = BoxUnion(right, triBoxes[sorted[t.hi - i + t.lo]]);
            hx[i - t.lo] = BoxSurface(left) / parentSurface * (float)(int)(i - t.lo + 1);
            hy[t.hi - i - 1] = BoxSurface(right) / parentSurface * (float)(int)(i - t.lo + 1);
        }
        // The minimum search starts at 1 (sweep.cpp:244), kept as is.
        float minCost = std::numeric_limits<float>::infinity();
        uint32_t split = t.lo;
        for (uint32_t i = 1; i < m; ++i) {
            float c = hx[i] + hy[i];
            if (c < minCost) {
                minCost = c;
                split = i + t.lo;
            }
        }
        stack.push_back(Task{split + 1, t.hi, idx, true});
        depthStack.push_back(depth + 1);
        stack.push_back(Task{t.lo, split, idx, false});
        depthStack.push_back(depth + 1);
    }
}

// BuildKdtree (bvhmake/buildmethods/kdtree.cpp:9-157): median split of the
// triangle centres along the axis of largest centre extent.
void BuildKdtree(gpugi_bvh& b) {
    const uint32_t n = (uint32_t)(b.triangles.size() / 4);
    std::vector<V3> centers(n);
    for (uint32_t i = 0; i < n; ++i) centers[i] = b.Center(i);
    std::vector<uint32_t> sorted[3];
    for (int d = 0; d < 3; ++d) {
        sorted[d].resize(n);
        for (uint32_t i = 0; i < n; ++i) sorted[d][i] = i;
        std::stable_sort(sorted[d].begin(), sorted[d].end(),
                         [&](uint32_t l, uint32_t r) { return centers[l][d] < centers[r][d]; });
    }
    std::vector<uint32_t> tmp;
    // kdtree.cpp:63-83: stable partition of a co-dimension array by the plane.
    auto split = [&](uint32_t* list, uint32_t size, int dim, float plane) {
        tmp.resize(size);
        uint32_t rightOff = (size + 1) / 2;
        uint32_t l = 0, r = rightOff;
        for (uint32_t i = 0; i < size; ++i) {
            if (centers[list[i]][dim] <= plane) {
                if (l < size) tmp[l] = list[i];
                ++l;
            } else {
                if (r < size) tmp[r] = list[i];
                ++r;
            }
        }
        if (l != rightOff) return false;
        std::memcpy(list, tmp.data(), size * sizeof(uint32_t));
        return true;
    };
    std::vector<Task> stack{Task{0, n - 1, UINT32_MAX, false}};
    std::vector<uint32_t> depthStack{1};
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        uint32_t depth = depthStack.back();
        depthStack.pop_back();
        b.maxDepth = std::max(b.maxDepth, depth);
        uint32_t idx = (uint32_t)b.nodes.size();
        b.nodes.push_back(Node{0, 0});
        b.boxes.push_back(Box{});
        Link(b, t, idx);
        if (t.hi - t.lo < b.leafSize) {
            uint32_t leaf = b.NewLeaf(sorted[0].data(), t.lo, t.hi);
            b.nodes[idx].left = 0x80000000u | leaf;
            Box bx = b.TriBox(sorted[0][t.lo]);
            for (uint32_t i = t.lo + 1; i <= t.hi; ++i) bx = BoxUnion(bx, b.TriBox(sorted[0][i]));
            b.boxes[idx] = bx;
            continue;
        }
        V3 lo(centers[sorted[0][t.lo]].x, centers[sorted[1][t.lo]].y, centers[sorted[2][t.lo]].z);
        V3 hi(centers[sorted[0][t.hi]].x, centers[sorted[1][t.hi]].y, centers[sorted[2][t.hi]].z);
        V3 w = hi - lo;
        int dim = 0;
        if (w[1] > w[0] && w[1] > w[2]) dim = 1;
        if (w[2] > w[0] && w[2] > w[1]) dim = 2;
        int codim1 = (dim + 1) % 3, codim2 = (dim + 2) % 3;
        uint32_t m = (t.lo + t.hi) / 2;
        uint32_t numChanged = 0;
        float plane = centers[sorted[dim][m]][dim];
        while (m + numChanged < t.hi && centers[sorted[dim][m + 1 + numChanged]][dim] == plane) {
            centers[sorted[dim][m + 1 + numChanged]][dim] = std::nextafter(plane, INFINITY) + 1.0f;
            ++numChanged;
        }
        bool ok = split(&sorted[codim1][t.lo], t.hi - t.lo + 1, dim, plane) &&
                  split(&sorted[codim2][t.lo], t.hi - t.lo + 1, dim, plane);
        for (uint32_t i = m + 1; i < m + 1 + numChanged; ++i) centers[sorted[dim][i]][dim] = plane;
        if (!ok) throw std::runtime_error("kdtree split lost elements (degenerate centres)");
        stack.push_back(Task{m + 1, t.hi, idx, true});
        depthStack.push_back(depth + 1);
        stack.push_back(Task{t.lo, m, idx, false});
        depthStack.push_back(depth + 1);
    }
    // Inner boxes bottom-up: children always follow their parent in preorder.
    for (int64_t i = (int64_t)b.nodes.size() - 1; i >= 0; --i) {
        const Node& nd = b.nodes[i];
        if (!(nd.left & 0x80000000u)) b.boxes[i] = BoxUnion(b.boxes[nd.left], b.boxes[nd.right]);
    }
}

// --- Ellipsoid fit (bvhmake/fitmethods/aaellipsoidfit.cpp, optimize.inl) -----
Ellipsoid FitFromCenter(const std::vector<V3>& verts, V3 center) {
    Ellipsoid e{center, V3(0, 0, 0)};
    for (const V3& v : verts) {
        if (!PointInEllipsoid(v, e)) {
            V3 off = v - center;
            float cnt = (float)((off.x != 0.0f) + (off.y != 0.0f) + (off.z != 0.0f));
            float s = std::sqrt(cnt);
            V3 r(s * std::fabs(off.x), s * std::fabs(off.y), s * std::fabs(off.z));
            e.radii = vmax(e.radii, r);
        }
    }
    return e;
}

struct Particle {
    V3 position, optPosition, velocity;
    float optFitness, globalAttraction, localAttraction, randomAttraction, charge, damping;
};

void RandomizeParameters(Particle& p, V3 domain, uint64_t& s) {
    p.globalAttraction = XorshiftRange(s, 0.05f, 0.5f);
    p.localAttraction = XorshiftRange(s, 0.0f, 0.25f);
    p.randomAttraction = XorshiftRange(s, 0.0f, 0.001f);
    p.charge = XorshiftRange(s, 0.0f, 0.01f);
    p.damping = XorshiftRange(s, 0.35f, 0.55f);
    for (int d = 0; d < 3; ++d) p.velocity[d] = XorshiftRange(s, domain[d] * 0.01f, domain[d] * 0.02f);
    p.optFitness = std::numeric_limits<float>::infinity();
}

// Particle swarm minimisation over a box (optimize.inl:21-176): 30 particles,
// 27 of them stratified on a 3x3x3 grid, maxIterations rounds.
V3 OptimizeCenter(V3 mn, V3 mx, const std::function<float(const V3&)>& f, int maxIterations, uint64_t seed) {
    uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ULL;
    std::vector<Particle> pop;
    V3 domain = mx - mn;
    const int cells = 3, num = 27;
    int x[3] = {0, 0, 0};
    for (int i = 0; i < num; ++i) {
        Particle p{};
        // optimize.inl:51-52 places stratified particles relative to 0, not
        // to _min; kept, the move step clamps them into the box.
        for (int d = 0; d < 3; ++d)
            p.position[d] = x[d] * domain[d] / cells + XorshiftRange(s, 0.0f, domain[d] / cells);
        RandomizeParameters(p, domain, s);
        pop.push_back(p);
        int d = 0;
        bool carry = true;
        while (carry && d < 3) {
            carry = ++x[d] == cells;
            if (carry) x[d] = 0;
            ++d;
        }
    }
    for (int i = num; i < 30; ++i) {
        Particle p{};
        for (int d = 0; d < 3; ++d) p.position[d] = XorshiftRange(s, mn[d], mx[d]);
        RandomizeParameters(p, domain, s);
        pop.push_back(p);
    }
    V3 globalOpt = pop[0].position;
    float globalFit = std::numeric_limits<float>::infinity();
    const float domainLen = std::sqrt(lensq(mx - mn));
    for (int turn = 0; turn < maxIterations; ++turn) {
        for (auto& p : pop) {
            float v = f(p.position);
            if (v <= p.optFitness) {
                p.optFitness = v;
                p.optPosition = p.position;
            }
            if (v < globalFit) {
                globalFit = v;
                globalOpt = p.position;
            }
        }
        for (size_t i = 0; i < pop.size(); ++i) {
            Particle& p = pop[i];
            V3 toGlobal = globalOpt - p.position;
            V3 toPersonal = p.optPosition - p.position;
            V3 rnd;
            for (int d = 0; d < 3; ++d) rnd[d] = XorshiftRange(s, mn[d], mx[d]);
            rnd = rnd * (domainLen / (std::sqrt(lensq(rnd)) + 1e-10f));
            p.velocity = p.velocity * p.damping + toGlobal * p.globalAttraction +
                         toPersonal * p.localAttraction + rnd * p.randomAttraction;
            for (size_t j = 0; j < pop.size(); ++j) {
                if (j == i) continue;
                V3 jToi = p.position - pop[j].position;
                p.velocity = p.velocity + jToi * (std::exp(-lensq(jToi) * 0.4f) * p.charge);
            }
            p.position = p.position + p.velocity;
            for (int d = 0; d < 3; ++d) {
                if (p.position[d] < mn[d] || p.position[d] > mx[d]) {
                    p.position[d] = std::fmin(std::fmax(p.position[d], mn[d]), mx[d]);
                    p.velocity[d] = -p.velocity[d];
                }
            }
        }
    }
    return globalOpt;
}

inline Ellipsoid Inflate(Ellipsoid e, const Box& bx) {
    V3 ext = bx.max - bx.min;
    float tiny = 1e-7f * std::fmax(std::fmax(ext.x, ext.y), ext.z);
    for (int d = 0; d < 3; ++d) e.radii[d] = e.radii[d] * (1.0f + 1.0f / 262144.0f) + tiny;
    return e;
}

void FitEllipsoids(gpugi_bvh& b, uint64_t seed) {
    const size_t nn = b.nodes.size();
    b.ellipsoids.assign(nn, Ellipsoid{});
    std::vector<uint32_t> leafNodes;
    for (size_t i = 0; i < nn; ++i) {
        if (b.nodes[i].left & 0x80000000u) leafNodes.push_back((uint32_t)i);
        else b.ellipsoids[i] = Inflate(EllipsoidOfBox(b.boxes[i]), b.boxes[i]);
    }
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t) {
        pool.emplace_back([&, t]() {
            std::vector<V3> verts;
            for (size_t k = t; k < leafNodes.size(); k += nt) {
                uint32_t ni = leafNodes[k];
                uint32_t blk = b.nodes[ni].left & 0x7FFFFFFFu;
                verts.clear();
                V3 mn(INFINITY, INFINITY, INFINITY), mx(-INFINITY, -INFINITY, -INFINITY);
                const uint32_t* slot = &b.leaves[(size_t)blk * b.leafSize * 4];
                for (uint32_t j = 0; j < b.leafSize; ++j) {
                    if (slot[4 * j] == slot[4 * j + 1]) break;
                    for (int c = 0; c < 3; ++c) {
                        V3 v = b.Pos(slot[4 * j + c]);
                        verts.push_back(v);
                        mn = vmin(mn, v);
                        mx = vmax(mx, v);
                    }
                }
                uint64_t s = seed ^ (0xD1B54A32D192ED03ULL * (uint64_t)(ni + 1));
                V3 c = OptimizeCenter(mn, mx, [&](const V3& ctr) { return EllipsoidSurface(FitFromCenter(verts, ctr)); },
                                      15, s);
                Ellipsoid e = Inflate(FitFromCenter(verts, c), Box{mn, mx});
                // A fitted ellipsoid must hold every vertex; fall back to the box
                // ellipsoid when rounding leaves one outside.
                bool ok = true;
                for (const V3& v : verts) ok = ok && PointInEllipsoid(v, e);
                if (!ok) e = Inflate(EllipsoidOfBox(Box{mn, mx}), Box{mn, mx});
                b.ellipsoids[ni] = e;
            }
        });
    }
    for (auto& th : pool) th.join();
}

// Escape pointers and parents (RecursiveWriteHierarchy, bvhbuilder.cpp:710-722).
void AssignEscapes(gpugi_bvh& b) {
    const size_t nn = b.nodes.size();
    b.escapes.assign(nn, 0);
    b.parents.assign(nn, 0);
    for (size_t i = 0; i < nn; ++i) {  // preorder: the parent is final before its children
        const Node& nd = b.nodes[i];
        if (nd.left & 0x80000000u) continue;
        b.escapes[nd.left] = nd.right;
        b.escapes[nd.right] = b.escapes[i];
        b.parents[nd.left] = (uint32_t)i;
        b.parents[nd.right] = (uint32_t)i;
    }
}

// --- Node NDFs (bvhmake/processing/approx_sggx.cpp) -------------------------
// The symmetric SGGX matrix of a node, S = Q^T diag(lambda) Q, from the
// vertex normals of the triangles below it. Per leaf block: 1000 normals
// spread over the triangles by area at Halton (2, 3) barycentric points,
// the eigenvectors Q of their second-moment matrix, and lambda_k the mean
// |q_k . n| (approx_sggx.cpp:88-154). Inner nodes blend their two children
// weighted by the children's bounding-volume surfaces (approx_sggx.cpp:
// 156-184). epsilon's decomposeQl is not available; the eigenvectors come
// from the cyclic Jacobi method in double precision. S does not depend on
// the eigenvectors' order or signs (lambda_k pairs with its own q_k), only
// on their directions, except within a repeated eigenvalue, where the
// choice of basis can change lambda: parity of these values is unpinned.
struct Sggx {
    float xx, xy, xz, yy, yz, zz;
};

// approx_sggx.cpp:13-25
inline int HaltonRev(int i, int p) { return i == 0 ? i : p - i; }
inline float Halton(int base, int i) {
    float h = 0.0f;
    const float f = 1.0f / (float)base;
    float fct = f;
    while (i > 0) {
        h += (float)HaltonRev(i % base, base) * fct;
        i /= base;
        fct *= f;
    }
    return h;
}

inline float Dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 Cross(V3 a, V3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 Normalize(V3 a) { return a / std::sqrt(Dot(a, a)); }
// epsilon's surface(Triangle), restated: half the length of the edge cross product.
inline float TriangleSurface(V3 a, V3 b, V3 c) {
    V3 n = Cross(b - a, c - a);
    return std::sqrt(Dot(n, n)) * 0.5f;
}

// Cyclic Jacobi rotations on a symmetric 3x3 matrix: rows of q are the
// eigenvectors, lambda (optional) the eigenvalues in the same order (Golub &
// Van Loan, "Matrix Computations", 8.5).
void SymmetricEigen3(const double in[3][3], double q[3][3], double* lambda = nullptr) {
    double a[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            a[r][c] = in[r][c];
            q[r][c] = r == c ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 64; ++sweep) {
        const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        const double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int r = p + 1; r < 3; ++r) {
                if (a[p][r] == 0.0) continue;
                const double theta = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; ++k) {  // A <- A J (columns p, r)
                    const double akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - sn * akr;
                    a[k][r] = sn * akp + c * akr;
                }
                for (int k = 0; k < 3; ++k) {  // A <- J^T A (rows p, r)
                    const double apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - sn * ark;
                    a[r][k] = sn * apk + c * ark;
                }
                for (int k = 0; k < 3; ++k) {  // eigenvector rows: Q <- J^T Q
                    const double qp = q[p][k], qr = q[r][k];
                    q[p][k] = c * qp - sn * qr;
                    q[r][k] = sn * qp + c * qr;
                }
            }
    }
    if (lambda)
        for (int k = 0; k < 3; ++k) lambda[k] = a[k][k];
}

// ComputeLeafSGGXBase (approx_sggx.cpp:88-154) for leaf block blk.
Sggx LeafSggx(const gpugi_bvh& b, uint32_t blk) {
    const int kSamples = 1000;  // NORMAL_SAMPLES
    std::vector<V3> pos, nrm;
    for (uint32_t k = 0; k < b.leafSize; ++k) {
        const uint32_t* t = &b.leaves[4 * ((size_t)blk * b.leafSize + k)];
        if (t[0] == 0 && t[1] == 0 && t[2] == 0 && t[3] == 0) break;  // INVALID_TRIANGLE
        for (int v = 0; v < 3; ++v) {
            pos.push_back(b.Pos(t[v]));
            nrm.push_back(V3(b.normals[3 * (size_t)t[v]], b.normals[3 * (size_t)t[v] + 1],
                             b.normals[3 * (size_t)t[v] + 2]));
        }
    }
    const int n = (int)pos.size() / 3;
    float area = 0.0f;
    for (int i = 0; i < n; ++i) area += TriangleSurface(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    // The reference interpolates with the second vertex normal twice
    // (nrm[i*3+1] * gamma, approx_sggx.cpp:114,143); kept.
    auto sampleNormal = [&](int i, int j) {
        float al = Halton(2, j), be = Halton(3, j);
        if (al + be > 1.0f) {
            al = 1.0f - al;
            be = 1.0f - be;
        }
        const float ga = 1.0f - al - be;
        return Normalize((nrm[3 * i] * al + nrm[3 * i + 1] * be) + nrm[3 * i + 1] * ga);
    };
    auto count = [&](int i) {
        return (int)((float)kSamples * TriangleSurface(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]) / area);
    };
    float E[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < n; ++i)
        for (int j = 0, ns = count(i); j < ns; ++j) {
            const V3 nv = sampleNormal(i, j);
            E[0][0] += nv.x * nv.x;
            E[0][1] += nv.x * nv.y;
            E[0][2] += nv.x * nv.z;
            E[1][1] += nv.y * nv.y;
            E[1][2] += nv.y * nv.z;
            E[2][2] += nv.z * nv.z;
        }
    E[1][0] = E[0][1];
    E[2][0] = E[0][2];
    E[2][1] = E[1][2];
    double Ed[3][3], Qd[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Ed[r][c] = E[r][c];
    SymmetricEigen3(Ed, Qd);
    V3 q[3];
    for (int k = 0; k < 3; ++k) q[k] = V3((float)Qd[k][0], (float)Qd[k][1], (float)Qd[k][2]);
    float lam[3] = {0.0f, 0.0f, 0.0f};
    int total = 0;
    for (int i = 0; i < n; ++i) {
        const int ns = count(i);
        total += ns;
        for (int j = 0; j < ns; ++j) {
            const V3 nv = sampleNormal(i, j);
            for (int k = 0; k < 3; ++k) lam[k] += std::fabs(Dot(q[k], nv));
        }
    }
    Sggx s{0, 0, 0, 0, 0, 0};
    if (total == 0) return s;
    for (int k = 0; k < 3; ++k) lam[k] /= (float)total;
    float S[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            S[r][c] = (q[0][r] * lam[0] * q[0][c] + q[1][r] * lam[1] * q[1][c]) + q[2][r] * lam[2] * q[2][c];
    s.xx = S[0][0];
    s.xy = S[0][1];
    s.xz = S[0][2];
    s.yy = S[1][1];
    s.yz = S[1][2];
    s.zz = S[2][2];
    return s;
}

// FitMethod::Surface of a node's bounding volume (aaboxfit.cpp:25-28,
// aaellipsoidfit.cpp:81-84).
float NodeSurface(const gpugi_bvh& b, uint32_t i) {
    if (b.boundsKind == GPUGI_FIT_OBOX) {  // epsilon's surface(OBox): the box of the half sides
        const V3 h = b.oboxes[i].halfSides;
        return 8.0f * ((h.x * h.y + h.x * h.z) + h.y * h.z);
    }
    return b.boundsKind == GPUGI_FIT_ELLIPSOID ? EllipsoidSurface(b.ellipsoids[i]) : BoxSurface(b.boxes[i]);
}

// The stored form (approx_sggx.cpp:185-187, filedef.hpp:79-95): sigma =
// sqrt(diagonal) and r = off-diagonal / sqrt(product of the diagonals), as
// truncated 16-bit integers (r shifted to [0, 65534]). A zero diagonal
// (division by zero in the reference) stores r = 0.
void PackSggx(const Sggx& s, uint16_t* o) {
    auto u16 = [](float v) {
        if (!(v > 0.0f)) return (uint16_t)0;
        return v >= 65535.0f ? (uint16_t)65535 : (uint16_t)v;
    };
    o[0] = u16(std::sqrt(s.xx) * 65535.0f);
    o[1] = u16(std::sqrt(s.yy) * 65535.0f);
    o[2] = u16(std::sqrt(s.zz) * 65535.0f);
    const float d[3] = {std::sqrt(s.xx * s.yy), std::sqrt(s.xx * s.zz), std::sqrt(s.yy * s.zz)};
    const float off[3] = {s.xy, s.xz, s.yz};
    for (int k = 0; k < 3; ++k) o[3 + k] = d[k] > 0.0f ? u16(off[k] / d[k] * 32767.0f + 32767.0f) : (uint16_t)32767;
}

// BuildLDS (bvhmake/buildmethods/lds.cpp:11-164, LDS_SPLITMODE_SWEEP): at
// every node the triangle centres are projected on the eigenvector of the
// largest eigenvalue of their covariance (n - 1 normalised), sorted by that
// projection, and split where the SAH sweep of the sweep builder is
// smallest (the minimum search starts at 0 here, lds.cpp:145). epsilon's
// decomposeQl is replaced by the Jacobi method above: the eigenvector's sign
// (which orders the children) is fixed by making its largest component
// positive, ties of eigenvalues pick the first as the reference's
// comparisons do, and the unstable std::sort of the reference is a stable
// sort: the trees are unpinned.
void BuildLds(gpugi_bvh& b) {
    const uint32_t n = (uint32_t)(b.triangles.size() / 4);
    std::vector<V3> centers(n);
    std::vector<Box> triBoxes(n);
    for (uint32_t i = 0; i < n; ++i) {
        centers[i] = b.Center(i);
        triBoxes[i] = b.TriBox(i);
    }
    std::vector<uint32_t> ids(n);
    for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    std::vector<float> proj(n), hx, hy;
    std::vector<Task> stack{Task{0, n - 1, UINT32_MAX, false}};
    std::vector<uint32_t> depthStack{1};
    while (!stack.empty()) {
        const Task t = stack.back();
        stack.pop_back();
        const uint32_t depth = depthStack.back();
        depthStack.pop_back();
        b.maxDepth = std::max(b.maxDepth, depth);
        const uint32_t idx = (uint32_t)b.nodes.size();
        b.nodes.push_back(Node{0, 0});
        Link(b, t, idx);
        Box nodeBox = triBoxes[ids[t.hi]];
        for (uint32_t i = t.lo; i < t.hi; ++i) nodeBox = BoxUnion(nodeBox, triBoxes[ids[i]]);
        b.boxes.push_back(nodeBox);
        if (t.hi - t.lo < b.leafSize) {
            const uint32_t leaf = b.NewLeaf(ids.data(), t.lo, t.hi);
            b.nodes[idx].left = 0x80000000u | leaf;
            b.nodes[idx].right = 0;
            continue;
        }
        // covariance of the centres (lds.cpp:67-82)
        V3 m = centers[ids[t.lo]];
        for (uint32_t i = t.lo + 1; i <= t.hi; ++i) m = m + centers[ids[i]];
        m = m / (float)(t.hi - t.lo + 1);
        float cov[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (uint32_t i = t.lo; i <= t.hi; ++i) {
            const V3 e = centers[ids[i]] - m;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) cov[r][c] += e[r] * e[c];
        }
        double covd[3][3], q[3][3], lam[3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) covd[r][c] = cov[r][c] / (float)(t.hi - t.lo);
        SymmetricEigen3(covd, q, lam);
        const int k = (lam[0] > lam[1] && lam[0] > lam[2]) ? 0 : (lam[1] > lam[2] ? 1 : 2);
        int big = 0;
        for (int c = 1; c < 3; ++c)
            if (std::fabs(q[k][c]) > std::fabs(q[k][big])) big = c;
        const double sgn = q[k][big] < 0.0 ? -1.0 : 1.0;
        const V3 dir((float)(sgn * q[k][0]), (float)(sgn * q[k][1]), (float)(sgn * q[k][2]));
        for (uint32_t i = t.lo; i <= t.hi; ++i) proj[ids[i]] = Dot(centers[ids[i]], dir);
        std::stable_sort(ids.begin() + t.lo, ids.begin() + t.hi + 1,
                         [&](uint32_t l, uint32_t r) { return proj[l] < proj[r]; });
        // SAH sweep over the sorted range (lds.cpp:118-152)
        const uint32_t cnt = t.hi - t.lo;
        hx.assign(cnt, 0.0f);
        hy.assign(cnt, 0.0f);
        const float parentSurface = BoxSurface(nodeBox);
        Box left = triBoxes[ids[t.lo]], right = triBoxes[ids[t.hi]];
        for (uint32_t i = t.lo; i < t.hi; ++i) {
            left = BoxUnion(left, triBoxes[ids[i]]);
            right = BoxUnion(right, triBoxes[ids[t.hi - i + t.lo]]);
            hx[i - t.lo] = BoxSurface(left) / parentSurface * (float)(int)(i - t.lo + 1);
            hy[t.hi - i - 1] = BoxSurface(right) / parentSurface * (float)(int)(i - t.lo + 1);
        }
        float minCost = std::numeric_limits<float>::infinity();
        uint32_t split = t.lo;
        for (uint32_t i = 0; i < cnt; ++i) {
            const float c = hx[i] + hy[i];
            if (c < minCost) {
                minCost = c;
                split = i + t.lo;
            }
        }
        stack.push_back(Task{split + 1, t.hi, idx, true});
        depthStack.push_back(depth + 1);
        stack.push_back(Task{t.lo, split, idx, false});
        depthStack.push_back(depth + 1);
    }
}

// ComputeSGGXBases (approx_sggx.cpp:156-203): leaves in parallel, then the
// inner nodes children-first (reverse preorder).
void ComputeSggx(const gpugi_bvh& b) {
    const size_t nn = b.nodes.size();
    std::vector<Sggx> s(nn);
    std::vector<uint32_t> leafNodes;
    for (size_t i = 0; i < nn; ++i)
        if (b.nodes[i].left & 0x80000000u) leafNodes.push_back((uint32_t)i);
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&, t]() {
            for (size_t k = t; k < leafNodes.size(); k += nt) {
                const uint32_t i = leafNodes[k];
                s[i] = LeafSggx(b, b.nodes[i].left & 0x7FFFFFFFu);
            }
        });
    for (auto& th : pool) th.join();
    for (size_t ii = nn; ii-- > 0;) {
        const uint32_t left = b.nodes[ii].left;
        if (left & 0x80000000u) continue;
        const uint32_t right = b.escapes[left];
        float lw = NodeSurface(b, left), rw = NodeSurface(b, right);
        const float wsum = lw + rw;
        lw /= wsum;
        rw /= wsum;
        const Sggx &l = s[left], &r = s[right];
        s[ii] = Sggx{l.xx * lw + r.xx * rw, l.xy * lw + r.xy * rw, l.xz * lw + r.xz * rw,
                     l.yy * lw + r.yy * rw, l.yz * lw + r.yz * rw, l.zz * lw + r.zz * rw};
    }
    b.sggx.resize(6 * nn);
    for (size_t i = 0; i < nn; ++i) PackSggx(s[i], &b.sggx[6 * i]);
}


// --- Oriented-box fit (GPUGI_FIT_OBOX) -------------------------------------
// The reference walks oriented-box hierarchies (FetchIntersectOBoxNode,
// intersectiontests.glsl:114-128; OBOX_BVH, traceray.glsl:68-70) that the
// missing Bim library supplies; bvhmake itself fits only boxes and
// ellipsoids. This fit refits the built topology: every node's box around
// the vertices of the triangles below it. The orientation is the principal
// axes of those points (the covariance's eigenvectors, cyclic Jacobi in
// double, right-handed); the extents are measured with the shader's own
// float rotation, rotate(p - centre, rotationInv), and widened until every
// point lies inside in that arithmetic, plus a margin of 2^-16 of the
// extent and 2^-20 of the coordinates' magnitude for the rounding of ray
// transforms. Each node is fitted to all vertices below it (an inner node
// around its children's boxes would grow level by level).

// rotate(x, q) (intersectiontests.glsl:82-89), float, in the shader's order.
V3 QRotate(V3 x, const float q[4]) {
    const V3 t = Cross(V3(q[0], q[1], q[2]), x);
    const V3 u((q[3] * t.x + q[1] * t.z) - q[2] * t.y, (q[3] * t.y + q[2] * t.x) - q[0] * t.z,
               (q[3] * t.z + q[0] * t.y) - q[1] * t.x);
    return x + u * 2.0f;
}

OBox FitOBox(const std::vector<V3>& pts) {
    const size_t n = pts.size();
    double mean[3] = {0, 0, 0};
    for (const V3& v : pts)
        for (int k = 0; k < 3; ++k) mean[k] += v[k];
    for (int k = 0; k < 3; ++k) mean[k] /= (double)n;
    double cov[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (const V3& v : pts)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) cov[r][c] += ((double)v[r] - mean[r]) * ((double)v[c] - mean[c]);
    double m[3][3];  // rows: box axes in world space (world -> box frame)
    SymmetricEigen3(cov, m);
    const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                       m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                       m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    if (det < 0.0)
        for (int k = 0; k < 3; ++k) m[2][k] = -m[2][k];
    // quaternion of the rotation matrix m (Shepperd's method)
    double q[4];
    const double tr = m[0][0] + m[1][1] + m[2][2];
    if (tr > 0.0) {
        const double sq = std::sqrt(tr + 1.0) * 2.0;
        q[3] = 0.25 * sq;
        q[0] = (m[2][1] - m[1][2]) / sq;
        q[1] = (m[0][2] - m[2][0]) / sq;
        q[2] = (m[1][0] - m[0][1]) / sq;
    } else if (m[0][0] > m[1][1] && m[0][0] > m[2][2]) {
        const double sq = std::sqrt(1.0 + m[0][0] - m[1][1] - m[2][2]) * 2.0;
        q[3] = (m[2][1] - m[1][2]) / sq;
        q[0] = 0.25 * sq;
        q[1] = (m[0][1] + m[1][0]) / sq;
        q[2] = (m[0][2] + m[2][0]) / sq;
    } else if (m[1][1] > m[2][2]) {
        const double sq = std::sqrt(1.0 + m[1][1] - m[0][0] - m[2][2]) * 2.0;
        q[3] = (m[0][2] - m[2][0]) / sq;
        q[0] = (m[0][1] + m[1][0]) / sq;
        q[1] = 0.25 * sq;
        q[2] = (m[1][2] + m[2][1]) / sq;
    } else {
        const double sq = std::sqrt(1.0 + m[2][2] - m[0][0] - m[1][1]) * 2.0;
        q[3] = (m[1][0] - m[0][1]) / sq;
        q[0] = (m[0][2] + m[2][0]) / sq;
        q[1] = (m[1][2] + m[2][1]) / sq;
        q[2] = 0.25 * sq;
    }
    const double qn = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    OBox o;
    for (int k = 0; k < 4; ++k) o.qInv[k] = (float)(q[k] / qn);
    const float qFwd[4] = {-o.qInv[0], -o.qInv[1], -o.qInv[2], o.qInv[3]};
    const V3 c0((float)mean[0], (float)mean[1], (float)mean[2]);
    V3 lo(INFINITY, INFINITY, INFINITY), hi(-INFINITY, -INFINITY, -INFINITY);
    float mag = 0.0f;
    for (const V3& v : pts) {
        const V3 l = QRotate(v - c0, o.qInv);
        lo = vmin(lo, l);
        hi = vmax(hi, l);
        mag = std::fmax(mag, std::fmax(std::fabs(v.x), std::fmax(std::fabs(v.y), std::fabs(v.z))));
    }
    o.center = c0 + QRotate((lo + hi) * 0.5f, qFwd);
    V3 h = (hi - lo) * 0.5f;
    for (const V3& v : pts) {  // every point inside in the shader's arithmetic
        const V3 l = QRotate(v - o.center, o.qInv);
        for (int k = 0; k < 3; ++k) h[k] = std::fmax(h[k], std::fabs(l[k]));
    }
    const float ext = std::fmax(h.x, std::fmax(h.y, h.z));
    const float pad = ext * (1.0f / 65536.0f) + mag * (1.0f / 1048576.0f) + 1e-30f;
    for (int k = 0; k < 3; ++k) o.halfSides[k] = h[k] + pad;
    return o;
}

void FitOBoxes(gpugi_bvh& b) {
    const size_t nn = b.nodes.size();
    b.oboxes.assign(nn, OBox{});
    // The leaf blocks below a node are contiguous (blocks are allocated in
    // the order of the preorder walk): a node's box is fitted to the
    // vertices of all of them.
    std::vector<uint32_t> lo(nn), hi(nn);
    for (size_t i = nn; i-- > 0;) {
        const Node& nd = b.nodes[i];
        if (nd.left & 0x80000000u) {
            lo[i] = hi[i] = nd.left & 0x7FFFFFFFu;
        } else {
            lo[i] = std::min(lo[nd.left], lo[nd.right]);
            hi[i] = std::max(hi[nd.left], hi[nd.right]);
        }
    }
    const unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t) {
        pool.emplace_back([&]() {
            std::vector<V3> pts;
            for (size_t i = next++; i < nn; i = next++) {
                pts.clear();
                for (uint64_t sIdx = (uint64_t)lo[i] * b.leafSize; sIdx < ((uint64_t)hi[i] + 1) * b.leafSize; ++sIdx) {
                    const uint32_t* slot = &b.leaves[4 * sIdx];
                    if (slot[0] == slot[1]) continue;
                    for (int c = 0; c < 3; ++c) pts.push_back(b.Pos(slot[c]));
                }
                b.oboxes[i] = FitOBox(pts);
            }
        });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

const char* gpugi_bvh_last_error(void) { return g_lastError.c_str(); }

int gpugi_bvh_sggx(const gpugi_bvh* b, uint16_t* out) {
    if (!b || !out) return -1;
    if (b->sggx.size() != 6 * b->nodes.size()) {
        if (b->normals.size() != b->positions.size()) {
            g_lastError = "node NDFs need the vertex normals (gpugi_bvh_set_vertex_attributes)";
            return -2;
        }
        try {
            ComputeSggx(*b);
        } catch (const std::exception& e) {
            g_lastError = e.what();
            return -3;
        }
    }
    std::memcpy(out, b->sggx.data(), b->sggx.size() * sizeof(uint16_t));
    return 0;
}

int gpugi_bvh_build(const float* positions, uint32_t numVertices, const uint32_t* triangles,
                    uint32_t numTriangles, uint32_t buildMethod, uint32_t fitMethod,
                    uint32_t leafSize, uint64_t seed, gpugi_bvh** out) {
    if (!out) return -1;
    *out = nullptr;
    if (!positions || !triangles || numTriangles == 0 || numVertices == 0) {
        g_lastError = "empty scene: a hierarchy needs at least one triangle";
        return -2;
    }
    if (leafSize < 1 || leafSize > 64) {
        g_lastError = "leafSize must be in [1, 64]";
        return -3;
    }
    if (buildMethod > GPUGI_BUILD_LDS || fitMethod > GPUGI_FIT_OBOX) {
        g_lastError = "unknown build or fit method";
        return -4;
    }
    for (uint64_t i = 0; i < (uint64_t)numTriangles * 4; ++i) {
        if (i % 4 != 3 && triangles[i] >= numVertices) {
            g_lastError = "triangle references a vertex out of range";
            return -5;
        }
        if (i % 4 == 0 && triangles[i] == triangles[i + 1]) {
            g_lastError = "degenerate index triangle (v0 == v1 marks padding in leaf blocks)";
            return -6;
        }
    }
    try {
        std::unique_ptr<gpugi_bvh> b(new gpugi_bvh());
        b->positions.assign(positions, positions + 3 * (size_t)numVertices);
        b->triangles.assign(triangles, triangles + 4 * (size_t)numTriangles);
        b->leafSize = leafSize;
        b->boundsKind = fitMethod;
        if (buildMethod == GPUGI_BUILD_SWEEP) BuildSweep(*b);
        else if (buildMethod == GPUGI_BUILD_LDS) BuildLds(*b);
        else BuildKdtree(*b);
        if (b->nodes.size() >= 0x80000000u) {
            g_lastError = "scene too large: the node index MSB is the leaf flag";
            return -7;
        }
        AssignEscapes(*b);
        if (fitMethod == GPUGI_FIT_ELLIPSOID) FitEllipsoids(*b, seed);
        if (fitMethod == GPUGI_FIT_OBOX) FitOBoxes(*b);
        *out = b.release();
        return 0;
    } catch (const std::exception& e) {
        g_lastError = e.what();
        return -8;
    }
}

int gpugi_bvh_info(const gpugi_bvh* b, uint32_t* numNodes, uint32_t* numLeafBlocks,
                   uint32_t* leafSize, uint32_t* boundsKind, uint32_t* maxDepth) {
    if (!b) return -1;
    if (numNodes) *numNodes = (uint32_t)b->nodes.size();
    if (numLeafBlocks) *numLeafBlocks = (uint32_t)(b->leaves.size() / (4 * b->leafSize));
    if (leafSize) *leafSize = b->leafSize;
    if (boundsKind) *boundsKind = b->boundsKind;
    if (maxDepth) *maxDepth = b->maxDepth;
    return 0;
}

int gpugi_bvh_export(const gpugi_bvh* b, float* hierarchy, int32_t* slots, uint32_t* parents) {
    if (!b) return -1;
    const size_t nn = b->nodes.size();
    if (hierarchy && b->boundsKind == GPUGI_FIT_OBOX) {
        // Scene::TreeNode<OBox>: {center, firstChild}, {sidesHalf, escape}, rotationInv
        for (size_t i = 0; i < nn; ++i) {
            float* o = hierarchy + 12 * i;
            const OBox& ob = b->oboxes[i];
            uint32_t fc = b->nodes[i].left, esc = b->escapes[i];
            o[0] = ob.center.x; o[1] = ob.center.y; o[2] = ob.center.z; std::memcpy(&o[3], &fc, 4);
            o[4] = ob.halfSides.x; o[5] = ob.halfSides.y; o[6] = ob.halfSides.z; std::memcpy(&o[7], &esc, 4);
            for (int k = 0; k < 4; ++k) o[8 + k] = ob.qInv[k];
        }
    } else if (hierarchy) {
        for (size_t i = 0; i < nn; ++i) {
            float* o = hierarchy + 8 * i;
            V3 a, c;
            if (b->boundsKind == GPUGI_FIT_ELLIPSOID) {
                a = b->ellipsoids[i].center;
                c = b->ellipsoids[i].radii;
            } else {
                a = b->boxes[i].min;
                c = b->boxes[i].max;
            }
            uint32_t fc = b->nodes[i].left, esc = b->escapes[i];
            o[0] = a.x; o[1] = a.y; o[2] = a.z; std::memcpy(&o[3], &fc, 4);
            o[4] = c.x; o[5] = c.y; o[6] = c.z; std::memcpy(&o[7], &esc, 4);
        }
    }
    if (slots) std::memcpy(slots, b->leaves.data(), b->leaves.size() * sizeof(uint32_t));
    if (parents) std::memcpy(parents, b->parents.data(), nn * sizeof(uint32_t));
    return 0;
}

void gpugi_bvh_free(gpugi_bvh* b) { delete b; }

// --- NamedArray file (documentation/fileformat.tex; bvhmake/filedef.hpp:8-54) ---
namespace {
struct NamedArray {
    char name[32];
    uint32_t numElements;
    uint32_t elementSize;
};
static_assert(sizeof(NamedArray) == 40, "NamedArray header is 40 bytes");

bool WriteChunk(FILE* f, const char* name, uint32_t num, uint32_t size, const void* data) {
    NamedArray h;
    std::memset(&h, 0, sizeof(h));
    std::strncpy(h.name, name, 31);
    h.numElements = num;
    h.elementSize = size;
    return std::fwrite(&h, sizeof(h), 1, f) == 1 &&
           (num == 0 || std::fwrite(data, (size_t)size, num, f) == num);
}
}  // namespace

int gpugi_bvh_write_file(const gpugi_bvh* b, const char* path) {
    if (!b || !path) return -1;
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        g_lastError = std::string("cannot open for writing: ") + path;
        return -2;
    }
    const uint32_t nv = (uint32_t)(b->positions.size() / 3), nn = (uint32_t)b->nodes.size();
    // "vertices": {position, normal, texcoord} = 32 bytes (filedef.hpp:15-20).
    std::vector<float> verts((size_t)nv * 8, 0.0f);
    const bool haveN = b->normals.size() == 3 * (size_t)nv, haveT = b->texcoords.size() == 2 * (size_t)nv;
    for (uint32_t v = 0; v < nv; ++v) {
        for (int k = 0; k < 3; ++k) verts[8 * (size_t)v + k] = b->positions[3 * (size_t)v + k];
        for (int k = 0; k < 3 && haveN; ++k) verts[8 * (size_t)v + 3 + k] = b->normals[3 * (size_t)v + k];
        for (int k = 0; k < 2 && haveT; ++k) verts[8 * (size_t)v + 6 + k] = b->texcoords[2 * (size_t)v + k];
    }
    // "hierarchy": {parent, firstChild, escape} (filedef.hpp:41-46).
    std::vector<uint32_t> hier((size_t)nn * 3);
    for (uint32_t i = 0; i < nn; ++i) {
        hier[3 * (size_t)i] = b->parents[i];
        hier[3 * (size_t)i + 1] = b->nodes[i].left;
        hier[3 * (size_t)i + 2] = b->escapes[i];
    }
    std::vector<float> bv((size_t)nn * 6);
    for (uint32_t i = 0; i < nn; ++i) {
        V3 a = b->boundsKind == GPUGI_FIT_ELLIPSOID ? b->ellipsoids[i].center : b->boxes[i].min;
        V3 c = b->boundsKind == GPUGI_FIT_ELLIPSOID ? b->ellipsoids[i].radii : b->boxes[i].max;
        for (int k = 0; k < 3; ++k) {
            bv[6 * (size_t)i + k] = a[k];
            bv[6 * (size_t)i + 3 + k] = c[k];
        }
    }
    // oriented boxes: {center, halfSides, orientation quaternion x y z w}, 40 B
    // (the fields Scene::UploadHierarchy reads, scene.cpp:113-115; the GPU
    // node holds the conjugate)
    std::vector<float> ob;
    if (b->boundsKind == GPUGI_FIT_OBOX) {
        ob.resize((size_t)nn * 10);
        for (uint32_t i = 0; i < nn; ++i) {
            const OBox& o = b->oboxes[i];
            float* e = &ob[10 * (size_t)i];
            for (int k = 0; k < 3; ++k) {
                e[k] = o.center[k];
                e[3 + k] = o.halfSides[k];
                e[6 + k] = -o.qInv[k];
            }
            e[9] = o.qInv[3];
        }
    }
    const uint32_t nBlocks = (uint32_t)(b->leaves.size() / (4 * b->leafSize));
    bool ok = WriteChunk(f, "vertices", nv, 32, verts.data()) &&
              (b->boundsKind == GPUGI_FIT_OBOX
                   ? WriteChunk(f, "bounding_obox", nn, 40, ob.data())
                   : WriteChunk(f, b->boundsKind == GPUGI_FIT_ELLIPSOID ? "bounding_ellipsoid" : "bounding_aabox", nn,
                                24, bv.data())) &&
              WriteChunk(f, "hierarchy", nn, 12, hier.data()) &&
              WriteChunk(f, "triangles", nBlocks, 16 * b->leafSize, b->leaves.data()) &&
              (b->materials.empty() ||
               WriteChunk(f, "gpugi_materials", (uint32_t)(b->materials.size() / 24), 96, b->materials.data()));
    // bvhmake's main writes the node NDFs after the hierarchy (main.cpp:143-144)
    if (ok && (b->sggx.size() == 6 * (size_t)nn || b->normals.size() == 3 * (size_t)nv)) {
        if (b->sggx.size() != 6 * (size_t)nn) ComputeSggx(*b);
        ok = WriteChunk(f, "approx_sggx", nn, 12, b->sggx.data());
    }
    if (ok && !b->materialNames.empty()) {
        std::vector<char> names(b->materialNames.size() * 32, 0);
        for (size_t i = 0; i < b->materialNames.size(); ++i)
            std::strncpy(&names[32 * i], b->materialNames[i].c_str(), 31);
        ok = WriteChunk(f, "materialref", (uint32_t)b->materialNames.size(), 32, names.data());
    }
    std::fclose(f);
    if (!ok) {
        g_lastError = "short write";
        return -3;
    }
    return 0;
}

int gpugi_bvh_read_file(const char* path, gpugi_bvh** out) {
    if (!path || !out) return -1;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        g_lastError = std::string("cannot open: ") + path;
        return -2;
    }
    std::unique_ptr<gpugi_bvh> b(new gpugi_bvh());
    std::vector<uint32_t> hier;
    std::vector<float> bv, ob;
    bool haveBV = false, haveTris = false, haveHier = false;
    NamedArray h;
    int rc = 0;
    while (std::fread(&h, sizeof(h), 1, f) == 1) {
        h.name[31] = 0;
        const uint64_t bytes = (uint64_t)h.numElements * h.elementSize;
        std::string name(h.name);
        std::vector<char> data(bytes);
        if (bytes && std::fread(data.data(), 1, bytes, f) != bytes) { rc = -3; g_lastError = "truncated chunk " + name; break; }
        if (name == "vertices") {
            if (h.elementSize < 12) { rc = -4; g_lastError = "vertices element too small"; break; }
            b->positions.resize((size_t)h.numElements * 3);
            for (uint32_t v = 0; v < h.numElements; ++v)
                std::memcpy(&b->positions[3 * (size_t)v], &data[(size_t)v * h.elementSize], 12);
            if (h.elementSize >= 32) {
                b->normals.resize((size_t)h.numElements * 3);
                b->texcoords.resize((size_t)h.numElements * 2);
                for (uint32_t v = 0; v < h.numElements; ++v) {
                    std::memcpy(&b->normals[3 * (size_t)v], &data[(size_t)v * h.elementSize + 12], 12);
                    std::memcpy(&b->texcoords[2 * (size_t)v], &data[(size_t)v * h.elementSize + 24], 8);
                }
            }
        } else if (name == "materialref") {
            if (h.elementSize != 32) { rc = -4; g_lastError = "materialref element must be 32 bytes"; break; }
            b->materialNames.clear();
            for (uint32_t i = 0; i < h.numElements; ++i) {
                char nm[33];
                std::memcpy(nm, &data[32 * (size_t)i], 32);
                nm[32] = 0;
                b->materialNames.emplace_back(nm);
            }
        } else if (name == "gpugi_materials") {
            if (h.elementSize != 96) { rc = -4; g_lastError = "gpugi_materials element must be 96 bytes"; break; }
            b->materials.resize((size_t)h.numElements * 24);
            std::memcpy(b->materials.data(), data.data(), bytes);
        } else if (name == "approx_sggx") {
            if (h.elementSize != 12) { rc = -4; g_lastError = "approx_sggx element must be 12 bytes"; break; }
            b->sggx.resize((size_t)h.numElements * 6);
            std::memcpy(b->sggx.data(), data.data(), bytes);
        } else if (name == "hierarchy") {
            if (h.elementSize != 12) { rc = -4; g_lastError = "hierarchy element must be 12 bytes"; break; }
            hier.resize((size_t)h.numElements * 3);
            std::memcpy(hier.data(), data.data(), bytes);
            haveHier = true;
        } else if (name == "bounding_aabox" || name == "bounding_ellipsoid") {
            if (h.elementSize != 24) { rc = -4; g_lastError = "bounding volume element must be 24 bytes"; break; }
            b->boundsKind = name == "bounding_aabox" ? GPUGI_FIT_AABOX : GPUGI_FIT_ELLIPSOID;
            bv.resize((size_t)h.numElements * 6);
            std::memcpy(bv.data(), data.data(), bytes);
            haveBV = true;
        } else if (name == "bounding_obox") {
            if (h.elementSize != 40) { rc = -4; g_lastError = "oriented box element must be 40 bytes"; break; }
            b->boundsKind = GPUGI_FIT_OBOX;
            ob.resize((size_t)h.numElements * 10);
            std::memcpy(ob.data(), data.data(), bytes);
            bv.assign((size_t)h.numElements * 6, 0.0f);
            haveBV = true;
        } else if (name == "triangles") {
            if (h.elementSize == 0 || h.elementSize % 16 != 0) { rc = -4; g_lastError = "triangles block size"; break; }
            b->leafSize = h.elementSize / 16;  // leaf size comes from the file
            b->leaves.resize(bytes / 4);
            std::memcpy(b->leaves.data(), data.data(), bytes);
            haveTris = true;
        }  // other chunks are skipped, as the format allows
    }
    std::fclose(f);
    if (rc) return rc;
    if (!haveBV || !haveTris || !haveHier || hier.size() / 3 != bv.size() / 6) {
        g_lastError = "file lacks hierarchy, bounding volumes or triangles";
        return -5;
    }
    if (!b->sggx.empty() && b->sggx.size() != hier.size() * 2) {
        g_lastError = "approx_sggx does not have one record per node";
        return -5;
    }
    const size_t nn = hier.size() / 3;
    b->nodes.resize(nn);
    b->escapes.resize(nn);
    b->parents.resize(nn);
    b->boxes.resize(nn);
    if (b->boundsKind == GPUGI_FIT_ELLIPSOID) b->ellipsoids.resize(nn);
    if (b->boundsKind == GPUGI_FIT_OBOX) {
        b->oboxes.resize(nn);
        for (size_t i = 0; i < nn; ++i) {
            const float* e = &ob[10 * i];
            OBox& o = b->oboxes[i];
            for (int k = 0; k < 3; ++k) {
                o.center[k] = e[k];
                o.halfSides[k] = e[3 + k];
                o.qInv[k] = -e[6 + k];
            }
            o.qInv[3] = e[9];
        }
    }
    for (size_t i = 0; i < nn; ++i) {
        b->parents[i] = hier[3 * i];
        b->nodes[i].left = hier[3 * i + 1];
        b->escapes[i] = hier[3 * i + 2];
        V3 a(bv[6 * i], bv[6 * i + 1], bv[6 * i + 2]), c(bv[6 * i + 3], bv[6 * i + 4], bv[6 * i + 5]);
        if (b->boundsKind == GPUGI_FIT_ELLIPSOID) b->ellipsoids[i] = Ellipsoid{a, c};
        else b->boxes[i] = Box{a, c};
    }
    *out = b.release();
    return 0;
}

int gpugi_bvh_vertices(const gpugi_bvh* b, uint32_t* numVertices, float* positions) {
    if (!b) return -1;
    if (numVertices) *numVertices = (uint32_t)(b->positions.size() / 3);
    if (positions) std::memcpy(positions, b->positions.data(), b->positions.size() * sizeof(float));
    return 0;
}

int gpugi_bvh_set_vertex_attributes(gpugi_bvh* b, const float* normals, const float* texcoords) {
    if (!b) return -1;
    const size_t nv = b->positions.size() / 3;
    if (normals) b->normals.assign(normals, normals + 3 * nv);
    else b->normals.clear();
    b->sggx.clear();  // the node NDFs follow the normals
    if (texcoords) b->texcoords.assign(texcoords, texcoords + 2 * nv);
    else b->texcoords.clear();
    return 0;
}

int gpugi_bvh_vertex_attributes(const gpugi_bvh* b, float* normals, float* texcoords) {
    if (!b) return -1;
    const size_t nv = b->positions.size() / 3;
    if (normals) {
        if (b->normals.size() == 3 * nv) std::memcpy(normals, b->normals.data(), 3 * nv * sizeof(float));
        else std::memset(normals, 0, 3 * nv * sizeof(float));
    }
    if (texcoords) {
        if (b->texcoords.size() == 2 * nv) std::memcpy(texcoords, b->texcoords.data(), 2 * nv * sizeof(float));
        else std::memset(texcoords, 0, 2 * nv * sizeof(float));
    }
    return 0;
}

int gpugi_bvh_set_material_names(gpugi_bvh* b, const char* const* names, uint32_t numNames) {
    if (!b || (numNames && !names)) return -1;
    b->materialNames.clear();
    for (uint32_t i = 0; i < numNames; ++i) {
        if (!names[i] || std::strlen(names[i]) > 31) {
            g_lastError = "material names must be 1-31 characters";
            return -2;
        }
        b->materialNames.emplace_back(names[i]);
    }
    return 0;
}

const char* gpugi_bvh_material_name(const gpugi_bvh* b, uint32_t index) {
    return (b && index < b->materialNames.size()) ? b->materialNames[index].c_str() : nullptr;
}

uint32_t gpugi_bvh_num_material_names(const gpugi_bvh* b) { return b ? (uint32_t)b->materialNames.size() : 0; }

int gpugi_bvh_set_materials(gpugi_bvh* b, const float* records, uint32_t numMaterials) {
    if (!b || (numMaterials && !records)) return -1;
    b->materials.assign(records, records + 24 * (size_t)numMaterials);
    return 0;
}

int gpugi_bvh_materials(const gpugi_bvh* b, uint32_t* numMaterials, float* records) {
    if (!b) return -1;
    if (numMaterials) *numMaterials = (uint32_t)(b->materials.size() / 24);
    if (records && !b->materials.empty())
        std::memcpy(records, b->materials.data(), b->materials.size() * sizeof(float));
    return 0;
}

}  // extern "C"
