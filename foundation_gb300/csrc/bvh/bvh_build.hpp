// bvh_build.hpp — binned-SAH binary BVH over triangles (host, multi-threaded).
//
// Algorithm (Wald 2007, "On fast Construction of SAH-based Bounding Volume
// Hierarchies"): per node, bin triangle bounding-box centroids into K bins
// along each axis with non-zero centroid extent, sweep bin bounds from both
// ends, split where C_trav + C_isect * (A_L N_L + A_R N_R) / A_node is least
// (C_isect = 1, C_trav = trav_cost, 1 by default; half surface areas, first
// minimum wins, axes in x, y, z order); make a leaf when the node holds at
// most max_leaf triangles and the leaf cost N is not above the split cost.
// A larger trav_cost gives fuller leaves, hence fewer binary nodes and
// fuller 8-wide nodes after the collapse; when all centroids of a
// node coincide, split at the median of the triangle indices. The tree this
// produces is a function of the triangle set only (not of thread timing).
#pragma once

#include <cstdint>
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace Foundation {
namespace RT {

// Allocator whose value-initialisation (vector(n), resize(n)) leaves the
// elements uninitialised: the builders and the collapse write every element
// themselves, on several threads, instead of one thread zero-filling
// gigabytes first.
template <class T>
struct NoInitAllocator : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAllocator<U>;
    };
    NoInitAllocator() = default;
    template <class U>
    NoInitAllocator(const NoInitAllocator<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept {
        ::new (static_cast<void*>(p)) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
    }
};
struct Aabb {
    float lo[3], hi[3];
};

struct BinaryNode {
    float lo[3], hi[3];
    uint32_t a;      // internal: left child index (right = a + 1); leaf: first slot in prims
    uint32_t count;  // 0 for internal nodes, triangle count for leaves
};

struct BinaryBvh {
    std::vector<BinaryNode, NoInitAllocator<BinaryNode>> nodes;  // nodes[0] is the root
    std::vector<uint32_t, NoInitAllocator<uint32_t>> prims;      // leaf slots -> original triangle index
    uint32_t depth = 0;
    uint32_t leaves = 0;
    double sah_cost = 0.0;  // normalised by the root half-area
};

struct BuildParams {
    uint32_t bins = 32;
    uint32_t max_leaf = 4;
    uint32_t threads = 0;          // 0: hardware concurrency
    float trav_cost = 1.0f;        // SAH cost of a traversal step relative to a triangle test
    bool spatial_splits = false;   // BuildBinarySbvh only
    float spatial_alpha = 1e-5f;   // try spatial splits when child overlap > alpha x root half area
    double max_refs_factor = 2.0;  // spatial splits add at most this many references per triangle
};

// tri: 9 floats per triangle (v0, v1, v2). nt > 0.
void BuildBinaryBvh(const float* tri, uint32_t nt, const BuildParams& params, BinaryBvh& out);

// Binned SAH with spatial splits (sbvh_build.cpp): leaves may reference a
// triangle more than once; out.prims holds the references. The build threads
// draw on one shared duplicate budget (max_refs_factor): while it lasts the
// tree is a function of the triangle set only; once it runs out, which nodes
// still split spatially depends on thread timing.
void BuildBinarySbvh(const float* tri, uint32_t nt, const BuildParams& params, BinaryBvh& out);

}  // namespace RT
}  // namespace Foundation
