// rt_oracle_internal.hpp — TEST INFRASTRUCTURE ONLY: the oracle's binary
// BVH record, shared by the traversal (rt_oracle.cpp) and the FP64 path
// tracer (pt_oracle.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace oracle {

struct BNode {
    float lo[3], hi[3];
    uint32_t a;      // internal: left child (right = a + 1); leaf: first prim slot
    uint32_t count;  // 0: internal, else number of triangles
};

}  // namespace oracle

struct orc_bvh {
    std::vector<oracle::BNode> nodes;
    std::vector<uint32_t> prims;  // leaf slots -> original triangle index
    std::vector<float> tri;       // 9 floats per original triangle
    uint32_t nt = 0;
    uint32_t depth = 0;
    uint32_t max_leaf = 4;
    double sah = 0.0;
    float margin = 0.0f;
};

namespace oracle {

using BNodeView = BNode;
inline const BNode& node_view(const orc_bvh& b, uint32_t i) { return b.nodes[i]; }
inline uint32_t node_count(const orc_bvh& b) { return (uint32_t)b.nodes.size(); }
inline uint32_t prim_at(const orc_bvh& b, uint32_t slot) { return b.prims[slot]; }
inline const float* tri_at(const orc_bvh& b, uint32_t t) { return &b.tri[9 * (size_t)t]; }
inline uint32_t tri_count(const orc_bvh& b) { return b.nt; }

}  // namespace oracle
