// wide_bvh.hpp — compressed 8-wide BVH and the triangle arrays the traversal
// kernels read. Shared by the host collapser and the device code.
//
// Node (80 bytes, 16-byte aligned, fetched as five 16-byte vectors):
//   bytes  0..11  p[3]        float origin of the child-box quantisation grid
//   bytes 12..14  e[3]        biased exponents: grid step along axis a is
//                             2^(e[a] - 127), so decoding is exact scaling
//   byte  15      imask       bit s set: slot s holds an internal child
//   bytes 16..19  child_base  index of the first internal child; the internal
//                             child in slot s is child_base + popc(imask & ((1<<s)-1))
//   bytes 20..23  tri_base    index of the first triangle of this node's leaves
//   bytes 24..31  meta[8]     0: empty slot; 0x01: internal child;
//                             leaf: 0x80 | (count-1) << 5 | offset, its triangles
//                             are tri_base + offset .. + count - 1 (count <= 4)
//   bytes 32..55  qlo[3][8]   child box lower corners (x[8], y[8], z[8]), uint8
//   bytes 56..79  qhi[3][8]   child box upper corners
// Child box: p + 2^e * q, quantised outward (floor / ceil) after every box
// was inflated by the scene margin, so decoded boxes enclose their contents
// with room for the FP32 rounding of the slab test.
//
// Slot order: slot s holds the child whose centroid lies most towards the
// corner with signs (bit a of s) ? + : - (greedy assignment). A ray with
// direction-sign bits oct (bit a set when dir[a] < 0) visits slots in the
// order s = i ^ oct for i = 0..7, which is near-to-far along its octant.
//
// Triangles: three float4 arrays ("vertex planes"), one entry per triangle in
// leaf order: v0 = (x, y, z, original index as bits), v1 = (x, y, z, 0),
// v2 = (x, y, z, 0).
#pragma once

#include <cstdint>

namespace Foundation {
namespace RT {

struct alignas(16) WideNode {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "wide node is five 16-byte vectors");

constexpr uint8_t kMetaInternal = 0x01;
constexpr uint8_t kMetaLeafFlag = 0x80;
constexpr int kWidth = 8;
constexpr int kMaxLeafTris = 4;

}  // namespace RT
}  // namespace Foundation
