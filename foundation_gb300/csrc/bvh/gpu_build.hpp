// gpu_build.hpp — BVH construction on the GPU (gpu_build.cu).
//
// Same output format as the host builder + collapse (wide_bvh.hpp), built in
// device memory: linear BVH over 63-bit Morton codes of the triangle
// centroids (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012) with a stable LSD radix sort, a
// bottom-up refit that also takes the SAH leaf decision (subtrees of at most
// max_leaf triangles become one leaf when that is not more expensive), and
// the greedy or the SAH-optimal 8-wide collapse of collapse.cpp run level by
// level on the device, with the same margin and outward quantisation. Hits are identical
// to any other valid BVH over the same triangles; the tree itself differs
// from the binned-SAH tree.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace Foundation {
namespace RT {

constexpr uint32_t kGpuBuildMaxTris = 1u << 27;  // radix-sort scan capacity

struct GpuBuildParams {
    uint32_t max_leaf = 4;
    float trav_cost = 1.0f;
    float margin_scale = 1.0f;
    bool sah_collapse = false;  // SAH-optimal collapse (collapse.hpp) instead of the greedy one
    float c_tri = 0.3f;         // its cost of a triangle test relative to a wide-node visit
    uint32_t width = 8;         // children per wide node, 2..8
    uint32_t ploc_radius = 0;   // binary tree by locally-ordered clustering with this search radius
                                // (1..64); 0: Karras hierarchy
};

struct GpuBuildOutput {
    void* d_nodes = nullptr;      // WideNode[num_nodes], exact size
    void* d_tris = nullptr;       // three float4 planes of num_refs entries
    void* d_tri_shade = nullptr;  // float4 per triangle: unit normal, material 0
    uint32_t num_nodes = 0, num_refs = 0, depth = 0, leaves = 0, num_binary_nodes = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    float margin = 0.0f;
    double sah_cost = 0.0;  // of the binary tree after the leaf decision, root half-area normalised
    double build_ms = 0.0, collapse_ms = 0.0;
};

// d_verts: 3 * nv floats, d_idx: 3 * nt indices, both device memory. Fails
// (RtCore::FndError) on invalid input: FND_ERR_INVALID_ARG for an index out of
// range or a non-finite coordinate, FND_ERR_INVALID_SCENE when the tree is
// deeper than the traversal stack allows. Temporary buffers are freed.
void BuildWideGpu(const float* d_verts, uint32_t nv, const uint32_t* d_idx, uint32_t nt, const GpuBuildParams& p,
                  GpuBuildOutput& out, cudaStream_t s);

// tri_shade[t].w = material id bits of triangle t.
cudaError_t WriteMaterialIds(float4* d_tri_shade, const uint32_t* d_ids, uint32_t nt, cudaStream_t s);

// Shading records of a two-level scene: for instance i (prefix[i] .. prefix[i+1]
// of the flat triangle range) and its triangle t, the world-space normal
// normalize(inv(A)^T n) of the bottom level's normal n (inv: the instance's
// world-to-object rows, row-major 3x4), written at prim_offset[i] + t with
// material 0.
cudaError_t InstanceShade(const float* d_inv, const uint32_t* d_prefix, const uint32_t* d_prim_offset,
                          const float4* const* d_blas_shade, uint32_t n_inst, uint32_t total, float4* d_out,
                          cudaStream_t s);

}  // namespace RT
}  // namespace Foundation
