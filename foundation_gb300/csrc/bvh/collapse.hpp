// collapse.hpp — binary BVH -> compressed 8-wide BVH + triangle vertex planes.
#pragma once

#include <cstdint>
#include <memory>
#include <new>
#include <utility>
#include <vector>

#include "bvh_build.hpp"
#include "wide_bvh.hpp"

namespace Foundation {
namespace RT {

using PlaneVector = std::vector<float, NoInitAllocator<float>>;

struct WideBvh {
    std::vector<WideNode> nodes;
    PlaneVector v0, v1, v2;  // 4 floats per triangle each (see wide_bvh.hpp)
    uint32_t depth = 0;             // wide levels on the longest root-to-leaf path
    uint32_t leaves = 0;
    float margin = 0.0f;            // absolute outward inflation of every box
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

// Absolute box inflation that keeps the FP32 slab test conservative: 2^-16 of
// the largest of |coordinate| and extent over the scene bounds. It covers the
// rounding of (p - o) * inv_dir for ray origins within about 50x that size.
float SceneMargin(const float lo[3], const float hi[3]);

struct CollapseOptions {
    bool sah = false;       // SAH-optimal collapse instead of the greedy one
    double c_node = 1.0;    // its cost of a wide-node visit per unit of half area
    double c_tri = 0.3;     // and of a triangle test (the kernel's best of 0.05 - 1)
    uint32_t threads = 0;   // host threads; 0: all cores. The output does not depend on it
    uint32_t width = 8;     // children per wide node, 2..8 (the record always has 8 slots)
};

// Greedy collapse (largest-surface-area internal child expanded first until
// opt.width children) or SAH-optimal collapse (opt.sah), octant-ordered slot assignment,
// 8-bit outward quantisation; wide nodes in breadth-first order, computed a
// level at a time on opt.threads threads. margin_scale multiplies SceneMargin (a
// bottom-level scene whose instances shrink it far below the world's size
// needs a wider margin: its object-space ray origins lie further away, see
// fnd_rt_instances_upload).
void CollapseToWide(const BinaryBvh& bin, const float* tri, uint32_t nt, WideBvh& out, float margin_scale = 1.0f,
                    const CollapseOptions& opt = CollapseOptions{});

}  // namespace RT
}  // namespace Foundation
