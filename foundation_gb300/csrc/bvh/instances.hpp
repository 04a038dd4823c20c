// instances.hpp — host side of two-level scenes: FP64 inverse transforms
// (rounded to FP32), world boxes of the instances, the top-level tree over
// them (binned SAH on one degenerate triangle per instance spanning its box,
// collapsed to the 8-wide format; a leaf "triangle" index word holds the
// instance id) and the object-space reach used to check bottom-level margins.
#pragma once

#include <cstdint>
#include <vector>

#include "bvh_build.hpp"
#include "collapse.hpp"

namespace Foundation {
namespace RT {

struct InstanceInput {
    float transform[12];  // object -> world, row-major 3x4
    float lo[3], hi[3];   // bounds of the bottom level (object space)
};

struct InstanceTop {
    BinaryBvh bin;
    WideBvh wide;
    std::vector<float> inv;  // 12 per instance: world -> object, row-major 3x4
    double lo[3], hi[3];     // union of the instances' world boxes
};

// Adjugate / determinant in FP64, translation -inv(A) b, each entry rounded to
// FP32. False for a singular or non-finite transform.
bool InstanceInverse(const float* m, float inv[12]);

// Builds the top level; fails (RtCore::FndError) on a singular transform.
void BuildInstanceTop(const InstanceInput* in, uint32_t n, InstanceTop& out);

// Largest |coordinate| of the world box's corners mapped by `inv` (FP64 of the
// FP32 entries): how far object-space ray origins reach for rays that start in
// the world box.
double InstanceReach(const float inv[12], const double lo[3], const double hi[3]);

}  // namespace RT
}  // namespace Foundation
