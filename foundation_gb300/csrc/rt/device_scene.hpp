// device_scene.hpp — plain (host-compilable) types shared by the traversal
// kernels and the host launch code.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../../include/fnd_rt.h"

namespace Foundation {
namespace RT {

// Device status bits (latched, read back by fnd_rt_sync).
constexpr uint32_t kStatusStackOverflow = 1u;
constexpr uint32_t kStatusTimeout = 2u;
constexpr uint32_t kStatusBadIndex = 4u;  // node / triangle index outside the scene arrays

// The fnd_status a latched status word reports (the first that applies):
// stack overflow, then a timed-out wait, then a bad index; an unknown bit
// is reported as a CUDA failure. Every entry point that reads a status word
// maps it through here.
inline int StatusCode(uint32_t bits) {
    if (bits == 0u) return FND_OK;
    if (bits & kStatusStackOverflow) return FND_ERR_STACK_OVERFLOW;
    if (bits & kStatusTimeout) return FND_ERR_TIMEOUT;
    if (bits & kStatusBadIndex) return FND_ERR_INVALID_SCENE;
    return FND_ERR_CUDA;
}

constexpr int kMaxStack = 64;  // node-group + triangle-group entries per ray

struct DeviceScene {
    const uint4* nodes;  // 5 uint4 per WideNode
    const float4* v0;    // (x, y, z, original index bits)
    const float4* v1;
    const float4* v2;
    uint32_t num_nodes;
    uint32_t num_tris;
};

// One instance of a two-level scene (104 bytes): its bottom-level scene, the
// world-to-object transform (row-major 3x4, FP32 rounding of the FP64
// inverse of the instance transform) and the hit id of its triangle 0.
struct InstanceRec {
    DeviceScene blas;
    float inv[12];
    uint32_t prim_offset;
    uint32_t flags;  // kInstanceIdentity: inv is [I | 0] bit for bit
    uint32_t pad[2];
};
// An identity instance keeps the world ray and its set-up (the transform
// would change at most the sign of zero components); the oracle's instanced
// brute force makes the same choice.
constexpr uint32_t kInstanceIdentity = 1u;
static_assert(sizeof(InstanceRec) == 104, "instance record layout");

}  // namespace RT
}  // namespace Foundation
