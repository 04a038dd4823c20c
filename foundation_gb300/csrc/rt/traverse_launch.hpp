// traverse_launch.hpp — host-visible launch interface of the traversal kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../../include/fnd_rt.h"
#include "device_scene.hpp"

namespace Foundation {
namespace RT {

constexpr int kTraceBlock = 128;     // threads per block (4 warps)
constexpr int kTraceShortStack = 8;  // stack entries per thread kept in shared memory

struct TraceLaunch {
    DeviceScene scene;
    const float4* rays;  // 2 float4 per fnd_ray
    uint32_t n;              // ray count, or the capacity when n_dev is set
    const uint32_t* n_dev;   // device-side ray count (a queue length), or null
    unsigned long long* ray_total;  // if set, the launch adds its ray count here
    void* hits;          // fnd_hit[n] (closest)
    uint8_t* occluded;   // uint8[n]   (any)
    uint32_t* counter;   // work-queue counter (zeroed before each launch)
    uint32_t* status;    // latched kStatus* bits
    unsigned long long* stats;  // [0] node fetches, [1] triangle tests (stats variants)
    uint32_t refill_min;        // refill a warp once this many lanes are idle
};

// variant: 0 closest, 1 any, 2 closest+stats, 3 any+stats
cudaError_t TraceOccupancy(int variant, int* blocks_per_sm);
cudaError_t LaunchTrace(const TraceLaunch& L, bool any, bool stats, int grid, cudaStream_t stream);

}  // namespace RT
}  // namespace Foundation
