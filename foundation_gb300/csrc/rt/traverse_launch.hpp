// traverse_launch.hpp — host-visible launch interface of the traversal kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../../include/fnd_rt.h"
#include "device_scene.hpp"

namespace Foundation {
namespace RT {

constexpr int kTraceBlock = 128;     // default threads per block (4 warps)
constexpr int kTraceShortStack = 8;  // default stack entries per thread kept in shared memory

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
    unsigned long long* stats;  // [0] node fetches, [1] triangle tests, [2] / [3] warp steps of the node /
                                // triangle tests (stats variants)
    uint32_t refill_min;        // refill a warp once this many lanes are idle
    uint32_t postpone_min;      // triangle postponement threshold (0: off)
    const uint32_t* order;      // fetch position -> ray index (ray_sort.hpp), or null: input order
};

// Launch shape of a traversal kernel (the autotuner's search space).
struct TraceConfig {
    int block = kTraceBlock;             // 64, 128 or 256 threads
    int short_stack = kTraceShortStack;  // 4, 8 or 16 shared-memory stack entries per thread
    uint32_t refill_min = 8;             // 1..32 idle lanes before a warp refills
    uint32_t postpone_min = 0;           // postpone triangles when fewer lanes have them (0: never)
    int blocks_per_sm = 0;               // 0: as many as fit
    uint32_t sort_bits = 0;              // coherence order key bits (ray_sort.hpp), 0: input order
};
bool ValidTraceConfig(const TraceConfig& c);

// One job of a batched launch: a ray batch against one scene.
struct BatchJob {
    DeviceScene scene;
    const float4* rays;
    void* out;       // fnd_hit* (closest) or uint8_t* (any)
    uint32_t n;
    uint32_t any;    // 0 closest, 1 any
};

struct BatchLaunch {
    const BatchJob* jobs;     // device job table
    const uint32_t* prefix;   // device prefix sums of ray counts (njobs + 1)
    uint32_t njobs;
    uint32_t total;           // sum of ray counts
    uint32_t* counter;
    uint32_t* status;
    uint32_t refill_min;
    uint32_t postpone_min;
};

// Rays against a two-level scene (instances.cu).
struct InstancedLaunch {
    DeviceScene tlas;            // leaves' index words hold instance ids
    const InstanceRec* inst;
    uint32_t num_inst;
    const float4* rays;
    uint32_t n;                  // ray count, or the capacity when n_dev is set
    const uint32_t* n_dev;       // device-side ray count (a queue length), or null
    unsigned long long* ray_total;  // if set, the launch adds its ray count here
    void* hits;                  // fnd_hit[n] (closest)
    uint8_t* occluded;           // uint8[n]   (any)
    uint32_t* counter;
    uint32_t* status;
};
cudaError_t LaunchInstanced(const InstancedLaunch& L, bool any, int sm_count, cudaStream_t stream);

// variant: 0 closest, 1 any, 2 closest+stats, 3 any+stats, 4 batch
cudaError_t TraceOccupancy(int variant, int* blocks_per_sm);
cudaError_t TraceOccupancyFor(const TraceConfig& c, int variant, int* blocks_per_sm);
cudaError_t LaunchTrace(const TraceLaunch& L, bool any, bool stats, int grid, cudaStream_t stream);
cudaError_t LaunchTraceConfigured(const TraceLaunch& L, bool any, bool stats, const TraceConfig& c, int grid,
                                  cudaStream_t stream);
cudaError_t LaunchBatch(const BatchLaunch& B, const TraceConfig& c, int grid, cudaStream_t stream);

}  // namespace RT
}  // namespace Foundation
