// instances.cu — closest / any hit through a two-level scene (instances of
// bottom-level scenes under a top-level tree over their world boxes).
//
// One thread per ray, rays taken 32 at a time per warp from a work counter;
// each thread runs trace_two_level (traverse.cuh): the top-level leaves are
// instances, whose bottom levels are traversed in object space. Hits are
// written at the ray's index, as by the single-level kernels.
#include <cuda_runtime.h>

#include "../../../include/fnd_rt.h"
#include "traverse.cuh"
#include "traverse_launch.hpp"

namespace Foundation {
namespace RT {
namespace {

constexpr int kInstBlock = 128;

template <bool kAny>
__global__ void __launch_bounds__(kInstBlock) instanced_kernel(const InstancedLaunch L) {
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(L.counter, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= L.n) break;
        const uint32_t i = base + lane;
        if (i >= L.n) continue;
        const float4 r0 = __ldcs(L.rays + 2 * (size_t)i), r1 = __ldcs(L.rays + 2 * (size_t)i + 1);
        float t = r1.w;
        uint32_t p;
        const bool hit = trace_two_level<kAny>(L.tlas, L.inst, L.num_inst, r0, r1, t, p, L.status);
        if (kAny) {
            __stcs(L.occluded + i, (uint8_t)(hit ? 1 : 0));
        } else {
            __stcs(reinterpret_cast<uint2*>(L.hits) + i,
                   make_uint2(hit ? p : FND_INVALID_ID, hit ? __float_as_uint(t) : 0x7F800000u));
        }
    }
}

}  // namespace

cudaError_t LaunchInstanced(const InstancedLaunch& L, bool any, int sm_count, cudaStream_t s) {
    if (L.n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(L.counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, any ? instanced_kernel<true> : instanced_kernel<false>,
                                                      kInstBlock, 0);
    if (e != cudaSuccess) return e;
    const int grid = sm_count * (blocks > 0 ? blocks : 1);
    if (any)
        instanced_kernel<true><<<grid, kInstBlock, 0, s>>>(L);
    else
        instanced_kernel<false><<<grid, kInstBlock, 0, s>>>(L);
    return cudaGetLastError();
}

}  // namespace RT
}  // namespace Foundation
