// ray_sort.hpp — coherence ordering of ray batches (ray_sort.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace Foundation {
namespace RT {

constexpr uint32_t kMaxSortBits = 21;    // 2^18 origin cells x 8 octants
constexpr uint32_t kMaxSortTiles = 2048;  // 2^21 counters / 1024 per scan tile

struct RaySortBuffers {
    uint32_t* keys;   // cap
    uint32_t* order;  // cap: fetch position -> ray index
    uint32_t* hist;   // 2^bits
    uint32_t* sums;   // kMaxSortTiles scan tile sums
};

// bits: 0 (no sorting) or a multiple of 3 in [6, 21].
bool ValidSortBits(uint32_t bits);
size_t RaySortScratchBytes(uint32_t cap, uint32_t bits);

// Writes B.order[0..n) for the rays [0, n), n = min(*n_dev, cap) when n_dev is
// set (a device queue length), else cap. lo / hi: the scene box.
cudaError_t LaunchRaySort(const float4* rays, uint32_t cap, const uint32_t* n_dev, const float lo[3],
                          const float hi[3], uint32_t bits, const RaySortBuffers& B, cudaStream_t s);

}  // namespace RT
}  // namespace Foundation
