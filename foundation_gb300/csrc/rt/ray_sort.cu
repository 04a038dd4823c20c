// ray_sort.cu — coherence ordering of a ray batch before traversal.
//
// Rays are bucketed by a key of `bits` bits: the Morton code of the origin's
// cell on a 2^p x 2^p x 2^p grid over the scene box (p = (bits - 3) / 3,
// origins outside the box clamped to the border cells) followed by the
// direction octant. A counting sort (histogram, exclusive scan, scatter)
// produces the fetch order; the persistent traversal then takes rays in that
// order and still writes every hit at the ray's own index, so results do not
// depend on it. Order within a bucket follows the scatter atomics and is not
// deterministic, which changes nothing but the schedule.
//
// Warps then hold rays that start in the same region and head the same way:
// they visit the same nodes (L1 / L2 reuse) and diverge less, which pays when
// rays are short against the scene (dense soups, secondary bounces).
#include <cuda_runtime.h>

#include "ray_sort.hpp"

namespace Foundation {
namespace RT {
namespace {

constexpr int kSortBlock = 256;
constexpr int kScanThreads = 1024;

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    // bits 0..9 of v to positions 0, 3, 6, ...
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

struct KeyParams {
    float lo[3];
    float scale[3];  // 2^p / extent
    float cmax;      // 2^p - 1
    uint32_t pbits;
};

__global__ void __launch_bounds__(kSortBlock) key_kernel(const float4* rays, uint32_t cap, const uint32_t* n_dev,
                                                         KeyParams P, uint32_t* keys, uint32_t* hist) {
    const uint32_t n = n_dev ? min(*n_dev, cap) : cap;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 o = __ldg(rays + 2 * (size_t)i);
    const float4 d = __ldg(rays + 2 * (size_t)i + 1);
    uint32_t q[3];
    const float c[3] = {o.x, o.y, o.z};
    for (int a = 0; a < 3; ++a) {
        // fminf / fmaxf drop a NaN operand, so NaN origins land in cell 0
        const float x = fminf(fmaxf((c[a] - P.lo[a]) * P.scale[a], 0.0f), P.cmax);
        q[a] = (uint32_t)x;
    }
    const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    const uint32_t morton = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
    const uint32_t key = (morton << 3) | oct;
    keys[i] = key;
    atomicAdd(hist + key, 1u);
}

// Exclusive scan of the m counters in place, in tiles of kTile counters
// (256 threads x 4): tile sums, one block scans the tile sums, each tile
// rescans itself from its offset.
constexpr int kTileThreads = 256;
constexpr uint32_t kTile = 4 * kTileThreads;

// Block-wide exclusive scan of one value per thread; returns the prefix and
// the block total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t& total, uint32_t* s_warp) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if ((int)lane >= o) incl += u;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    const uint32_t nw = blockDim.x >> 5;
    if (warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if ((int)lane >= o) w += u;
        }
        if (lane < nw) s_warp[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    total = s_warp[nw - 1];
    const uint32_t before = warp ? s_warp[warp - 1] : 0u;
    __syncthreads();
    return before + incl - v;
}

__global__ void __launch_bounds__(kTileThreads) tile_sum_kernel(const uint32_t* hist, uint32_t m, uint32_t* sums) {
    __shared__ uint32_t s_warp[32];
    const uint32_t k = blockIdx.x * kTile + 4u * threadIdx.x;
    uint32_t v = 0;
    for (uint32_t j = 0; j < 4; ++j) v += k + j < m ? hist[k + j] : 0u;
    uint32_t total;
    block_exclusive(v, total, s_warp);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block of kScanThreads threads scans up to 2 * kScanThreads tile sums.
__global__ void __launch_bounds__(kScanThreads) sums_scan_kernel(uint32_t* sums, uint32_t tiles) {
    __shared__ uint32_t s_warp[32];
    const uint32_t k = 2u * threadIdx.x;
    const uint32_t a = k < tiles ? sums[k] : 0u, b = k + 1 < tiles ? sums[k + 1] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive(a + b, total, s_warp);
    if (k < tiles) sums[k] = ex;
    if (k + 1 < tiles) sums[k + 1] = ex + a;
}

__global__ void __launch_bounds__(kTileThreads) tile_scan_kernel(uint32_t* hist, uint32_t m, const uint32_t* sums) {
    __shared__ uint32_t s_warp[32];
    const uint32_t k = blockIdx.x * kTile + 4u * threadIdx.x;
    uint32_t c[4];
    for (uint32_t j = 0; j < 4; ++j) c[j] = k + j < m ? hist[k + j] : 0u;
    uint32_t total;
    uint32_t run = sums[blockIdx.x] + block_exclusive(c[0] + c[1] + c[2] + c[3], total, s_warp);
    for (uint32_t j = 0; j < 4; ++j) {
        if (k + j < m) hist[k + j] = run;
        run += c[j];
    }
}

__global__ void __launch_bounds__(kSortBlock) scatter_kernel(uint32_t cap, const uint32_t* n_dev, const uint32_t* keys,
                                                             uint32_t* hist, uint32_t* order) {
    const uint32_t n = n_dev ? min(*n_dev, cap) : cap;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t slot = atomicAdd(hist + keys[i], 1u);
    order[slot] = i;
}

}  // namespace

bool ValidSortBits(uint32_t bits) { return bits == 0 || (bits >= 6 && bits <= kMaxSortBits && bits % 3 == 0); }

size_t RaySortScratchBytes(uint32_t cap, uint32_t bits) {
    return (bits ? (size_t(1) << bits) : 0) * sizeof(uint32_t) + 2 * sizeof(uint32_t) * (size_t)cap +
           sizeof(uint32_t) * kMaxSortTiles;
}

cudaError_t LaunchRaySort(const float4* rays, uint32_t cap, const uint32_t* n_dev, const float lo[3],
                          const float hi[3], uint32_t bits, const RaySortBuffers& B, cudaStream_t s) {
    if (!ValidSortBits(bits) || bits == 0) return cudaErrorInvalidValue;
    if (cap == 0) return cudaSuccess;
    const uint32_t m = 1u << bits;
    KeyParams P{};
    P.pbits = (bits - 3) / 3;
    const float cells = (float)(1u << P.pbits);
    P.cmax = cells - 1.0f;
    for (int a = 0; a < 3; ++a) {
        const float ext = hi[a] - lo[a];
        P.lo[a] = lo[a];
        P.scale[a] = ext > 0.0f ? cells / ext : 0.0f;
    }
    cudaError_t e = cudaMemsetAsync(B.hist, 0, sizeof(uint32_t) * (size_t)m, s);
    if (e != cudaSuccess) return e;
    const uint32_t blocks = (cap + kSortBlock - 1) / kSortBlock;
    const uint32_t tiles = (m + kTile - 1) / kTile;  // <= 2 * kScanThreads for bits <= 21
    key_kernel<<<blocks, kSortBlock, 0, s>>>(rays, cap, n_dev, P, B.keys, B.hist);
    tile_sum_kernel<<<tiles, kTileThreads, 0, s>>>(B.hist, m, B.sums);
    sums_scan_kernel<<<1, kScanThreads, 0, s>>>(B.sums, tiles);
    tile_scan_kernel<<<tiles, kTileThreads, 0, s>>>(B.hist, m, B.sums);
    scatter_kernel<<<blocks, kSortBlock, 0, s>>>(cap, n_dev, B.keys, B.hist, B.order);
    return cudaGetLastError();
}

}  // namespace RT
}  // namespace Foundation
