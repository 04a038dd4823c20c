// gpu_build.cu — BVH construction on the GPU (see gpu_build.hpp).
//
//  1. prep: per triangle its box, its shading normal, input validation, and
//     the scene box / centroid box (warp-reduced float atomics);
//  2. 63-bit Morton code of each centroid on a grid of 2^21 cubic cells per
//     axis over the centroid box's largest extent (dense scenes keep a
//     spatial order far below the triangle size);
//  3. stable LSD radix sort of (code, triangle) in eight 8-bit passes: per
//     2,048-element warp tile a digit histogram, one exclusive scan over the
//     digit-major counts, then a scatter in which each warp ranks its
//     elements in order with __match_any_sync;
//  4. Karras (2012): internal node i of the n-1 finds its key range and
//     split by binary searches on the common-prefix length of the sorted
//     keys (ties between equal codes broken by sorted position); or
//     locally-ordered clustering of the sorted triangles (Meister & Bittner
//     2018), rounds of mutual-nearest-neighbour merges within a window of
//     the cluster array;
//  5. refit from the leaves upwards (the second thread to reach a node
//     finishes it): box, triangle count and the SAH decision
//     cost(n) = min(N A, C_trav A + cost(l) + cost(r)), a subtree of at most
//     max_leaf triangles becoming one leaf when that is not dearer;
//     With the SAH-optimal collapse the same walk also computes, per node,
//     the costs C(n, i) of representing its subtree by at most i roots (wide
//     nodes or leaf slots of up to 4 triangles) and their decisions, as
//     collapse.cpp does on the host;
//  6. collapse to 8-wide nodes, one wide level per launch: the children by
//     the greedy rule of collapse.cpp (expand the largest-area internal child
//     until 8) or by those decisions, octant slots, margin inflation and
//     outward quantisation in FP32 with directed rounding (conservative by
//     construction; the host collapse uses FP64), children and leaf
//     triangles allocated with atomics.
#include "gpu_build.hpp"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <vector>

#include "../../../include/fnd_rt.h"
#include "../core/core.hpp"
#include "../rt/device_scene.hpp"
#include "collapse.hpp"
#include "wide_bvh.hpp"

namespace Foundation {
namespace RT {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kLeafRef = 0x80000000u;  // reference to a sorted single-triangle leaf
constexpr uint32_t kLeafNode = 0x80000000u;  // count word: this subtree is one leaf
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kMaxLevels = kMaxStack / 2;  // wide levels the traversal stack allows
constexpr uint32_t kPrepBadIndex = 1u, kPrepNonFinite = 2u;

struct Buffers {
    float4 *blo, *bhi;            // triangle boxes (original order)
    unsigned long long *keys;     // sorted codes
    uint32_t* vals;               // triangle ids
    unsigned long long* keys2;    // radix-sort ping-pong
    uint32_t* vals2;
    uint32_t* cnt;                // digit-major tile counts
    uint32_t* sums;               // scan tile sums
    uint32_t *left, *right;       // internal node children (kLeafRef | sorted index for leaves)
    uint32_t *parent_i, *parent_l;
    float4 *nlo, *nhi;            // internal node boxes
    uint32_t* ncount;             // triangle count | kLeafNode
    float* ncost;
    uint32_t* flag;               // refit arrival counters
    float* bounds;                // scene lo[3], hi[3], centroid lo[3], hi[3]
    uint32_t* status;
    uint32_t* counters;           // [0] nodes, [1] tris, [2] leaves, [4..] per-level queue counts
    uint2 *qa, *qb;               // collapse queues (binary ref, wide node)
    // SAH-optimal collapse (null: greedy), per internal node k:
    float* dpc;                   // [8 k + i - 1]: C(k, i), least cost of k's subtree as at most i roots
    uint8_t* dpch;                // [8 k + i - 1], i >= 2: 0 = C(k, i - 1), else roots given to the left child
    uint8_t* dpj;                 // roots given to the left child when k is a wide node
    uint8_t* dpleaf;              // C(k, 1) is one leaf slot
    float c_tri;                  // cost of a triangle test relative to a wide-node visit
    uint32_t width;               // children per wide node (2..8)
};

__device__ __forceinline__ void atomic_min_f(float* a, float v) {
    if (v >= 0.0f)
        atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
    else
        atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
    if (v >= 0.0f)
        atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
    else
        atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

__global__ void init_bounds_kernel(float* b) {
    const int i = threadIdx.x;
    if (i < 12) b[i] = (i % 6) < 3 ? __int_as_float(0x7F800000) : __int_as_float(0xFF800000);
}

// Grid-stride over the triangles: each thread folds its triangles' boxes and
// centroids into its own bounds, the block reduces them, and one thread per
// block updates the scene bounds (a few thousand atomics in all, not one set
// per warp).
__global__ void __launch_bounds__(256) prep_kernel(const float* __restrict__ verts, uint32_t nv,
                                                   const uint32_t* __restrict__ idx, uint32_t nt, Buffers B,
                                                   float4* __restrict__ shade) {
    __shared__ float s_red[8][12];
    float lo[3], hi[3], c[3], cmax[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = c[a] = __int_as_float(0x7F800000);
        hi[a] = cmax[a] = __int_as_float(0xFF800000);
    }
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
        uint32_t vi[3];
        bool ok = true;
        for (int k = 0; k < 3; ++k) {
            vi[k] = idx[3 * (size_t)t + k];
            if (vi[k] >= nv) ok = false;
        }
        if (!ok) {
            atomicOr(B.status, kPrepBadIndex);
            continue;
        }
        float v[9];
        bool finite = true;
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
                v[3 * k + a] = verts[3 * (size_t)vi[k] + a];
                finite = finite && isfinite(v[3 * k + a]);
            }
        if (!finite) atomicOr(B.status, kPrepNonFinite);
        float tlo[3], thi[3];
        for (int a = 0; a < 3; ++a) {
            tlo[a] = fminf(fminf(v[a], v[3 + a]), v[6 + a]);
            thi[a] = fmaxf(fmaxf(v[a], v[3 + a]), v[6 + a]);
            const float cc = __fmul_rn(0.5f, __fadd_rn(tlo[a], thi[a]));
            lo[a] = fminf(lo[a], tlo[a]);
            hi[a] = fmaxf(hi[a], thi[a]);
            c[a] = fminf(c[a], cc);
            cmax[a] = fmaxf(cmax[a], cc);
        }
        B.blo[t] = make_float4(tlo[0], tlo[1], tlo[2], 0.0f);
        B.bhi[t] = make_float4(thi[0], thi[1], thi[2], 0.0f);
        // geometric normal (winding order), the host's expression tree
        const float e1x = __fsub_rn(v[3], v[0]), e1y = __fsub_rn(v[4], v[1]), e1z = __fsub_rn(v[5], v[2]);
        const float e2x = __fsub_rn(v[6], v[0]), e2y = __fsub_rn(v[7], v[1]), e2z = __fsub_rn(v[8], v[2]);
        float nx = __fsub_rn(__fmul_rn(e1y, e2z), __fmul_rn(e1z, e2y));
        float ny = __fsub_rn(__fmul_rn(e1z, e2x), __fmul_rn(e1x, e2z));
        float nz = __fsub_rn(__fmul_rn(e1x, e2y), __fmul_rn(e1y, e2x));
        const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz)));
        if (l > 0.0f) {
            nx = __fdiv_rn(nx, l);
            ny = __fdiv_rn(ny, l);
            nz = __fdiv_rn(nz, l);
        } else {
            nx = ny = 0.0f;
            nz = 1.0f;
        }
        shade[t] = make_float4(nx, ny, nz, 0.0f);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(kFull, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(kFull, hi[a], o));
            c[a] = fminf(c[a], __shfl_xor_sync(kFull, c[a], o));
            cmax[a] = fmaxf(cmax[a], __shfl_xor_sync(kFull, cmax[a], o));
        }
    const uint32_t warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31u) == 0)
        for (int a = 0; a < 3; ++a) {
            s_red[warp][a] = lo[a];
            s_red[warp][3 + a] = hi[a];
            s_red[warp][6 + a] = c[a];
            s_red[warp][9 + a] = cmax[a];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t w = 1; w < nw; ++w)
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], s_red[w][a]);
                hi[a] = fmaxf(hi[a], s_red[w][3 + a]);
                c[a] = fminf(c[a], s_red[w][6 + a]);
                cmax[a] = fmaxf(cmax[a], s_red[w][9 + a]);
            }
        if (lo[0] <= hi[0])
            for (int a = 0; a < 3; ++a) {
                atomic_min_f(B.bounds + a, lo[a]);
                atomic_max_f(B.bounds + 3 + a, hi[a]);
                atomic_min_f(B.bounds + 6 + a, c[a]);
                atomic_max_f(B.bounds + 9 + a, cmax[a]);
            }
    }
}

// bits 0..20 of v to positions 0, 3, 6, ... 60
__device__ __forceinline__ unsigned long long spread3(unsigned long long v) {
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// The grid's cells are cubes: every axis is scaled by the centroid box's
// largest extent, so a flat scene's thin axis takes few of the code's bits
// and the first splits of the order are along the long axes.
__global__ void __launch_bounds__(256) morton_kernel(uint32_t nt, Buffers B) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const float4 lo = B.blo[t], hi = B.bhi[t];
    const float c[3] = {__fmul_rn(0.5f, __fadd_rn(lo.x, hi.x)), __fmul_rn(0.5f, __fadd_rn(lo.y, hi.y)),
                        __fmul_rn(0.5f, __fadd_rn(lo.z, hi.z))};
    unsigned long long q[3];
    const float emax = fmaxf(fmaxf(B.bounds[9] - B.bounds[6], B.bounds[10] - B.bounds[7]), B.bounds[11] - B.bounds[8]);
    for (int a = 0; a < 3; ++a) {
        const float u = emax > 0.0f ? (c[a] - B.bounds[6 + a]) * (2097152.0f / emax) : 0.0f;
        q[a] = (unsigned long long)fminf(fmaxf(u, 0.0f), 2097151.0f);
    }
    B.keys[t] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
    B.vals[t] = t;
}

// ---- stable LSD radix sort ---------------------------------------------------
constexpr int kSortWarps = 8;
constexpr uint32_t kSortIters = 64;
constexpr uint32_t kSortTile = 32 * kSortIters;  // elements per warp tile
constexpr int kScanThreads = 256;
constexpr uint32_t kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;  // 4096 counters per scan tile
constexpr int kTopThreads = 1024;                           // scans up to 4 * 1024 tile sums

__global__ void __launch_bounds__(32 * kSortWarps) hist_kernel(const unsigned long long* __restrict__ keys, uint32_t n,
                                                               uint32_t shift, uint32_t units, uint32_t* cnt) {
    __shared__ uint32_t s_cnt[kSortWarps][256];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t u = blockIdx.x * kSortWarps + warp;
    if (u >= units) return;
    for (uint32_t d = lane; d < 256; d += 32) s_cnt[warp][d] = 0;
    __syncwarp();
    const uint32_t base = u * kSortTile;
    for (uint32_t it = 0; it < kSortIters; ++it) {
        const uint32_t i = base + it * 32 + lane;
        if (i < n) atomicAdd(&s_cnt[warp][(uint32_t)(keys[i] >> shift) & 255u], 1u);
    }
    __syncwarp();
    for (uint32_t d = lane; d < 256; d += 32) cnt[(size_t)d * units + u] = s_cnt[warp][d];
}

template <typename T>
__device__ __forceinline__ T block_exclusive(T v, T& total, T* s_warp) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    T incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const T x = __shfl_up_sync(kFull, incl, o);
        if ((int)lane >= o) incl += x;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    const uint32_t nw = blockDim.x >> 5;
    if (warp == 0) {
        T w = lane < nw ? s_warp[lane] : T(0);
        for (int o = 1; o < 32; o <<= 1) {
            const T x = __shfl_up_sync(kFull, w, o);
            if ((int)lane >= o) w += x;
        }
        if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[nw - 1];
    const T before = warp ? s_warp[warp - 1] : T(0);
    __syncthreads();
    return before + incl - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_tile_sum_kernel(const uint32_t* a, uint32_t m, uint32_t* sums) {
    __shared__ uint32_t s_warp[32];
    const uint32_t k = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v = 0;
    for (uint32_t j = 0; j < kScanItems; ++j) v += k + j < m ? a[k + j] : 0u;
    uint32_t total;
    block_exclusive(v, total, s_warp);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kTopThreads) scan_top_kernel(uint32_t* sums, uint32_t tiles) {
    __shared__ uint32_t s_warp[32];
    const uint32_t k = 4u * threadIdx.x;
    uint32_t c[4], v = 0;
    for (uint32_t j = 0; j < 4; ++j) {
        c[j] = k + j < tiles ? sums[k + j] : 0u;
        v += c[j];
    }
    uint32_t total;
    uint32_t run = block_exclusive(v, total, s_warp);
    for (uint32_t j = 0; j < 4; ++j) {
        if (k + j < tiles) sums[k + j] = run;
        run += c[j];
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(uint32_t* a, uint32_t m, const uint32_t* sums) {
    __shared__ uint32_t s_warp[32];
    const uint32_t k = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t c[kScanItems], v = 0;
    for (uint32_t j = 0; j < kScanItems; ++j) {
        c[j] = k + j < m ? a[k + j] : 0u;
        v += c[j];
    }
    uint32_t total;
    uint32_t run = sums[blockIdx.x] + block_exclusive(v, total, s_warp);
    for (uint32_t j = 0; j < kScanItems; ++j) {
        if (k + j < m) a[k + j] = run;
        run += c[j];
    }
}

__global__ void __launch_bounds__(32 * kSortWarps) scatter_kernel(const unsigned long long* __restrict__ keys,
                                                                  const uint32_t* __restrict__ vals, uint32_t n,
                                                                  uint32_t shift, uint32_t units,
                                                                  const uint32_t* __restrict__ cnt,
                                                                  unsigned long long* ok_,
                                                                  uint32_t* ov) {
    __shared__ uint32_t s_run[kSortWarps][256];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t u = blockIdx.x * kSortWarps + warp;
    if (u >= units) return;
    for (uint32_t d = lane; d < 256; d += 32) s_run[warp][d] = cnt[(size_t)d * units + u];
    __syncwarp();
    const uint32_t base = u * kSortTile;
    for (uint32_t it = 0; it < kSortIters; ++it) {
        const uint32_t i = base + it * 32 + lane;
        const bool ok = i < n;
        const unsigned long long k = ok ? keys[i] : 0ull;
        const uint32_t d = ok ? ((uint32_t)(k >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(kFull, d);
        const uint32_t rank = (uint32_t)__popc(peers & ((1u << lane) - 1u));
        const uint32_t start = ok ? s_run[warp][d] : 0u;
        __syncwarp();
        if (ok) {
            ok_[start + rank] = k;
            ov[start + rank] = vals[i];
            if (lane == (uint32_t)__ffs(peers) - 1u) s_run[warp][d] = start + (uint32_t)__popc(peers);
        }
        __syncwarp();
    }
}

// ---- hierarchy (Karras 2012) -------------------------------------------------
__device__ __forceinline__ int prefix(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = k[i], b = k[j];
    if (a != b) return __clzll(a ^ b);
    return 64 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void __launch_bounds__(256) hierarchy_kernel(int n, Buffers B) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n - 1) return;
    const unsigned long long* k = B.keys;
    const int d = prefix(k, n, i, i + 1) - prefix(k, n, i, i - 1) > 0 ? 1 : -1;
    const int dmin = prefix(k, n, i, i - d);
    int lmax = 2;
    while (prefix(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix(k, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = prefix(k, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        const int t = (l + div - 1) / div;
        if (prefix(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const uint32_t lc = lo == gamma ? (kLeafRef | (uint32_t)gamma) : (uint32_t)gamma;
    const uint32_t rc = hi == gamma + 1 ? (kLeafRef | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    B.left[i] = lc;
    B.right[i] = rc;
    if (lc & kLeafRef)
        B.parent_l[gamma] = (uint32_t)i;
    else
        B.parent_i[gamma] = (uint32_t)i;
    if (rc & kLeafRef)
        B.parent_l[gamma + 1] = (uint32_t)i;
    else
        B.parent_i[gamma + 1] = (uint32_t)i;
}

__host__ __device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

// ---- hierarchy by locally-ordered clustering (Meister & Bittner 2018) -----------
// Clusters start as the sorted single triangles. Each round, every cluster
// finds the neighbour within r positions of the current cluster array whose
// merged box has the least half area (ties: the nearer-to-the-front
// neighbour, which orders every pair by (area, lower index, higher index)
// alike from both ends); mutual neighbours merge into a new internal node at
// the lower position, and the array is compacted in order. The least pair of
// a round is always mutual, so every round of two or more clusters merges at
// least one pair. Internal nodes are numbered down from n - 2 in creation
// order, so the last merge, the root, is node 0 as in the Karras tree, and
// the same refit and collapse follow.
constexpr int kPlocBlock = 256;
constexpr int kPlocMaxRadius = 64;
constexpr uint32_t kPlocItems = 16;
constexpr uint32_t kPlocTile = kPlocBlock * kPlocItems;  // clusters per scan tile

struct PlocState {
    uint32_t count;      // clusters
    uint32_t next_node;  // internal nodes 0 .. next_node - 1 are still to be made
};

__global__ void __launch_bounds__(kPlocBlock) ploc_init_kernel(uint32_t n, Buffers B, uint32_t* __restrict__ cref,
                                                               float4* __restrict__ lo, float4* __restrict__ hi,
                                                               PlocState* st) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *st = PlocState{n, n - 1u};
    if (i >= n) return;
    const uint32_t t = B.vals[i];
    cref[i] = kLeafRef | i;
    lo[i] = B.blo[t];
    hi[i] = B.bhi[t];
}

__global__ void __launch_bounds__(kPlocBlock) ploc_nn_kernel(const PlocState* __restrict__ st,
                                                             const float4* __restrict__ lo,
                                                             const float4* __restrict__ hi, uint32_t* __restrict__ nn,
                                                             int r) {
    __shared__ float4 s_lo[kPlocBlock + 2 * kPlocMaxRadius], s_hi[kPlocBlock + 2 * kPlocMaxRadius];
    const int count = (int)st->count;
    const int b0 = (int)(blockIdx.x * kPlocBlock);
    if (b0 >= count) return;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * r; k += kPlocBlock) {
        const int g = b0 - r + k;
        if (g >= 0 && g < count) {
            s_lo[k] = lo[g];
            s_hi[k] = hi[g];
        }
    }
    __syncthreads();
    const int i = b0 + (int)threadIdx.x;
    if (i >= count) return;
    const int li = (int)threadIdx.x + r;
    const float4 alo = s_lo[li], ahi = s_hi[li];
    float best = __int_as_float(0x7F800000);
    int bj = i;
    const int jlo = max(0, i - r), jhi = min(count - 1, i + r);
    for (int j = jlo; j <= jhi; ++j) {
        if (j == i) continue;
        const int lj = j - b0 + r;
        // the lower position's box first, so both ends compute the same bits
        const float4 plo = j < i ? s_lo[lj] : alo, phi = j < i ? s_hi[lj] : ahi;
        const float4 qlo = j < i ? alo : s_lo[lj], qhi = j < i ? ahi : s_hi[lj];
        const float dx = fmaxf(phi.x, qhi.x) - fminf(plo.x, qlo.x);
        const float dy = fmaxf(phi.y, qhi.y) - fminf(plo.y, qlo.y);
        const float dz = fmaxf(phi.z, qhi.z) - fminf(plo.z, qlo.z);
        // overflowing extents compare as +inf, so the order stays total
        const float d = fminf(dx * dy + dy * dz + dz * dx, __int_as_float(0x7F800000));
        if (d < best || bj == i) {
            best = d;
            bj = j;
        }
    }
    nn[i] = (uint32_t)bj;
}

// per cluster i with neighbour j: merges here (mutual, i < j), survives
// (not mutual, or the merge's lower end)
__device__ __forceinline__ void ploc_flags(const uint32_t* __restrict__ nn, uint32_t i, uint32_t& j, bool& merge,
                                           bool& survive) {
    j = nn[i];
    const bool mutual = j != i && nn[j] == i;
    merge = mutual && i < j;
    survive = !mutual || i < j;
}

// per tile: (merges << 32) | survivors
__global__ void __launch_bounds__(kPlocBlock) ploc_count_kernel(const PlocState* __restrict__ st,
                                                                const uint32_t* __restrict__ nn,
                                                                unsigned long long* __restrict__ tsum) {
    __shared__ unsigned long long s_warp[32];
    const uint32_t count = st->count;
    if (blockIdx.x * kPlocTile >= count) return;
    const uint32_t base = blockIdx.x * kPlocTile + threadIdx.x * kPlocItems;
    unsigned long long v = 0;
    for (uint32_t k = 0; k < kPlocItems; ++k) {
        const uint32_t i = base + k;
        if (i >= count) break;
        uint32_t j;
        bool merge, survive;
        ploc_flags(nn, i, j, merge, survive);
        v += (merge ? (1ull << 32) : 0ull) + (survive ? 1ull : 0ull);
    }
    unsigned long long total;
    block_exclusive(v, total, s_warp);
    if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

// exclusive scan of the tile sums (one block, 4,096 tiles at a time), and
// the next round's state
__global__ void __launch_bounds__(1024) ploc_scan_kernel(const PlocState* __restrict__ st, PlocState* __restrict__ next,
                                                         unsigned long long* __restrict__ tsum) {
    __shared__ unsigned long long s_warp[32];
    const uint32_t count = st->count;
    const uint32_t tiles = (count + kPlocTile - 1) / kPlocTile;
    unsigned long long carry = 0;
    for (uint32_t c0 = 0; c0 < tiles; c0 += 4 * 1024) {
        const uint32_t k = c0 + 4u * threadIdx.x;
        unsigned long long c[4], v = 0;
        for (uint32_t j = 0; j < 4; ++j) {
            c[j] = k + j < tiles ? tsum[k + j] : 0ull;
            v += c[j];
        }
        unsigned long long total;
        unsigned long long run = carry + block_exclusive(v, total, s_warp);
        for (uint32_t j = 0; j < 4; ++j) {
            if (k + j < tiles) tsum[k + j] = run;
            run += c[j];
        }
        carry += total;
    }
    if (threadIdx.x == 0) *next = PlocState{(uint32_t)carry, st->next_node - (uint32_t)(carry >> 32)};
}

__device__ __forceinline__ void ploc_set_parent(const Buffers& B, uint32_t ref, uint32_t node) {
    if (ref & kLeafRef)
        B.parent_l[ref & ~kLeafRef] = node;
    else
        B.parent_i[ref] = node;
}

__global__ void __launch_bounds__(kPlocBlock) ploc_merge_kernel(
    const PlocState* __restrict__ st, const unsigned long long* __restrict__ tsum, const uint32_t* __restrict__ nn,
    const uint32_t* __restrict__ cin, const float4* __restrict__ lin, const float4* __restrict__ hin,
    uint32_t* __restrict__ cout, float4* __restrict__ lout, float4* __restrict__ hout, Buffers B) {
    __shared__ unsigned long long s_warp[32];
    const uint32_t count = st->count, next_node = st->next_node;
    if (blockIdx.x * kPlocTile >= count) return;
    const uint32_t base = blockIdx.x * kPlocTile + threadIdx.x * kPlocItems;
    uint32_t jj[kPlocItems], merge_bits = 0, survive_bits = 0;
    unsigned long long v = 0;
    for (uint32_t k = 0; k < kPlocItems; ++k) {
        const uint32_t i = base + k;
        bool merge = false, survive = false;
        jj[k] = i;
        if (i < count) ploc_flags(nn, i, jj[k], merge, survive);
        merge_bits |= (merge ? 1u : 0u) << k;
        survive_bits |= (survive ? 1u : 0u) << k;
        v += (merge ? (1ull << 32) : 0ull) + (survive ? 1ull : 0ull);
    }
    unsigned long long total;
    unsigned long long run = tsum[blockIdx.x] + block_exclusive(v, total, s_warp);
    for (uint32_t k = 0; k < kPlocItems; ++k) {
        if (!(survive_bits >> k & 1u)) continue;
        const uint32_t i = base + k, at = (uint32_t)run;
        if (merge_bits >> k & 1u) {
            const uint32_t j = jj[k];
            const uint32_t node = next_node - 1u - (uint32_t)(run >> 32);
            const uint32_t a = cin[i], b = cin[j];
            B.left[node] = a;
            B.right[node] = b;
            ploc_set_parent(B, a, node);
            ploc_set_parent(B, b, node);
            const float4 al = lin[i], ah = hin[i], bl = lin[j], bh = hin[j];
            cout[at] = node;
            lout[at] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
            hout[at] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
            run += (1ull << 32) + 1ull;
        } else {
            cout[at] = cin[i];
            lout[at] = lin[i];
            hout[at] = hin[i];
            run += 1ull;
        }
    }
}

struct RefBox {
    float4 lo, hi;
    uint32_t count;  // | kLeafNode when the subtree is one leaf
    float cost;
};

__device__ __forceinline__ RefBox ref_box(const Buffers& B, uint32_t ref) {
    RefBox r;
    if (ref & kLeafRef) {
        const uint32_t t = B.vals[ref & ~kLeafRef];
        r.lo = B.blo[t];
        r.hi = B.bhi[t];
        r.count = 1u | kLeafNode;
        r.cost = half_area(r.lo, r.hi);
    } else {
        r.lo = __ldcg(B.nlo + ref);
        r.hi = __ldcg(B.nhi + ref);
        r.count = __ldcg(B.ncount + ref);
        r.cost = __ldcg(B.ncost + ref);
    }
    return r;
}

// C(ref, 1..8) of a child: a single-triangle leaf costs c_tri x its half area
// whatever the number of roots.
__device__ __forceinline__ void dp_child(const Buffers& B, uint32_t ref, float c[8]) {
    if (ref & kLeafRef) {
        const uint32_t t = B.vals[ref & ~kLeafRef];
        const float v = B.c_tri * half_area(B.blo[t], B.bhi[t]);
        for (int i = 0; i < 8; ++i) c[i] = v;
    } else {
        const float4 a = __ldcg(reinterpret_cast<const float4*>(B.dpc + 8 * (size_t)ref));
        const float4 b = __ldcg(reinterpret_cast<const float4*>(B.dpc + 8 * (size_t)ref) + 1);
        c[0] = a.x, c[1] = a.y, c[2] = a.z, c[3] = a.w, c[4] = b.x, c[5] = b.y, c[6] = b.z, c[7] = b.w;
    }
}

__global__ void __launch_bounds__(256) refit_kernel(uint32_t n, Buffers B, uint32_t max_leaf, float trav_cost) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || n < 2) return;
    uint32_t p = B.parent_l[k];
    // a root path has fewer than n nodes; the bound only guards the walk
    for (uint32_t steps = 0; p != kNone; ++steps) {
        if (steps >= n) {
            atomicOr(B.status, 8u);
            return;
        }
        __threadfence();
        if (atomicAdd(B.flag + p, 1u) == 0u) return;  // the sibling subtree is not finished yet
        __threadfence();
        const RefBox l = ref_box(B, B.left[p]), r = ref_box(B, B.right[p]);
        float4 lo = make_float4(fminf(l.lo.x, r.lo.x), fminf(l.lo.y, r.lo.y), fminf(l.lo.z, r.lo.z), 0.0f);
        float4 hi = make_float4(fmaxf(l.hi.x, r.hi.x), fmaxf(l.hi.y, r.hi.y), fmaxf(l.hi.z, r.hi.z), 0.0f);
        const uint32_t cnt = (l.count & ~kLeafNode) + (r.count & ~kLeafNode);
        const float a = half_area(lo, hi);
        const float split = trav_cost * a + l.cost + r.cost;
        const bool leaf = cnt <= max_leaf && (float)cnt * a <= split;
        B.nlo[p] = lo;
        B.nhi[p] = hi;
        B.ncount[p] = cnt | (leaf ? kLeafNode : 0u);
        B.ncost[p] = leaf ? (float)cnt * a : split;
        if (B.dpc) {
            // SAH-optimal collapse: wide node at cost a, leaf slot at c_tri a cnt
            float cl[8], cr[8], sp[9];
            uint8_t sj[9];
            dp_child(B, B.left[p], cl);
            dp_child(B, B.right[p], cr);
            for (int i = 2; i <= 8; ++i) {
                sp[i] = FLT_MAX;
                sj[i] = 1;
                for (int j = 1; j < i; ++j) {
                    const float v = cl[j - 1] + cr[i - j - 1];
                    if (v < sp[i]) {
                        sp[i] = v;
                        sj[i] = (uint8_t)j;
                    }
                }
            }
            float c[8];
            const float node_cost = a + sp[B.width];
            c[0] = node_cost;
            uint8_t as_leaf = 0;
            if (cnt <= (uint32_t)kMaxLeafTris) {
                const float leaf_cost = B.c_tri * a * (float)cnt;
                if (leaf_cost <= node_cost) {
                    c[0] = leaf_cost;
                    as_leaf = 1;
                }
            }
            uint8_t ch[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int i = 2; i <= 8; ++i) {
                if (sp[i] < c[i - 2]) {
                    c[i - 1] = sp[i];
                    ch[i - 1] = sj[i];
                } else {
                    c[i - 1] = c[i - 2];
                }
            }
            float4* dc = reinterpret_cast<float4*>(B.dpc + 8 * (size_t)p);
            dc[0] = make_float4(c[0], c[1], c[2], c[3]);
            dc[1] = make_float4(c[4], c[5], c[6], c[7]);
            for (int i = 0; i < 8; ++i) B.dpch[8 * (size_t)p + i] = ch[i];
            B.dpj[p] = sj[B.width];
            B.dpleaf[p] = as_leaf;
        }
        p = B.parent_i[p];
    }
}

// ---- collapse to 8-wide nodes -------------------------------------------------
struct CollapseArgs {
    Buffers B;
    const float* verts;
    const uint32_t* idx;
    WideNode* nodes;
    float4 *v0, *v1, *v2;
    float margin;
    int level;
};

__global__ void __launch_bounds__(128) collapse_kernel(const CollapseArgs A) {
    const Buffers& B = A.B;
    uint32_t* counters = B.counters;
    const uint32_t count = counters[4 + A.level];
    const uint2* qin = (A.level & 1) ? B.qb : B.qa;
    uint2* qout = (A.level & 1) ? B.qa : B.qb;
    for (uint32_t it = blockIdx.x * blockDim.x + threadIdx.x; it < count; it += gridDim.x * blockDim.x) {
        const uint2 item = qin[it];
        uint32_t kids[kWidth];
        bool dp_leaf[kWidth];
        int nk = 1;
        kids[0] = item.x;
        if (B.dpc && !(item.x & kLeafRef)) {
            // the children the SAH-optimal decisions give wide node item.x
            uint2 st[16];
            int sp = 0;
            const uint32_t j = B.dpj[item.x];
            st[sp++] = make_uint2(B.right[item.x], B.width - j);
            st[sp++] = make_uint2(B.left[item.x], j);
            nk = 0;
            while (sp > 0) {
                const uint2 e = st[--sp];
                uint32_t k = e.y;
                if (!(e.x & kLeafRef))
                    while (k >= 2u && B.dpch[8 * (size_t)e.x + k - 1] == 0) --k;
                if (!(e.x & kLeafRef) && k >= 2u && sp + 2 <= 16) {
                    const uint32_t jj = B.dpch[8 * (size_t)e.x + k - 1];
                    st[sp++] = make_uint2(B.right[e.x], k - jj);
                    st[sp++] = make_uint2(B.left[e.x], jj);
                } else if (nk < kWidth) {
                    kids[nk] = e.x;
                    dp_leaf[nk] = (e.x & kLeafRef) || B.dpleaf[e.x];
                    nk++;
                } else {
                    atomicOr(B.status, 8u);  // more than 8 roots: malformed decisions
                    break;
                }
            }
        }
        for (;;) {
            if (B.dpc && !(item.x & kLeafRef)) break;
            int pick = -1;
            float best = -1.0f;
            for (int c = 0; c < nk; ++c) {
                if (kids[c] & kLeafRef) continue;
                if (__ldcg(B.ncount + kids[c]) & kLeafNode) continue;
                const float a = half_area(__ldcg(B.nlo + kids[c]), __ldcg(B.nhi + kids[c]));
                if (a > best) {
                    best = a;
                    pick = c;
                }
            }
            if (pick < 0 || nk == (int)B.width) break;
            const uint32_t p = kids[pick];
            kids[pick] = B.left[p];
            kids[nk++] = B.right[p];
        }
        // child boxes inflated by the margin (one ulp outward when the
        // subtraction rounds back), node box
        float clo[kWidth][3], chi[kWidth][3];
        float nlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, nhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t cnt[kWidth];
        bool is_leaf[kWidth];
        for (int c = 0; c < nk; ++c) {
            float4 lo, hi;
            if (kids[c] & kLeafRef) {
                const uint32_t sk = kids[c] & ~kLeafRef;
                const uint32_t t = B.vals[sk];
                lo = B.blo[t];
                hi = B.bhi[t];
                cnt[c] = 1;
                is_leaf[c] = true;
            } else {
                lo = __ldcg(B.nlo + kids[c]);
                hi = __ldcg(B.nhi + kids[c]);
                const uint32_t w = __ldcg(B.ncount + kids[c]);
                is_leaf[c] = (B.dpc && !(item.x & kLeafRef)) ? dp_leaf[c] : (w & kLeafNode) != 0u;
                cnt[c] = w & ~kLeafNode;
            }
            const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z};
            for (int a = 0; a < 3; ++a) {
                float x = l3[a] - A.margin, y = h3[a] + A.margin;
                if (!(x < l3[a])) x = nextafterf(l3[a], -INFINITY);
                if (!(y > h3[a])) y = nextafterf(h3[a], INFINITY);
                clo[c][a] = x;
                chi[c][a] = y;
                nlo[a] = fminf(nlo[a], x);
                nhi[a] = fmaxf(nhi[a], y);
            }
        }
        // octant slots, greedy on the corner score (as collapse.cpp)
        int child_in_slot[kWidth];
        for (int s = 0; s < kWidth; ++s) child_in_slot[s] = -1;
        {
            const float cx = 0.5f * (nlo[0] + nhi[0]), cy = 0.5f * (nlo[1] + nhi[1]), cz = 0.5f * (nlo[2] + nhi[2]);
            float dxs[kWidth], dys[kWidth], dzs[kWidth];
            for (int c = 0; c < nk; ++c) {
                dxs[c] = 0.5f * (clo[c][0] + chi[c][0]) - cx;
                dys[c] = 0.5f * (clo[c][1] + chi[c][1]) - cy;
                dzs[c] = 0.5f * (clo[c][2] + chi[c][2]) - cz;
            }
            uint32_t used_k = 0, used_s = 0;
            for (int round = 0; round < nk; ++round) {
                int bk = -1, bs = -1;
                float bv = -FLT_MAX;
                for (int c = 0; c < nk; ++c) {
                    if (used_k & (1u << c)) continue;
                    for (int s = 0; s < kWidth; ++s) {
                        if (used_s & (1u << s)) continue;
                        const float sc = ((s & 1) ? dxs[c] : -dxs[c]) + ((s & 2) ? dys[c] : -dys[c]) +
                                         ((s & 4) ? dzs[c] : -dzs[c]);
                        if (sc > bv || bk < 0) {
                            bv = sc;
                            bk = c;
                            bs = s;
                        }
                    }
                }
                used_k |= 1u << bk;
                used_s |= 1u << bs;
                child_in_slot[bs] = bk;
            }
        }
        WideNode nd;
        uint32_t* ndw = reinterpret_cast<uint32_t*>(&nd);
        for (int w = 0; w < 20; ++w) ndw[w] = 0u;
        // grid step 2^e per axis: the least e with 255 2^e >= the node's
        // extent rounded up (all in FP32; 255 2^e and 2^-e are exact)
        float inv_step[3];
        bool bad = false;
        for (int a = 0; a < 3; ++a) {
            nd.p[a] = nlo[a];
            const float ext = __fsub_ru(nhi[a], nlo[a]);
            int e = ext > 0.0f ? ilogbf(ext) - 8 : -100;
            while (e <= 100 && ldexpf(255.0f, e) < ext) e++;
            while (e > -100 && ldexpf(255.0f, e - 1) >= ext) e--;
            if (e < -100 || e > 100) bad = true;
            nd.e[a] = (uint8_t)(e + 127);
            inv_step[a] = ldexpf(1.0f, -e);
        }
        uint32_t n_int = 0, n_tri = 0;
        bool bad_tree = false;
        for (int c = 0; c < nk; ++c) {
            if (is_leaf[c])
                n_tri += cnt[c];
            else
                n_int++;
        }
        const uint32_t child_base = n_int ? atomicAdd(counters + 0, n_int) : 0u;
        const uint32_t tri_base = n_tri ? atomicAdd(counters + 1, n_tri) : 0u;
        nd.child_base = child_base;
        nd.tri_base = tri_base;
        uint32_t tri_off = 0, int_off = 0, leaves = 0;
        for (int s = 0; s < kWidth; ++s) {
            const int c = child_in_slot[s];
            if (c < 0) continue;
            // outward: the offsets from p rounded down / up before the
            // exact scaling by 2^-e, so p + ql 2^e <= lo and p + qh 2^e >= hi
            // hold exactly; qh <= 255 since hi - p <= the node's extent
            for (int a = 0; a < 3; ++a) {
                const float p = nd.p[a];
                const float ql = floorf(__fmul_rd(__fsub_rd(clo[c][a], p), inv_step[a]));
                const float qh = ceilf(__fmul_ru(__fsub_ru(chi[c][a], p), inv_step[a]));
                nd.qlo[a][s] = (uint8_t)fminf(fmaxf(ql, 0.0f), 255.0f);
                nd.qhi[a][s] = (uint8_t)fminf(fmaxf(qh, 0.0f), 255.0f);
            }
            if (is_leaf[c]) {
                nd.meta[s] = (uint8_t)(kMetaLeafFlag | ((cnt[c] - 1u) << 5) | tri_off);
                // the leaf's triangles: its binary subtree's leaves, left to right
                // (a Morton-order range for the Karras tree, not for clusters)
                uint32_t st[2 * kMaxLeafTris];
                int sp = 0;
                st[sp++] = kids[c];
                uint32_t i = 0;
                for (int step = 0; sp > 0 && i < cnt[c] && step < 4 * kMaxLeafTris; ++step) {
                    const uint32_t ref = st[--sp];
                    if (!(ref & kLeafRef)) {
                        if (sp + 2 > 2 * kMaxLeafTris) break;
                        st[sp++] = B.right[ref];
                        st[sp++] = B.left[ref];
                        continue;
                    }
                    const uint32_t t = B.vals[ref & ~kLeafRef];
                    const size_t d = (size_t)tri_base + tri_off + i;
                    float v[9];
                    for (int k = 0; k < 3; ++k)
                        for (int q = 0; q < 3; ++q) v[3 * k + q] = A.verts[3 * (size_t)A.idx[3 * (size_t)t + k] + q];
                    A.v0[d] = make_float4(v[0], v[1], v[2], __uint_as_float(t));
                    A.v1[d] = make_float4(v[3], v[4], v[5], 0.0f);
                    A.v2[d] = make_float4(v[6], v[7], v[8], 0.0f);
                    i++;
                }
                if (i != cnt[c]) bad_tree = true;
                tri_off += cnt[c];
                leaves++;
            } else {
                nd.imask |= (uint8_t)(1u << s);
                nd.meta[s] = kMetaInternal;
                const uint32_t slot = atomicAdd(counters + 4 + A.level + 1, 1u);
                qout[slot] = make_uint2(kids[c], child_base + int_off);
                int_off++;
            }
        }
        if (bad) atomicOr(B.status, 4u);
        if (bad_tree) atomicOr(B.status, 8u);
        if (leaves) atomicAdd(counters + 2, leaves);
        A.nodes[item.y] = nd;
    }
}

__global__ void instance_shade_kernel(const float* __restrict__ inv, const uint32_t* __restrict__ prefix,
                                      const uint32_t* __restrict__ off, const float4* const* __restrict__ blas,
                                      uint32_t n_inst, uint32_t total, float4* __restrict__ out) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    uint32_t lo = 0, hi = n_inst;  // prefix[lo] <= g < prefix[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    const uint32_t t = g - prefix[lo];
    const float4 n = blas[lo][t];
    const float* m = inv + 12 * (size_t)lo;
    float w[3];
    for (int j = 0; j < 3; ++j) w[j] = m[j] * n.x + m[4 + j] * n.y + m[8 + j] * n.z;
    const float l = sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    const float k = l > 0.0f ? 1.0f / l : 0.0f;
    out[(size_t)off[lo] + t] = l > 0.0f ? make_float4(w[0] * k, w[1] * k, w[2] * k, 0.0f) : make_float4(0, 0, 1, 0);
}

__global__ void write_ids_kernel(float4* shade, const uint32_t* ids, uint32_t nt) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nt) reinterpret_cast<uint32_t*>(shade + t)[3] = ids[t];
}

double Ms(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void Check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        RtCore::Fail(e == cudaErrorMemoryAllocation ? FND_ERR_OUT_OF_MEMORY : FND_ERR_CUDA, "%s: %s", what,
                   cudaGetErrorString(e));
}

// Owner of the temporary device allocations of one build.
struct Scratch {
    std::vector<void*> ptrs;
    template <typename T>
    T* get(size_t count) {
        void* p = nullptr;
        Check(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), "cudaMalloc (GPU build scratch)");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

void RadixSort(Buffers& B, uint32_t n, cudaStream_t s) {
    const uint32_t units = (n + kSortTile - 1) / kSortTile;
    const uint32_t m = 256u * units;
    const uint32_t tiles = (m + kScanTile - 1) / kScanTile;
    const uint32_t blocks = (units + kSortWarps - 1) / kSortWarps;
    unsigned long long *k_in = B.keys, *k_out = B.keys2;
    uint32_t *v_in = B.vals, *v_out = B.vals2;
    for (uint32_t shift = 0; shift < 64; shift += 8) {
        hist_kernel<<<blocks, 32 * kSortWarps, 0, s>>>(k_in, n, shift, units, B.cnt);
        scan_tile_sum_kernel<<<tiles, kScanThreads, 0, s>>>(B.cnt, m, B.sums);
        scan_top_kernel<<<1, kTopThreads, 0, s>>>(B.sums, tiles);
        scan_tile_kernel<<<tiles, kScanThreads, 0, s>>>(B.cnt, m, B.sums);
        scatter_kernel<<<blocks, 32 * kSortWarps, 0, s>>>(k_in, v_in, n, shift, units, B.cnt, k_out, v_out);
        std::swap(k_in, k_out);
        std::swap(v_in, v_out);
    }
    Check(cudaGetLastError(), "radix sort launch");
    // eight passes: the sorted data is back in keys / vals
}

// The clustering rounds of ploc_*_kernel. Each round's grids are sized by
// the cluster count read back one round late (an upper bound: counts only
// fall), so the host never waits for the round it has just queued.
void PlocHierarchy(Buffers& B, uint32_t n, int r, cudaStream_t s) {
    Scratch S;
    uint32_t* cref[2] = {S.get<uint32_t>(n), S.get<uint32_t>(n)};
    float4* lo[2] = {S.get<float4>(n), S.get<float4>(n)};
    float4* hi[2] = {S.get<float4>(n), S.get<float4>(n)};
    uint32_t* nn = S.get<uint32_t>(n);
    unsigned long long* tsum = S.get<unsigned long long>((n + kPlocTile - 1) / kPlocTile);
    PlocState* st = S.get<PlocState>(2);
    PlocState* h = nullptr;  // one pinned slot per round in flight
    Check(cudaHostAlloc(reinterpret_cast<void**>(&h), 2 * sizeof(PlocState), cudaHostAllocDefault),
          "cudaHostAlloc (cluster counts)");
    cudaEvent_t ev[2] = {nullptr, nullptr};
    struct Release {
        PlocState* h;
        cudaEvent_t* ev;
        ~Release() {
            for (int k = 0; k < 2; ++k)
                if (ev[k]) cudaEventDestroy(ev[k]);
            cudaFreeHost(h);
        }
    } release{h, ev};
    for (int k = 0; k < 2; ++k) Check(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming), "event");
    ploc_init_kernel<<<(n + kPlocBlock - 1) / kPlocBlock, kPlocBlock, 0, s>>>(n, B, cref[0], lo[0], hi[0], st);
    uint32_t bound = n, last = n, launched = 0;
    int cur = 0;
    bool done = false, stuck = false;
    // every round of two or more clusters merges a pair: at most n - 1 rounds
    for (uint32_t round = 0; !done && round <= n; ++round) {
        launched = round + 1;
        const uint32_t tiles = (bound + kPlocTile - 1) / kPlocTile;
        ploc_nn_kernel<<<(bound + kPlocBlock - 1) / kPlocBlock, kPlocBlock, 0, s>>>(st + cur, lo[cur], hi[cur], nn, r);
        ploc_count_kernel<<<tiles, kPlocBlock, 0, s>>>(st + cur, nn, tsum);
        ploc_scan_kernel<<<1, 1024, 0, s>>>(st + cur, st + (cur ^ 1), tsum);
        ploc_merge_kernel<<<tiles, kPlocBlock, 0, s>>>(st + cur, tsum, nn, cref[cur], lo[cur], hi[cur],
                                                       cref[cur ^ 1], lo[cur ^ 1], hi[cur ^ 1], B);
        Check(cudaMemcpyAsync(h + (round & 1), st + (cur ^ 1), sizeof(PlocState), cudaMemcpyDeviceToHost, s),
              "cluster count");
        Check(cudaEventRecord(ev[round & 1], s), "event");
        cur ^= 1;
        if (round == 0) continue;
        Check(cudaEventSynchronize(ev[(round - 1) & 1]), "clustering round");
        const uint32_t c = h[(round - 1) & 1].count;
        done = c <= 1;
        stuck = c >= last;  // no merge in a round of two or more clusters
        if (stuck) break;
        last = bound = c;
    }
    Check(cudaStreamSynchronize(s), "clustering");
    const PlocState fin = h[(launched - 1) & 1];
    CHECK_CODE(!stuck && done && fin.count == 1 && fin.next_node == 0, FND_ERR_INVALID_SCENE,
               "GPU build: clustering stopped at %u clusters", fin.count);
}

}  // namespace

void BuildWideGpu(const float* d_verts, uint32_t nv, const uint32_t* d_idx, uint32_t nt, const GpuBuildParams& p,
                  GpuBuildOutput& out, cudaStream_t s) {
    CHECK_CODE(nt >= 1 && nt <= kGpuBuildMaxTris, FND_ERR_INVALID_ARG, "GPU build takes 1..%u triangles, not %u",
               kGpuBuildMaxTris, nt);
    CHECK_CODE(p.max_leaf >= 1 && p.max_leaf <= (uint32_t)kMaxLeafTris, FND_ERR_INVALID_ARG, "max_leaf %u",
               p.max_leaf);
    CHECK_CODE(p.width >= 2 && p.width <= (uint32_t)kWidth, FND_ERR_INVALID_ARG, "node width %u not in 2..%d",
               p.width, kWidth);
    CHECK_CODE(p.ploc_radius <= (uint32_t)kPlocMaxRadius, FND_ERR_INVALID_ARG, "clustering radius %u above %d",
               p.ploc_radius, kPlocMaxRadius);
    int dev = 0, sms = 0;
    Check(cudaGetDevice(&dev), "cudaGetDevice");
    Check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    const auto t0 = std::chrono::steady_clock::now();
    Scratch S;
    Buffers B{};
    const uint32_t n = nt;
    const uint32_t units = (n + kSortTile - 1) / kSortTile;
    B.blo = S.get<float4>(n);
    B.bhi = S.get<float4>(n);
    B.keys = S.get<unsigned long long>(n);
    B.vals = S.get<uint32_t>(n);
    B.keys2 = S.get<unsigned long long>(n);
    B.vals2 = S.get<uint32_t>(n);
    B.cnt = S.get<uint32_t>(256ull * units);
    B.sums = S.get<uint32_t>(4 * kTopThreads);
    B.left = S.get<uint32_t>(n);
    B.right = S.get<uint32_t>(n);
    B.parent_i = S.get<uint32_t>(n);
    B.parent_l = S.get<uint32_t>(n);
    B.nlo = S.get<float4>(n);
    B.nhi = S.get<float4>(n);
    B.ncount = S.get<uint32_t>(n);
    B.ncost = S.get<float>(n);
    B.flag = S.get<uint32_t>(n);
    B.bounds = S.get<float>(12);
    B.status = S.get<uint32_t>(1);
    B.counters = S.get<uint32_t>(4 + kMaxLevels + 2);
    B.width = p.width;
    B.qa = S.get<uint2>(n);
    B.qb = S.get<uint2>(n);
    if (p.sah_collapse && n >= 2) {
        B.dpc = S.get<float>(8ull * n);
        B.dpch = S.get<uint8_t>(8ull * n);
        B.dpj = S.get<uint8_t>(n);
        B.dpleaf = S.get<uint8_t>(n);
        B.c_tri = p.c_tri;
    }
    float4* shade = nullptr;
    Check(cudaMalloc(&shade, 16ull * n), "cudaMalloc (shading normals)");
    out.d_tri_shade = shade;
    Check(cudaMemsetAsync(B.status, 0, 4, s), "memset");
    Check(cudaMemsetAsync(B.flag, 0, 4ull * n, s), "memset");
    Check(cudaMemsetAsync(B.parent_i, 0xFF, 4ull * n, s), "memset");
    Check(cudaMemsetAsync(B.parent_l, 0xFF, 4ull * n, s), "memset");
    Check(cudaMemsetAsync(B.counters, 0, 4ull * (4 + kMaxLevels + 2), s), "memset");
    init_bounds_kernel<<<1, 32, 0, s>>>(B.bounds);
    const uint32_t g256 = (n + 255) / 256;
    prep_kernel<<<std::max(1u, std::min(g256, 8u * (uint32_t)sms)), 256, 0, s>>>(d_verts, nv, d_idx, n, B, shade);
    uint32_t h_status = 0;
    float h_bounds[12];
    Check(cudaMemcpyAsync(&h_status, B.status, 4, cudaMemcpyDeviceToHost, s), "status readback");
    Check(cudaMemcpyAsync(h_bounds, B.bounds, sizeof(h_bounds), cudaMemcpyDeviceToHost, s), "bounds readback");
    Check(cudaStreamSynchronize(s), "prep");
    CHECK_CODE(!(h_status & kPrepBadIndex), FND_ERR_INVALID_ARG, "vertex index out of range (nv = %u)", nv);
    CHECK_CODE(!(h_status & kPrepNonFinite), FND_ERR_INVALID_ARG, "non-finite vertex coordinate");
    for (int a = 0; a < 3; ++a) {
        out.lo[a] = h_bounds[a];
        out.hi[a] = h_bounds[3 + a];
    }
    out.margin = SceneMargin(out.lo, out.hi) * p.margin_scale;
    morton_kernel<<<g256, 256, 0, s>>>(n, B);
    RadixSort(B, n, s);
    if (n >= 2) {
        if (p.ploc_radius)
            PlocHierarchy(B, n, (int)p.ploc_radius, s);
        else
            hierarchy_kernel<<<(n - 1 + 255) / 256, 256, 0, s>>>((int)n, B);
        refit_kernel<<<g256, 256, 0, s>>>(n, B, p.max_leaf, p.trav_cost);
    }
    Check(cudaGetLastError(), "hierarchy launch");
    // root item: internal node 0, or the single leaf
    const uint2 root = make_uint2(n >= 2 ? 0u : kLeafRef, 0u);
    Check(cudaMemcpyAsync(B.qa, &root, sizeof(root), cudaMemcpyHostToDevice, s), "root");
    const uint32_t one[2] = {1u, 0u};  // one wide node (the root), level-0 queue of one item
    Check(cudaMemcpyAsync(B.counters + 0, &one[0], 4, cudaMemcpyHostToDevice, s), "root count");
    Check(cudaMemcpyAsync(B.counters + 4, &one[0], 4, cudaMemcpyHostToDevice, s), "queue count");
    float root_cost = 0.0f, wide_cost = 0.0f;
    float4 rlo{}, rhi{};
    if (n >= 2) {
        Check(cudaMemcpyAsync(&root_cost, B.ncost, 4, cudaMemcpyDeviceToHost, s), "cost readback");
        if (B.dpc) Check(cudaMemcpyAsync(&wide_cost, B.dpc, 4, cudaMemcpyDeviceToHost, s), "cost readback");
        Check(cudaMemcpyAsync(&rlo, B.nlo, 16, cudaMemcpyDeviceToHost, s), "root box");
        Check(cudaMemcpyAsync(&rhi, B.nhi, 16, cudaMemcpyDeviceToHost, s), "root box");
    }
    Check(cudaStreamSynchronize(s), "LBVH");
    out.build_ms = Ms(t0);
    const auto t1 = std::chrono::steady_clock::now();
    WideNode* nodes = nullptr;
    char* tris = nullptr;
    Check(cudaMalloc(&nodes, sizeof(WideNode) * (size_t)n), "cudaMalloc (wide nodes)");
    Scratch S2;
    S2.ptrs.push_back(nodes);
    Check(cudaMalloc(&tris, 48ull * n), "cudaMalloc (triangles)");
    out.d_tris = tris;
    CollapseArgs A{};
    A.B = B;
    A.verts = d_verts;
    A.idx = d_idx;
    A.nodes = nodes;
    A.v0 = reinterpret_cast<float4*>(tris);
    A.v1 = reinterpret_cast<float4*>(tris + 16ull * n);
    A.v2 = reinterpret_cast<float4*>(tris + 32ull * n);
    A.margin = out.margin;
    const int grid = std::max(1, sms * 8);
    for (int level = 0; level < kMaxLevels; ++level) {
        A.level = level;
        collapse_kernel<<<grid, 128, 0, s>>>(A);
    }
    Check(cudaGetLastError(), "collapse launch");
    uint32_t h_counters[4 + kMaxLevels + 2];
    Check(cudaMemcpyAsync(h_counters, B.counters, sizeof(h_counters), cudaMemcpyDeviceToHost, s), "counters");
    Check(cudaMemcpyAsync(&h_status, B.status, 4, cudaMemcpyDeviceToHost, s), "status readback");
    Check(cudaStreamSynchronize(s), "collapse");
    CHECK_CODE(h_counters[4 + kMaxLevels] == 0, FND_ERR_INVALID_SCENE,
               "wide BVH deeper than the traversal stack bound %d", kMaxLevels);
    CHECK_CODE(!(h_status & 4u), FND_ERR_INVALID_SCENE, "child box quantisation failed (scene extent out of range)");
    CHECK_CODE(!(h_status & 8u), FND_ERR_INVALID_SCENE, "GPU build: malformed hierarchy");
    CHECK_CODE(h_counters[1] == n, FND_ERR_INVALID_SCENE, "collapse placed %u of %u triangles", h_counters[1], n);
    out.num_nodes = h_counters[0];
    out.num_refs = n;
    out.leaves = h_counters[2];
    out.depth = 0;
    for (int l = 0; l < kMaxLevels; ++l)
        if (h_counters[4 + l]) out.depth = (uint32_t)l + 1;
    out.num_binary_nodes = 2 * n - 1;
    const float ra = n >= 2 ? half_area(rlo, rhi) : 0.0f;
    out.sah_cost = n >= 2 && ra > 0.0f ? (double)root_cost / (double)ra : 0.0;
    if (B.dpc)
        LOG_RUNTIME(FndRt, INFO, "SAH-optimal collapse: wide-tree cost %.4f (root half-area normalised)",
                    ra > 0.0f ? (double)wide_cost / (double)ra : 0.0);
    // exact-size node array
    void* exact = nullptr;
    Check(cudaMalloc(&exact, sizeof(WideNode) * (size_t)out.num_nodes), "cudaMalloc (wide nodes)");
    Check(cudaMemcpyAsync(exact, nodes, sizeof(WideNode) * (size_t)out.num_nodes, cudaMemcpyDeviceToDevice, s),
          "node copy");
    Check(cudaStreamSynchronize(s), "node copy");
    out.d_nodes = exact;
    out.collapse_ms = Ms(t1);
}

cudaError_t InstanceShade(const float* d_inv, const uint32_t* d_prefix, const uint32_t* d_prim_offset,
                          const float4* const* d_blas_shade, uint32_t n_inst, uint32_t total, float4* d_out,
                          cudaStream_t s) {
    if (total == 0 || n_inst == 0) return cudaSuccess;
    instance_shade_kernel<<<(total + 255) / 256, 256, 0, s>>>(d_inv, d_prefix, d_prim_offset, d_blas_shade, n_inst,
                                                                total, d_out);
    return cudaGetLastError();
}

cudaError_t WriteMaterialIds(float4* d_tri_shade, const uint32_t* d_ids, uint32_t nt, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    write_ids_kernel<<<(nt + 255) / 256, 256, 0, s>>>(d_tri_shade, d_ids, nt);
    return cudaGetLastError();
}

}  // namespace RT
}  // namespace Foundation
