// traverse.cu — persistent closest-hit / any-hit traversal of the compressed
// 8-wide BVH (sm_103a).
//
// Structure (after Aila & Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009, and Ylitie, Karras & Laine, HPG 2017):
//  * persistent warps: the grid is sized to fill every SM once; each warp
//    pulls rays from a global counter with one atomicAdd per refill and hands
//    the new rays to its idle lanes (dynamic fetch: a warp refills once at
//    least `refill_min` lanes are idle, so long rays do not hold 31 idle
//    lanes hostage);
//  * one thread per ray; the traversal state is a "node group" (base index of
//    a node's internal children + the ordered bit mask of children still to
//    visit) and a "triangle group" (base + bit mask of triangles to test);
//  * the stack holds node groups; its top kShort entries live in shared
//    memory (one column per thread, bank-conflict free), deeper entries spill
//    to a thread-local array; the depth bound kMaxStack is checked on the
//    host at scene upload and again on every push (a failed push latches
//    kStatusStackOverflow and ends the ray instead of writing out of bounds).
#include "traverse_launch.hpp"
#include "traverse.cuh"

#include <cfloat>

namespace Foundation {
namespace RT {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kTriGroupFlag = 0x80000000u;

template <bool kAny, bool kStats, int kShort>
__global__ void __launch_bounds__(kTraceBlock) trace_kernel(const TraceLaunch L) {
    static_assert((kShort & (kShort - 1)) == 0, "short stack size must be a power of two");
    __shared__ uint2 s_stack[kShort * kTraceBlock];
    uint2 l_stack[kMaxStack - kShort];
    const int tid = threadIdx.x;
    const uint32_t lane = tid & 31;
    const uint32_t n = L.n_dev ? min(*L.n_dev, L.n) : L.n;
    if (L.ray_total && blockIdx.x == 0 && tid == 0) atomicAdd(L.ray_total, (unsigned long long)n);

    bool active = false, exhausted = false;
    uint32_t ray_id = 0;
    RayState r;
    float best_t = 0.0f;
    uint32_t best_p = FND_INVALID_ID;
    uint32_t ng_base = 0, ng_group = 0, tg_base = 0, tg_mask = 0;
    int sp = 0;
    unsigned long long st_nodes = 0, st_tris = 0;

    for (;;) {
        // ---- dynamic fetch -------------------------------------------------
        const uint32_t idle = __ballot_sync(kFull, !active);
        if (!exhausted && idle != 0u && (__popc(idle) >= (int)L.refill_min || idle == kFull)) {
            const uint32_t cnt = (uint32_t)__popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(L.counter, cnt);
            base = __shfl_sync(kFull, base, 0);
            if (base + cnt >= n) exhausted = true;
            if (!active) {
                const uint32_t id = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (id < n) {
                    const float4 r0 = __ldcs(L.rays + 2 * (size_t)id);
                    const float4 r1 = __ldcs(L.rays + 2 * (size_t)id + 1);
                    r = setup_ray(r0, r1);
                    ray_id = id;
                    best_t = r.tmax;
                    best_p = FND_INVALID_ID;
                    ng_base = 0;
                    ng_group = (1u << 8) | (1u << r.oct);  // pseudo group holding the root in slot 0
                    tg_mask = 0;
                    sp = 0;
                    active = true;
                }
            }
        }
        if (__ballot_sync(kFull, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (!active) continue;

        bool overflow = false;
        // ---- one node --------------------------------------------------------
        if (ng_group & 0xFFu) {
            const uint32_t b = (uint32_t)__ffs(ng_group & 0xFFu) - 1u;
            ng_group &= ~(1u << b);
            const uint32_t slot = b ^ r.oct;
            const uint32_t child = ng_base + (uint32_t)__popc((ng_group >> 8) & ((1u << slot) - 1u));
            if (ng_group & 0xFFu) {
                if (sp >= kMaxStack) {
                    overflow = true;
                } else {
                    const int s = (sp & (kShort - 1)) * kTraceBlock + tid;
                    if (sp >= kShort) l_stack[sp - kShort] = s_stack[s];
                    s_stack[s] = make_uint2(ng_base, ng_group);
                    sp++;
                }
            }
            if (child < L.scene.num_nodes) {
                const NodeHits h = intersect_node(r, L.scene.nodes, child, best_t);
                if (kStats) st_nodes++;
                ng_base = h.child_base;
                ng_group = h.group;
                tg_base = h.tri_base;
                tg_mask = h.tris;
                // a node's triangles must lie inside the triangle arrays
                if (tg_mask && (uint64_t)tg_base + (uint64_t)(32 - __clz(tg_mask)) > L.scene.num_tris) {
                    atomicOr(L.status, kStatusBadIndex);
                    tg_mask = 0;
                    ng_group = 0;
                    sp = 0;
                }
            } else {
                atomicOr(L.status, kStatusBadIndex);
                ng_group = 0;
                tg_mask = 0;
                sp = 0;
            }
        }
        // ---- its triangles ---------------------------------------------------
        while (tg_mask) {
            const uint32_t k = (uint32_t)__ffs(tg_mask) - 1u;
            tg_mask &= tg_mask - 1u;
            const uint32_t ti = tg_base + k;
            const float4 v0 = __ldg(L.scene.v0 + ti);
            const float4 v1 = __ldg(L.scene.v1 + ti);
            const float4 v2 = __ldg(L.scene.v2 + ti);
            if (kStats) st_tris++;
            float t;
            if (intersect_tri(r, v0, v1, v2, best_t, t)) {
                const uint32_t pid = __float_as_uint(v0.w);
                if (kAny) {
                    best_t = t;
                    best_p = pid;
                    tg_mask = 0;
                    ng_group = 0;
                    sp = 0;
                } else if (best_p == FND_INVALID_ID || t < best_t || (t == best_t && pid < best_p)) {
                    best_t = t;
                    best_p = pid;
                }
            }
        }
        // ---- next group or done ------------------------------------------
        if ((ng_group & 0xFFu) == 0u && !overflow) {
            if (sp > 0) {
                sp--;
                const int s = (sp & (kShort - 1)) * kTraceBlock + tid;
                const uint2 e = s_stack[s];
                if (sp >= kShort) s_stack[s] = l_stack[sp - kShort];
                if (e.x & kTriGroupFlag) {
                    tg_base = e.x & ~kTriGroupFlag;
                    tg_mask = e.y;
                    ng_group = 0;
                } else {
                    ng_base = e.x;
                    ng_group = e.y;
                }
                continue;
            }
        } else if (!overflow) {
            continue;
        }
        // ray finished (or aborted on overflow)
        if (overflow) atomicOr(L.status, kStatusStackOverflow);
        if (kAny) {
            __stcs(L.occluded + ray_id, (uint8_t)(best_p != FND_INVALID_ID ? 1 : 0));
        } else {
            const uint2 o = make_uint2(best_p, best_p == FND_INVALID_ID ? 0x7F800000u : __float_as_uint(best_t));
            __stcs(reinterpret_cast<uint2*>(L.hits) + ray_id, o);
        }
        active = false;
    }
    if (kStats) {
        for (int o = 16; o > 0; o >>= 1) {
            st_nodes += __shfl_down_sync(kFull, st_nodes, o);
            st_tris += __shfl_down_sync(kFull, st_tris, o);
        }
        if (lane == 0) {
            atomicAdd(L.stats + 0, st_nodes);
            atomicAdd(L.stats + 1, st_tris);
        }
    }
}

__global__ void fill_miss_kernel(uint2* hits, uint8_t* occluded, uint32_t cap, const uint32_t* n_dev) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = n_dev ? min(*n_dev, cap) : cap;
    if (i >= n) return;
    if (hits) hits[i] = make_uint2(FND_INVALID_ID, 0x7F800000u);
    if (occluded) occluded[i] = 0;
}

template <bool kAny, bool kStats>
const void* kernel_ptr() {
    return reinterpret_cast<const void*>(&trace_kernel<kAny, kStats, kTraceShortStack>);
}

template <bool kAny, bool kStats>
cudaError_t launch(const TraceLaunch& L, int grid, cudaStream_t stream) {
    trace_kernel<kAny, kStats, kTraceShortStack><<<grid, kTraceBlock, 0, stream>>>(L);
    return cudaGetLastError();
}

}  // namespace

cudaError_t TraceOccupancy(int variant, int* blocks_per_sm) {
    const void* fn = nullptr;
    switch (variant) {
        case 0: fn = kernel_ptr<false, false>(); break;
        case 1: fn = kernel_ptr<true, false>(); break;
        case 2: fn = kernel_ptr<false, true>(); break;
        default: fn = kernel_ptr<true, true>(); break;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kTraceBlock, 0);
}

cudaError_t LaunchTrace(const TraceLaunch& L, bool any, bool stats, int grid, cudaStream_t stream) {
    if (L.n == 0) return cudaSuccess;
    if (L.scene.num_nodes == 0) {
        const uint32_t threads = 256;
        fill_miss_kernel<<<(L.n + threads - 1) / threads, threads, 0, stream>>>(
            any ? nullptr : reinterpret_cast<uint2*>(L.hits), any ? L.occluded : nullptr, L.n, L.n_dev);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(L.counter, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    if (any) return stats ? launch<true, true>(L, grid, stream) : launch<true, false>(L, grid, stream);
    return stats ? launch<false, true>(L, grid, stream) : launch<false, false>(L, grid, stream);
}

}  // namespace RT
}  // namespace Foundation
