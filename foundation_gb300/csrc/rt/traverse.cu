// traverse.cu — persistent closest-hit / any-hit traversal of the compressed
// 8-wide BVH (sm_103a), for one scene (trace_kernel) or for a table of
// (scene, ray batch, query kind) jobs in one launch (batch_kernel).
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
//  * a node's hit mask goes to the ray's traversal order (bit i: slot
//    i ^ oct) through a shared 8 x 256-byte table in the single-scene and
//    batched kernels (one load in place of three conditional bit swaps:
//    +1.6% on the issue-bound kernel; the two-level kernel, whose shared
//    memory already holds the world rays, keeps the swaps);
//  * the stack holds node groups; its top kShort entries live in shared
//    memory (one column per thread, bank-conflict free), deeper entries spill
//    to a thread-local array; the depth bound kMaxStack is checked on the
//    host at scene upload and again on every push (a failed push latches
//    kStatusStackOverflow and ends the ray instead of writing out of bounds).
// Block size, short-stack depth and the refill threshold are launch
// parameters chosen by the autotuner (capi/capi_batch.cpp); every
// combination below is compiled. Two-level scenes (instances) run the same
// loop with kTwoLevel: a lane descending into an instance pushes a return
// marker and swaps its ray and node arrays to the instance's object space.
#include <cfloat>

#include "traverse.cuh"
#include "ray_sort.hpp"
#include "traverse_launch.hpp"

namespace Foundation {
namespace RT {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kTriGroupFlag = 0x80000000u;

struct Common {
    uint32_t* counter;
    uint32_t* status;
    unsigned long long* stats;
    uint32_t refill_min;
    uint32_t postpone_min;  // postpone a triangle group when fewer lanes than this have one (0: never)
};

// ---- work sources -----------------------------------------------------------
// One scene, one ray array, one query kind for the whole launch.
struct SingleSource {
    DeviceScene scene;
    const float4* rays;
    void* hits;
    uint8_t* occluded;
    const uint32_t* order;  // fetch position -> ray index (coherence order), or null
    uint32_t n;
    struct Lane {};
    __device__ __forceinline__ uint32_t map(uint32_t pos) const { return order ? __ldg(order + pos) : pos; }
    __device__ __forceinline__ void load(uint32_t id, float4& r0, float4& r1, Lane&) const {
        r0 = __ldcs(rays + 2 * (size_t)id);
        r1 = __ldcs(rays + 2 * (size_t)id + 1);
    }
    __device__ __forceinline__ const DeviceScene& scene_of(const Lane&) const { return scene; }
    __device__ __forceinline__ bool any_of(const Lane&, bool dflt) const { return dflt; }
    __device__ __forceinline__ void store(uint32_t id, const Lane&, bool any, uint32_t prim, float t) const {
        if (any) {
            __stcs(occluded + id, (uint8_t)(prim != FND_INVALID_ID ? 1 : 0));
        } else {
            const uint2 o = make_uint2(prim, prim == FND_INVALID_ID ? 0x7F800000u : __float_as_uint(t));
            __stcs(reinterpret_cast<uint2*>(hits) + id, o);
        }
    }
};

// A job table; a global ray id is mapped to its job by binary search over
// the prefix of ray counts (kept in shared memory when it fits).
struct BatchSource {
    const BatchJob* jobs;
    const uint32_t* prefix;  // njobs + 1 entries
    uint32_t njobs;
    uint32_t n;
    struct Lane {
        uint32_t job;
        uint32_t local;
        DeviceScene scene;
        bool any;
    };
    __device__ __forceinline__ uint32_t map(uint32_t pos) const { return pos; }
    __device__ __forceinline__ void load(uint32_t id, float4& r0, float4& r1, Lane& ln) const {
        uint32_t lo = 0, hi = njobs;  // prefix[lo] <= id < prefix[hi]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (prefix[mid] <= id)
                lo = mid;
            else
                hi = mid;
        }
        ln.job = lo;
        ln.local = id - prefix[lo];
        const BatchJob& j = jobs[lo];
        ln.scene = j.scene;
        ln.any = j.any != 0;
        r0 = __ldcs(j.rays + 2 * (size_t)ln.local);
        r1 = __ldcs(j.rays + 2 * (size_t)ln.local + 1);
    }
    __device__ __forceinline__ const DeviceScene& scene_of(const Lane& ln) const { return ln.scene; }
    __device__ __forceinline__ bool any_of(const Lane& ln, bool) const { return ln.any; }
    __device__ __forceinline__ void store(uint32_t, const Lane& ln, bool any, uint32_t prim, float t) const {
        const BatchJob& j = jobs[ln.job];
        if (any) {
            __stcs(static_cast<uint8_t*>(j.out) + ln.local, (uint8_t)(prim != FND_INVALID_ID ? 1 : 0));
        } else {
            const uint2 o = make_uint2(prim, prim == FND_INVALID_ID ? 0x7F800000u : __float_as_uint(t));
            __stcs(reinterpret_cast<uint2*>(j.out) + ln.local, o);
        }
    }
};

// Rays against a two-level scene: the top level's leaves are instances.
struct InstancedSource {
    DeviceScene scene;  // the top level
    const InstanceRec* inst;
    uint32_t num_inst;
    const float4* rays;
    void* hits;
    uint8_t* occluded;
    uint32_t n;
    struct Lane {};
    __device__ __forceinline__ uint32_t map(uint32_t pos) const { return pos; }
    __device__ __forceinline__ void load(uint32_t id, float4& r0, float4& r1, Lane&) const {
        r0 = __ldg(rays + 2 * (size_t)id);
        r1 = __ldg(rays + 2 * (size_t)id + 1);
    }
    __device__ __forceinline__ const DeviceScene& scene_of(const Lane&) const { return scene; }
    __device__ __forceinline__ bool any_of(const Lane&, bool dflt) const { return dflt; }
    __device__ __forceinline__ void store(uint32_t id, const Lane&, bool any, uint32_t prim, float t) const {
        if (any) {
            __stcs(occluded + id, (uint8_t)(prim != FND_INVALID_ID ? 1 : 0));
        } else {
            const uint2 o = make_uint2(prim, prim == FND_INVALID_ID ? 0x7F800000u : __float_as_uint(t));
            __stcs(reinterpret_cast<uint2*>(hits) + id, o);
        }
    }
};

constexpr uint32_t kInstanceMarker = 0xFFFFFFFFu;  // stack entry: return to the top level

// ---- warp-cooperative triangle tests ----------------------------------------
// After a node step each lane holds a triangle group (base + bit mask); lane
// by lane the groups are uneven (most lanes have none, a few have a whole
// leaf set), so a loop over its own group leaves most of the warp idle. Here
// the warp lays its (ray, triangle) pairs out in lane order and tests up to
// 32 of them per round, one per lane: a round takes the owners (lanes with a
// group) in ascending lane order while their groups fit, each owner's
// triangles in ascending order. A pair lane finds its owner from the mask of
// group start positions (an OR over the warp) and its triangle as the k-th
// set bit of the owner's mask; the owner's ray constants come from its slot
// in shared memory, written when the ray was fetched. Each owner merges the
// hits of its pairs with the sequential rule (smaller t, on equal t the lower
// id), so the result is the one of a loop over its own group. A round tests
// against the owner's best t at its start; a later round sees the improved
// bound.

// Position of the k-th set bit (k from 0) of m; k < popc(m).
__device__ __forceinline__ uint32_t select_bit(uint32_t m, uint32_t k) {
    uint32_t pos = 0, c;
    c = (uint32_t)__popc(m & 0xFFFFu);
    if (k >= c) { k -= c; m >>= 16; pos += 16; }
    c = (uint32_t)__popc(m & 0xFFu);
    if (k >= c) { k -= c; m >>= 8; pos += 8; }
    c = (uint32_t)__popc(m & 0xFu);
    if (k >= c) { k -= c; m >>= 4; pos += 4; }
    c = (uint32_t)__popc(m & 0x3u);
    if (k >= c) { k -= c; m >>= 2; pos += 2; }
    return pos + (k >= (m & 1u) ? 1u : 0u);
}

// Per-thread shared slots of the cooperative stage (kBlock threads); with
// kMulti (lanes of one warp in different scenes) also the triangle planes of
// each lane's scene.
template <int kBlock, bool kMulti>
struct CoopShared {
    float4 ray[2 * kBlock];  // [tid]: ox, oy, oz, tmin; [kBlock + tid]: -Sx, -Sy, Sz, kz bits
    uint32_t owner[kBlock];  // per warp: lane of the group starting at a position
    float t[kBlock];         // per warp: hit t of the pair at a position
    uint32_t pid[kBlock];    // per warp: hit id of the pair at a position
    const float4* planes[kMulti ? 3 * kBlock : 1];  // [a * kBlock + tid]: vertex plane a of the lane's scene
    uint32_t prim_off[kMulti ? kBlock : 1];         // [tid]: hit-id offset of the lane's scene (instances)
};

template <int kBlock, bool kMulti>
__device__ __forceinline__ void coop_store_ray(CoopShared<kBlock, kMulti>* cs, const RayState& r,
                                               const DeviceScene& sc, uint32_t prim_off = 0u) {
    cs->ray[threadIdx.x] = make_float4(r.ox, r.oy, r.oz, r.tmin);
    cs->ray[kBlock + threadIdx.x] = make_float4(r.nSx, r.nSy, r.Sz, __int_as_float(r.kz));
    if constexpr (kMulti) {
        cs->planes[threadIdx.x] = sc.v0;
        cs->planes[kBlock + threadIdx.x] = sc.v1;
        cs->planes[2 * kBlock + threadIdx.x] = sc.v2;
        cs->prim_off[threadIdx.x] = prim_off;
    }
}

// All 32 lanes of the warp call this; lanes without a ray pass mine_ok = false.
template <int kKind, bool kStats, int kBlock, bool kMulti, bool kOffsets = false>
__device__ __forceinline__ void coop_triangles(const DeviceScene& sc, bool mine_ok, bool any_hit, uint32_t tg_base,
                                               uint32_t& tg_mask, float& best_t, uint32_t& best_p,
                                               uint32_t& ng_group, int& sp, CoopShared<kBlock, kMulti>* cs,
                                               unsigned long long& st_tris, uint32_t& st_wtri) {
    if (__ballot_sync(kFull, mine_ok && tg_mask != 0u) == 0u) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t wbase = threadIdx.x & ~31u;
    for (int round = 0; round < 33; ++round) {  // every round empties at least one group
        const uint32_t mine = mine_ok ? tg_mask : 0u;
        const uint32_t cnt = (uint32_t)__popc(mine);
        uint32_t inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, inc, o);
            if (lane >= (uint32_t)o) inc += v;
        }
        if (__shfl_sync(kFull, inc, 31) == 0u) break;
        const uint32_t off = inc - cnt;
        // this round: the owners whose whole group fits in positions 0..31
        // (the first owner always does, at position 0)
        const bool part = cnt != 0u && inc <= 32u;
        const uint32_t starts = __reduce_or_sync(kFull, part ? 1u << off : 0u);
        const uint32_t np = __reduce_max_sync(kFull, part ? inc : 0u);
        if (part) cs->owner[wbase + off] = lane;
        __syncwarp();
        const uint32_t q = 31u - (uint32_t)__clz(starts & ((2u << lane) - 1u));  // start of this lane's group
        const uint32_t owner = lane < np ? cs->owner[wbase + q] : 0u;
        const uint32_t omask = __shfl_sync(kFull, mine, owner);
        const uint32_t obase = __shfl_sync(kFull, tg_base, owner);
        const float qt = __shfl_sync(kFull, best_t, owner);
        bool hit = false;
        float t = 0.0f;
        uint32_t pid = 0;
        if (lane < np) {
            const uint32_t ti = obase + select_bit(omask, lane - q);
            const float4 a = cs->ray[wbase + owner];
            const float4 b = cs->ray[kBlock + wbase + owner];
            RayState rq;
            rq.ox = a.x;
            rq.oy = a.y;
            rq.oz = a.z;
            rq.tmin = a.w;
            rq.nSx = b.x;
            rq.nSy = b.y;
            rq.Sz = b.z;
            rq.kz = __float_as_int(b.w);
            const float4 *p0 = sc.v0, *p1 = sc.v1, *p2 = sc.v2;
            if constexpr (kMulti) {
                p0 = cs->planes[wbase + owner];
                p1 = cs->planes[kBlock + wbase + owner];
                p2 = cs->planes[2 * kBlock + wbase + owner];
            }
            const float4 v0 = __ldg(p0 + ti);
            hit = intersect_tri(rq, v0, __ldg(p1 + ti), __ldg(p2 + ti), qt, t);
            pid = __float_as_uint(v0.w);
            if constexpr (kOffsets) pid += cs->prim_off[wbase + owner];  // global id of an instance's triangle
            if (kStats) {
                st_tris++;
                if (lane == 0u) st_wtri++;
            }
        }
        if (part && mine_ok) tg_mask = 0u;
        const uint32_t hm = __ballot_sync(kFull, hit);
        if (hm) {
            if (hit) {
                cs->t[wbase + lane] = t;
                cs->pid[wbase + lane] = pid;
            }
            __syncwarp();
            uint32_t c = part ? hm & (cnt == 32u ? kFull : ((1u << cnt) - 1u) << off) : 0u;
            while (c) {
                const uint32_t j = (uint32_t)__ffs(c) - 1u;
                c &= c - 1u;
                const float tj = cs->t[wbase + j];
                const uint32_t pj = cs->pid[wbase + j];
                if (kKind == 1 || (kKind == 2 && any_hit)) {
                    best_t = tj;
                    best_p = pj;
                    tg_mask = 0;
                    ng_group = 0;
                    sp = 0;
                    break;
                }
                if (best_p == FND_INVALID_ID || tj < best_t || (tj == best_t && pj < best_p)) {
                    best_t = tj;
                    best_p = pj;
                }
            }
        }
        __syncwarp();  // the slots are rewritten by the next round
    }
}

// ---- the persistent traversal loop ----------------------------------------
// kKind: 0 closest, 1 any, 2 per-lane (from the source). kTwoLevel: the
// source is an InstancedSource (triangle leaves of the top level are
// instances; per-lane node / triangle arrays).
template <class Src, int kKind, bool kStats, int kShort, int kBlock, bool kTwoLevel = false, bool kCoop = false,
          bool kMulti = false>
__device__ __forceinline__ void persistent_trace(const Src& src, const Common& C, uint2* s_stack,
                                                 CoopShared<kBlock, kMulti>* s_coop = nullptr,
                                                 RayState* s_world = nullptr, const uint8_t* s_perm = nullptr) {
    // two-level cooperative rounds: each lane's planes and hit-id offset
    // come from its own slot (the lanes of a warp sit in different instances)
    static_assert(!(kCoop && kTwoLevel) || kMulti, "two-level cooperative rounds need per-lane scenes");
    static_assert((kShort & (kShort - 1)) == 0, "short stack size must be a power of two");
    uint2 l_stack[kMaxStack - kShort];
    const int tid = threadIdx.x;
    const uint32_t lane = tid & 31;
    const uint32_t n = src.n;

    bool active = false, exhausted = false, any_hit = kKind == 1;
    uint32_t ray_id = 0;
    typename Src::Lane ln{};
    RayState r;
    float best_t = 0.0f;
    uint32_t best_p = FND_INVALID_ID;
    uint32_t ng_base = 0, ng_group = 0, tg_base = 0, tg_mask = 0;
    int sp = 0;
    unsigned long long st_nodes = 0, st_tris = 0;
    uint32_t st_wnode = 0, st_wtri = 0;  // warp steps, counted by the lowest active lane
    // two-level state: the arrays the lane traverses now, and its instance
    bool in_blas = false, moved = false;  // moved: r holds an object-space ray, the world one is in s_world
    DeviceScene cur{};
    uint32_t prim_off = 0;

    auto push = [&](uint2 e) -> bool {
        if (sp >= kMaxStack) return false;
        const int s = (sp & (kShort - 1)) * kBlock + tid;
        if (sp >= kShort) l_stack[sp - kShort] = s_stack[s];
        s_stack[s] = e;
        sp++;
        return true;
    };
    // two-level: descend into instance I (from the top level, r the world
    // ray). Its object-space ray replaces r, and the world ray's set-up
    // waits in s_world for the return; an identity instance keeps r.
    auto enter_instance = [&](const InstanceRec& I) {
        if constexpr (kTwoLevel) {
            if (!(__ldg(&I.flags) & kInstanceIdentity)) {
                float inv[12];
                for (int q = 0; q < 12; ++q) inv[q] = __ldg(I.inv + q);
                float4 r0, r1, o0, o1;
                src.load(ray_id, r0, r1, ln);
                instance_ray(inv, r0, r1, o0, o1);
                s_world[tid] = r;
                r = setup_ray(o0, o1);
                moved = true;
            }
            cur = I.blas;
            prim_off = __ldg(&I.prim_offset);
            in_blas = true;
            ng_base = 0;
            ng_group = cur.num_nodes ? (1u << 8) | (1u << r.oct) : 0u;
            tg_mask = 0;
        }
    };

    for (;;) {
        // ---- dynamic fetch -------------------------------------------------
        const uint32_t idle = __ballot_sync(kFull, !active);
        if (!exhausted && idle != 0u && (__popc(idle) >= (int)C.refill_min || idle == kFull)) {
            const uint32_t cnt = (uint32_t)__popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(C.counter, cnt);
            base = __shfl_sync(kFull, base, 0);
            if (base + cnt >= n) exhausted = true;
            if (!active) {
                const uint32_t pos = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (pos < n) {
                    const uint32_t id = src.map(pos);
                    float4 r0, r1;
                    src.load(id, r0, r1, ln);
                    if (kKind == 2) any_hit = src.any_of(ln, false);
                    r = setup_ray(r0, r1);
                    if constexpr (kCoop) coop_store_ray<kBlock, kMulti>(s_coop, r, src.scene_of(ln));
                    ray_id = id;
                    best_t = r.tmax;
                    best_p = FND_INVALID_ID;
                    ng_base = 0;
                    ng_group = (1u << 8) | (1u << r.oct);  // pseudo group holding the root in slot 0
                    if (src.scene_of(ln).num_nodes == 0) ng_group = 0;  // empty scene: a miss
                    tg_mask = 0;
                    sp = 0;
                    active = true;
                    if constexpr (kTwoLevel) {
                        in_blas = false;
                        moved = false;
                        cur = src.scene;
                        prim_off = 0;
                    }
                }
            }
        }
        if (__ballot_sync(kFull, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        // the cooperative triangle stage needs the whole warp: idle lanes
        // run the iteration with empty node and triangle groups
        if (!kCoop && !active) continue;

        const DeviceScene& sc = kTwoLevel ? cur : src.scene_of(ln);
        bool overflow = false;
        // ---- one node --------------------------------------------------------
        if ((kCoop ? active : true) && (ng_group & 0xFFu)) {
            const uint32_t b = (uint32_t)__ffs(ng_group & 0xFFu) - 1u;
            ng_group &= ~(1u << b);
            const uint32_t slot = b ^ r.oct;
            const uint32_t child = ng_base + (uint32_t)__popc((ng_group >> 8) & ((1u << slot) - 1u));
            if (ng_group & 0xFFu) overflow = !push(make_uint2(ng_base, ng_group));
            if (overflow) {
            } else if (child < sc.num_nodes) {
                const NodeHits h = intersect_node(r, sc.nodes, child, best_t, s_perm);
                if (kStats) {
                    st_nodes++;
                    if (lane == (uint32_t)__ffs(__activemask()) - 1u) st_wnode++;
                }
                ng_base = h.child_base;
                ng_group = h.group;
                tg_base = h.tri_base;
                tg_mask = h.tris;
                // a node's triangles must lie inside the triangle arrays
                if (tg_mask && (uint64_t)tg_base + (uint64_t)(32 - __clz(tg_mask)) > sc.num_tris) {
                    atomicOr(C.status, kStatusBadIndex);
                    tg_mask = 0;
                    ng_group = 0;
                    sp = 0;
                }
                // triangle postponement (Ylitie et al. 2017): when only a few
                // lanes of the warp have triangles to test, keep traversing
                // nodes with the rest and test the triangles later
                if (!kTwoLevel && !kCoop && C.postpone_min) {
                    const uint32_t tri_lanes = __ballot_sync(__activemask(), tg_mask != 0u);
                    if (tg_mask && (ng_group & 0xFFu) && (uint32_t)__popc(tri_lanes) < C.postpone_min &&
                        push(make_uint2(tg_base | kTriGroupFlag, tg_mask)))
                        tg_mask = 0;
                }
            } else {
                atomicOr(C.status, kStatusBadIndex);
                ng_group = 0;
                tg_mask = 0;
                sp = 0;
            }
        }
        // ---- its triangles, tested by the whole warp ------------------------
        if constexpr (kCoop) {
            if constexpr (kTwoLevel) {
                // a top-level leaf holds instances: the lane enters the first
                // valid one by itself (resume order as in the per-lane loop
                // below) and publishes its object-space ray for the rounds
                while (active && !overflow && !in_blas && tg_mask) {
                    const uint32_t k = (uint32_t)__ffs(tg_mask) - 1u;
                    tg_mask &= tg_mask - 1u;
                    const uint32_t iid = __float_as_uint(__ldg(cur.v0 + tg_base + k).w);
                    if (iid >= src.num_inst) {
                        atomicOr(C.status, kStatusBadIndex);
                        continue;
                    }
                    overflow = ((ng_group & 0xFFu) && !push(make_uint2(ng_base, ng_group))) ||
                               (tg_mask && !push(make_uint2(tg_base | kTriGroupFlag, tg_mask))) ||
                               !push(make_uint2(kInstanceMarker, 0u));
                    if (overflow) break;
                    const InstanceRec& I = src.inst[iid];
                    enter_instance(I);
                    coop_store_ray<kBlock, kMulti>(s_coop, r, cur, prim_off);
                }
            }
            coop_triangles<kKind, kStats, kBlock, kMulti, kTwoLevel>(sc, active && !overflow, any_hit, tg_base,
                                                                     tg_mask, best_t, best_p, ng_group, sp, s_coop,
                                                                     st_tris, st_wtri);
            if (!active) continue;
        }
        // ---- its triangles (or, on the top level, its instances) ------------
        while (!kCoop && tg_mask && !overflow) {
            const uint32_t k = (uint32_t)__ffs(tg_mask) - 1u;
            tg_mask &= tg_mask - 1u;
            const uint32_t ti = tg_base + k;
            if constexpr (kTwoLevel) {
                if (!in_blas) {
                    const uint32_t iid = __float_as_uint(__ldg(sc.v0 + ti).w);
                    if (iid >= src.num_inst) {
                        atomicOr(C.status, kStatusBadIndex);
                        continue;
                    }
                    // resume order after the instance: this leaf's other
                    // instances, then the node's other children
                    overflow = ((ng_group & 0xFFu) && !push(make_uint2(ng_base, ng_group))) ||
                               (tg_mask && !push(make_uint2(tg_base | kTriGroupFlag, tg_mask))) ||
                               !push(make_uint2(kInstanceMarker, 0u));
                    if (overflow) break;
                    const InstanceRec& I = src.inst[iid];
                    enter_instance(I);
                    break;
                }
            }
            const float4 v0 = __ldg(sc.v0 + ti);
            const float4 v1 = __ldg(sc.v1 + ti);
            const float4 v2 = __ldg(sc.v2 + ti);
            if (kStats) {
                st_tris++;
                if (lane == (uint32_t)__ffs(__activemask()) - 1u) st_wtri++;
            }
            float t;
            if (intersect_tri(r, v0, v1, v2, best_t, t)) {
                const uint32_t pid = __float_as_uint(v0.w) + (kTwoLevel ? prim_off : 0u);
                if (any_hit) {
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
        if ((ng_group & 0xFFu) == 0u && tg_mask == 0u && !overflow) {
            if (sp > 0) {
                sp--;
                const int s = (sp & (kShort - 1)) * kBlock + tid;
                const uint2 e = s_stack[s];
                if (sp >= kShort) s_stack[s] = l_stack[sp - kShort];
                bool marker = false;
                if constexpr (kTwoLevel) {
                    if (e.x == kInstanceMarker) {
                        // back to the top level: the world ray again
                        if (moved) r = s_world[tid];
                        moved = false;
                        cur = src.scene;
                        prim_off = 0;
                        in_blas = false;
                        ng_group = 0;
                        tg_mask = 0;
                        marker = true;
                    }
                }
                if (marker) {
                } else if (e.x & kTriGroupFlag) {
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
        if (overflow) atomicOr(C.status, kStatusStackOverflow);
        src.store(ray_id, ln, any_hit, best_p, best_t);
        active = false;
        ng_group = 0;
        tg_mask = 0;
    }
    if (kStats) {
        for (int o = 16; o > 0; o >>= 1) {
            st_nodes += __shfl_down_sync(kFull, st_nodes, o);
            st_tris += __shfl_down_sync(kFull, st_tris, o);
            st_wnode += __shfl_down_sync(kFull, st_wnode, o);
            st_wtri += __shfl_down_sync(kFull, st_wtri, o);
        }
        if (lane == 0) {
            atomicAdd(C.stats + 0, st_nodes);
            atomicAdd(C.stats + 1, st_tris);
            atomicAdd(C.stats + 2, (unsigned long long)st_wnode);
            atomicAdd(C.stats + 3, (unsigned long long)st_wtri);
        }
    }
}

// 36 resident warps per SM (9 blocks of 128 threads: at most 56 registers)
// unless the block is 256 threads wide.
constexpr int MinBlocks(int block) { return block == 256 ? 4 : 1152 / block; }

// Fills the 8 x 256 byte table of xor_permute8 (all threads of the block).
__device__ __forceinline__ void fill_perm(uint8_t* t) {
    for (uint32_t i = threadIdx.x; i < 2048u; i += blockDim.x) t[i] = (uint8_t)xor_permute8(i & 255u, i >> 8);
    uint32_t* m = reinterpret_cast<uint32_t*>(t + 2048);
    for (uint32_t i = threadIdx.x; i < 256u; i += blockDim.x) m[i] = ((2u << ((i >> 5) & 3u)) - 1u) << (i & 31u);
    __syncthreads();
}

template <bool kAny, bool kStats, int kShort, int kBlock>
__global__ void __launch_bounds__(kBlock, MinBlocks(kBlock)) trace_kernel(const TraceLaunch L) {
    __shared__ uint2 s_stack[kShort * kBlock];
    __shared__ CoopShared<kBlock, false> s_coop;
    __shared__ __align__(16) uint8_t s_perm[2048 + 1024];
    fill_perm(s_perm);
    SingleSource src;
    src.scene = L.scene;
    src.rays = L.rays;
    src.hits = L.hits;
    src.occluded = L.occluded;
    src.order = L.order;
    src.n = L.n_dev ? min(*L.n_dev, L.n) : L.n;
    if (L.ray_total && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(L.ray_total, (unsigned long long)src.n);
    const Common C{L.counter, L.status, L.stats, L.refill_min, L.postpone_min};
    persistent_trace<SingleSource, kAny ? 1 : 0, kStats, kShort, kBlock, false, true>(src, C, s_stack, &s_coop, nullptr,
                                                                                     s_perm);
}

template <int kShort, int kBlock>
__global__ void __launch_bounds__(kBlock, MinBlocks(kBlock)) batch_kernel(const BatchLaunch B) {
    __shared__ uint2 s_stack[kShort * kBlock];
    __shared__ CoopShared<kBlock, true> s_coop;
    __shared__ __align__(16) uint8_t s_perm[2048 + 1024];
    fill_perm(s_perm);
    BatchSource src;
    src.jobs = B.jobs;
    src.prefix = B.prefix;
    src.njobs = B.njobs;
    src.n = B.total;
    const Common C{B.counter, B.status, nullptr, B.refill_min, B.postpone_min};
    persistent_trace<BatchSource, 2, false, kShort, kBlock, false, true, true>(src, C, s_stack, &s_coop, nullptr,
                                                                             s_perm);
}

template <bool kAny>
__global__ void __launch_bounds__(128, 8) instanced_trace_kernel(const InstancedLaunch L) {
    __shared__ uint2 s_stack[8 * 128];
    __shared__ CoopShared<128, true> s_coop;
    __shared__ RayState s_world[128];
    InstancedSource src;
    src.scene = L.tlas;
    src.inst = L.inst;
    src.num_inst = L.num_inst;
    src.rays = L.rays;
    src.hits = L.hits;
    src.occluded = L.occluded;
    src.n = L.n_dev ? min(*L.n_dev, L.n) : L.n;
    if (L.ray_total && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(L.ray_total, (unsigned long long)src.n);
    const Common C{L.counter, L.status, nullptr, 8u, 0u};
    persistent_trace<InstancedSource, kAny ? 1 : 0, false, 8, 128, true, true, true>(src, C, s_stack, &s_coop,
                                                                                     s_world);
}

__global__ void fill_miss_kernel(uint2* hits, uint8_t* occluded, uint32_t cap, const uint32_t* n_dev) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = n_dev ? min(*n_dev, cap) : cap;
    if (i >= n) return;
    if (hits) hits[i] = make_uint2(FND_INVALID_ID, 0x7F800000u);
    if (occluded) occluded[i] = 0;
}

// ---- variant tables ---------------------------------------------------------
template <bool kAny, bool kStats, int kShort, int kBlock>
const void* trace_ptr() {
    return reinterpret_cast<const void*>(&trace_kernel<kAny, kStats, kShort, kBlock>);
}

int block_index(int block) { return block == 64 ? 0 : (block == 256 ? 2 : 1); }
int short_index(int s) { return s == 4 ? 0 : (s == 16 ? 2 : 1); }

template <bool kAny>
const void* select_trace(const TraceConfig& c, bool stats) {
    if (stats) return kAny ? trace_ptr<true, true, 8, 128>() : trace_ptr<false, true, 8, 128>();
    static const void* table[3][3] = {
        {trace_ptr<kAny, false, 4, 64>(), trace_ptr<kAny, false, 8, 64>(), trace_ptr<kAny, false, 16, 64>()},
        {trace_ptr<kAny, false, 4, 128>(), trace_ptr<kAny, false, 8, 128>(), trace_ptr<kAny, false, 16, 128>()},
        {trace_ptr<kAny, false, 4, 256>(), trace_ptr<kAny, false, 8, 256>(), trace_ptr<kAny, false, 16, 256>()},
    };
    return table[block_index(c.block)][short_index(c.short_stack)];
}

const void* select_batch(const TraceConfig& c) {
    static const void* table[3][3] = {
        {(const void*)&batch_kernel<4, 64>, (const void*)&batch_kernel<8, 64>, (const void*)&batch_kernel<16, 64>},
        {(const void*)&batch_kernel<4, 128>, (const void*)&batch_kernel<8, 128>, (const void*)&batch_kernel<16, 128>},
        {(const void*)&batch_kernel<4, 256>, (const void*)&batch_kernel<8, 256>, (const void*)&batch_kernel<16, 256>},
    };
    return table[block_index(c.block)][short_index(c.short_stack)];
}

int normalized_block(int b) { return b == 64 || b == 256 ? b : 128; }

}  // namespace

bool ValidTraceConfig(const TraceConfig& c) {
    return (c.block == 64 || c.block == 128 || c.block == 256) &&
           (c.short_stack == 4 || c.short_stack == 8 || c.short_stack == 16) && c.refill_min >= 1 &&
           c.refill_min <= 32 && c.postpone_min <= 32 && c.blocks_per_sm >= 0 && c.blocks_per_sm <= 32 &&
           ValidSortBits(c.sort_bits);
}

cudaError_t TraceOccupancy(int variant, int* blocks_per_sm) {
    TraceConfig c{};
    return TraceOccupancyFor(c, variant, blocks_per_sm);
}

cudaError_t TraceOccupancyFor(const TraceConfig& c, int variant, int* blocks_per_sm) {
    const bool any = variant == 1 || variant == 3, stats = variant >= 2;
    const void* fn = variant == 4 ? select_batch(c) : (any ? select_trace<true>(c, stats) : select_trace<false>(c, stats));
    const int block = stats ? 128 : normalized_block(c.block);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, block, 0);
}

cudaError_t LaunchTraceConfigured(const TraceLaunch& L, bool any, bool stats, const TraceConfig& c, int grid,
                                  cudaStream_t stream) {
    if (L.n == 0) return cudaSuccess;
    if (L.scene.num_nodes == 0) {
        const uint32_t threads = 256;
        fill_miss_kernel<<<(L.n + threads - 1) / threads, threads, 0, stream>>>(
            any ? nullptr : reinterpret_cast<uint2*>(L.hits), any ? L.occluded : nullptr, L.n, L.n_dev);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(L.counter, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    const void* fn = any ? select_trace<true>(c, stats) : select_trace<false>(c, stats);
    const int block = stats ? 128 : normalized_block(c.block);
    TraceLaunch arg = L;
    arg.refill_min = c.refill_min ? c.refill_min : L.refill_min;
    arg.postpone_min = c.postpone_min;
    void* params[] = {&arg};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), params, 0, stream);
}

cudaError_t LaunchTrace(const TraceLaunch& L, bool any, bool stats, int grid, cudaStream_t stream) {
    TraceConfig c{};
    c.refill_min = L.refill_min;
    return LaunchTraceConfigured(L, any, stats, c, grid, stream);
}

cudaError_t LaunchInstanced(const InstancedLaunch& L, bool any, int sm_count, cudaStream_t stream) {
    if (L.n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(L.counter, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    const void* fn = any ? reinterpret_cast<const void*>(&instanced_trace_kernel<true>)
                         : reinterpret_cast<const void*>(&instanced_trace_kernel<false>);
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 128, 0);
    if (e != cudaSuccess) return e;
    InstancedLaunch arg = L;
    void* params[] = {&arg};
    return cudaLaunchKernel(fn, dim3(sm_count * (blocks > 0 ? blocks : 1)), dim3(128), params, 0, stream);
}

cudaError_t LaunchBatch(const BatchLaunch& B, const TraceConfig& c, int grid, cudaStream_t stream) {
    if (B.total == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(B.counter, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    BatchLaunch arg = B;
    arg.refill_min = c.refill_min ? c.refill_min : B.refill_min;
    arg.postpone_min = c.postpone_min;
    void* params[] = {&arg};
    return cudaLaunchKernel(select_batch(c), dim3(grid), dim3(normalized_block(c.block)), params, 0, stream);
}

}  // namespace RT
}  // namespace Foundation
