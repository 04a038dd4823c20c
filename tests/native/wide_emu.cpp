// wide_emu.cpp — TEST HARNESS: host emulation of the per-ray traversal logic
// of foundation_gb300/csrc/rt/traverse.cu, used by the CPU test suite to
// validate the product's BVH builder, wide-node collapse / quantisation and
// node + triangle tests without a GPU. It compiles the product's own
// traverse.cuh with g++ by supplying host definitions of the CUDA intrinsics
// it uses (round-to-nearest IEEE ops, byte_perm, bit casts), so the numbers
// are the ones the device computes. Not part of the product library.
#include <cuda_runtime.h>

#include <bit>
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
// directed-rounding fma: the host FPU in the requested mode (the harness is
// built with -frounding-math so the compiler keeps the mode switches)
static inline float fma_mode(float a, float b, float c, int mode) {
    const int old = std::fegetround();
    std::fesetround(mode);
    volatile float r = std::fma(a, b, c);
    std::fesetround(old);
    return r;
}
static inline float __fmaf_rd(float a, float b, float c) { return fma_mode(a, b, c, FE_DOWNWARD); }
static inline float __fmaf_ru(float a, float b, float c) { return fma_mode(a, b, c, FE_UPWARD); }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline float __double2float_rn(double d) { return (float)d; }
static inline float __uint_as_float(uint32_t u) { return std::bit_cast<float>(u); }
static inline uint32_t __float_as_uint(float f) { return std::bit_cast<uint32_t>(f); }
static inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s) {
    const uint64_t v = ((uint64_t)y << 32) | x;
    uint32_t r = 0;
    for (int i = 0; i < 4; ++i) {
        const uint32_t sel = (s >> (4 * i)) & 7u;
        r |= (uint32_t)((v >> (8 * sel)) & 0xFFu) << (8 * i);
    }
    return r;
}
template <typename T>
static inline T __ldg(const T* p) {
    return *p;
}
static inline int __ffs(uint32_t x) { return x ? __builtin_ctz(x) + 1 : 0; }
static inline int __popc(uint32_t x) { return __builtin_popcount(x); }
static inline int __clz(uint32_t x) { return x ? __builtin_clz(x) : 32; }
static inline uint32_t atomicOr(uint32_t* p, uint32_t v) {
    const uint32_t o = *p;
    *p |= v;
    return o;
}
using std::copysignf;

using std::signbit;

#include "../../include/fnd_rt.h"
#include "../../foundation_gb300/csrc/bvh/bvh_build.hpp"
#include "../../foundation_gb300/csrc/bvh/collapse.hpp"
#include "../../foundation_gb300/csrc/bvh/instances.hpp"
#include "../../foundation_gb300/csrc/rt/traverse.cuh"

using namespace Foundation::RT;

struct emu_bvh {
    BinaryBvh bin;
    WideBvh wide;
    DeviceScene view{};
};

extern "C" {

emu_bvh* emu_build2(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads,
                    int spatial);

emu_bvh* emu_build(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads) {
    return emu_build2(verts, nv, idx, nt, threads, 0);
}

emu_bvh* emu_build3(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads,
                    int spatial, float trav_cost);

emu_bvh* emu_build2(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads,
                    int spatial) {
    return emu_build3(verts, nv, idx, nt, threads, spatial, 1.0f);
}

emu_bvh* emu_build4(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads,
                    int spatial, float trav_cost, float margin_scale);

emu_bvh* emu_build3(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads,
                    int spatial, float trav_cost) {
    return emu_build4(verts, nv, idx, nt, threads, spatial, trav_cost, 1.0f);
}

emu_bvh* emu_build4(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t threads,
                    int spatial, float trav_cost, float margin_scale) {
    auto* e = new emu_bvh();
    std::vector<float> tri(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)idx[3 * (size_t)t + k] + c];
    BuildParams p;
    p.threads = threads;
    p.trav_cost = trav_cost;
    if (spatial)
        BuildBinarySbvh(tri.data(), nt, p, e->bin);
    else
        BuildBinaryBvh(tri.data(), nt, p, e->bin);
    CollapseToWide(e->bin, tri.data(), nt, e->wide, margin_scale);
    e->view.nodes = reinterpret_cast<const uint4*>(e->wide.nodes.data());
    e->view.v0 = reinterpret_cast<const float4*>(e->wide.v0.data());
    e->view.v1 = reinterpret_cast<const float4*>(e->wide.v1.data());
    e->view.v2 = reinterpret_cast<const float4*>(e->wide.v2.data());
    e->view.num_nodes = (uint32_t)e->wide.nodes.size();
    e->view.num_tris = (uint32_t)e->bin.prims.size();
    (void)nv;
    return e;
}

// Spatial-split build with a given split budget (extra references per triangle).
emu_bvh* emu_build_sbvh(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, float budget) {
    auto* e = new emu_bvh();
    std::vector<float> tri(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)idx[3 * (size_t)t + k] + c];
    BuildParams p;
    p.max_refs_factor = budget;
    BuildBinarySbvh(tri.data(), nt, p, e->bin);
    CollapseToWide(e->bin, tri.data(), nt, e->wide, 1.0f);
    e->view.nodes = reinterpret_cast<const uint4*>(e->wide.nodes.data());
    e->view.v0 = reinterpret_cast<const float4*>(e->wide.v0.data());
    e->view.v1 = reinterpret_cast<const float4*>(e->wide.v1.data());
    e->view.v2 = reinterpret_cast<const float4*>(e->wide.v2.data());
    e->view.num_nodes = (uint32_t)e->wide.nodes.size();
    e->view.num_tris = (uint32_t)e->bin.prims.size();
    (void)nv;
    return e;
}

// Binned SAH (spatial: with spatial splits at split budget 8) collapsed by the
// SAH-optimal rule with triangle cost c_tri.
emu_bvh* emu_build_sah_collapse(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, int spatial,
                                double c_tri) {
    auto* e = new emu_bvh();
    std::vector<float> tri(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)idx[3 * (size_t)t + k] + c];
    BuildParams p;
    p.max_refs_factor = 8.0;
    if (spatial)
        BuildBinarySbvh(tri.data(), nt, p, e->bin);
    else
        BuildBinaryBvh(tri.data(), nt, p, e->bin);
    CollapseOptions o;
    o.sah = true;
    o.c_tri = c_tri;
    CollapseToWide(e->bin, tri.data(), nt, e->wide, 1.0f, o);
    e->view.nodes = reinterpret_cast<const uint4*>(e->wide.nodes.data());
    e->view.v0 = reinterpret_cast<const float4*>(e->wide.v0.data());
    e->view.v1 = reinterpret_cast<const float4*>(e->wide.v1.data());
    e->view.v2 = reinterpret_cast<const float4*>(e->wide.v2.data());
    e->view.num_nodes = (uint32_t)e->wide.nodes.size();
    e->view.num_tris = (uint32_t)e->bin.prims.size();
    (void)nv;
    return e;
}

// Binned SAH collapsed to nodes of at most `width` children (greedy, or the
// SAH-optimal rule with sah != 0).
emu_bvh* emu_build_width(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, int sah,
                         uint32_t width) {
    auto* e = new emu_bvh();
    std::vector<float> tri(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)idx[3 * (size_t)t + k] + c];
    BuildParams p;
    BuildBinaryBvh(tri.data(), nt, p, e->bin);
    CollapseOptions o;
    o.sah = sah != 0;
    o.width = width;
    CollapseToWide(e->bin, tri.data(), nt, e->wide, 1.0f, o);
    e->view.nodes = reinterpret_cast<const uint4*>(e->wide.nodes.data());
    e->view.v0 = reinterpret_cast<const float4*>(e->wide.v0.data());
    e->view.v1 = reinterpret_cast<const float4*>(e->wide.v1.data());
    e->view.v2 = reinterpret_cast<const float4*>(e->wide.v2.data());
    e->view.num_nodes = (uint32_t)e->wide.nodes.size();
    e->view.num_tris = (uint32_t)e->bin.prims.size();
    (void)nv;
    return e;
}

// The wide tree's node records (80 bytes each), copied to out (nodes x 80
// bytes); returns the node count.
uint32_t emu_nodes(const emu_bvh* e, void* out) {
    if (out) std::memcpy(out, e->wide.nodes.data(), e->wide.nodes.size() * sizeof(WideNode));
    return (uint32_t)e->wide.nodes.size();
}

// FNV-1a hash of the binary tree the binned-SAH builder makes on `threads`
// threads, in depth-first order: every node's box and triangle count and
// every leaf's triangle indices (the node numbering is left out: it follows
// the order the threads take the nodes in).
uint64_t emu_binary_hash(const float* verts, const uint32_t* idx, uint32_t nt, uint32_t threads) {
    std::vector<float> tri(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)idx[3 * (size_t)t + k] + c];
    BuildParams p;
    p.threads = threads;
    BinaryBvh b;
    BuildBinaryBvh(tri.data(), nt, p, b);
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* q, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(q);
        for (size_t i = 0; i < n; ++i) {
            h ^= c[i];
            h *= 1099511628211ull;
        }
    };
    std::vector<uint32_t> stack{0u};
    while (!stack.empty()) {
        const BinaryNode& nd = b.nodes[stack.back()];
        stack.pop_back();
        mix(nd.lo, sizeof(nd.lo));
        mix(nd.hi, sizeof(nd.hi));
        mix(&nd.count, sizeof(nd.count));
        if (nd.count) {
            mix(&b.prims[nd.a], sizeof(uint32_t) * nd.count);
        } else {
            stack.push_back(nd.a + 1);
            stack.push_back(nd.a);
        }
    }
    return h;
}

// FNV-1a hash of the bytes of the wide tree (nodes, then the three plane
// arrays) that e's binary tree collapses to on `threads` threads, by the
// SAH-optimal rule (sah != 0) or the greedy one.
uint64_t emu_collapse_hash(const emu_bvh* e, const float* verts, const uint32_t* idx, uint32_t nt, int sah,
                           uint32_t threads) {
    std::vector<float> tri(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)idx[3 * (size_t)t + k] + c];
    CollapseOptions o;
    o.sah = sah != 0;
    o.threads = threads;
    WideBvh w;
    CollapseToWide(e->bin, tri.data(), nt, w, 1.0f, o);
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    mix(w.nodes.data(), w.nodes.size() * sizeof(WideNode));
    mix(w.v0.data(), 4 * w.v0.size());
    mix(w.v1.data(), 4 * w.v1.size());
    mix(w.v2.data(), 4 * w.v2.size());
    return h;
}

// Leaf references (triangles, plus the duplicates spatial splits added).
uint64_t emu_num_refs(const emu_bvh* e) { return e->bin.prims.size(); }

void emu_free(emu_bvh* e) { delete e; }

// out: binary nodes, leaves, binary depth, wide nodes, wide depth, wide leaves
void emu_stats(const emu_bvh* e, uint64_t* out, double* sah, float* margin) {
    out[0] = e->bin.nodes.size();
    out[1] = e->bin.leaves;
    out[2] = e->bin.depth;
    out[3] = e->wide.nodes.size();
    out[4] = e->wide.depth;
    out[5] = e->wide.leaves;
    *sah = e->bin.sah_cost;
    *margin = e->wide.margin;
}

// Per-ray restatement of trace_kernel's lane logic (same group / stack
// semantics, same node and triangle tests). max_sp receives the deepest stack.
void emu_trace(const emu_bvh* e, const float* rays, uint64_t n, uint32_t* hits, int any, uint64_t* stats) {
    uint64_t nodes = 0, tris = 0, max_sp = 0, occupied = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float* rp = rays + 8 * i;
        const float4 r0{rp[0], rp[1], rp[2], rp[3]}, r1{rp[4], rp[5], rp[6], rp[7]};
        const RayState r = setup_ray(r0, r1);
        float best_t = r.tmax;
        uint32_t best_p = FND_INVALID_ID;
        uint32_t ng_base = 0, ng_group = (1u << 8) | (1u << r.oct), tg_base = 0, tg_mask = 0;
        std::vector<uint2> stack;
        for (;;) {
            if (ng_group & 0xFFu) {
                const uint32_t b = (uint32_t)__builtin_ctz(ng_group & 0xFFu);
                ng_group &= ~(1u << b);
                const uint32_t slot = b ^ r.oct;
                const uint32_t child = ng_base + (uint32_t)__builtin_popcount((ng_group >> 8) & ((1u << slot) - 1u));
                if (ng_group & 0xFFu) stack.push_back(uint2{ng_base, ng_group});
                max_sp = std::max<uint64_t>(max_sp, stack.size());
                const NodeHits h = intersect_node(r, e->view.nodes, child, best_t);
                nodes++;
                for (int k = 0; k < 8; ++k) occupied += e->wide.nodes[child].meta[k] != 0;
                ng_base = h.child_base;
                ng_group = h.group;
                tg_base = h.tri_base;
                tg_mask = h.tris;
            }
            while (tg_mask) {
                const uint32_t k = (uint32_t)__builtin_ctz(tg_mask);
                tg_mask &= tg_mask - 1u;
                const uint32_t ti = tg_base + k;
                tris++;
                float t;
                if (intersect_tri(r, e->view.v0[ti], e->view.v1[ti], e->view.v2[ti], best_t, t)) {
                    const uint32_t pid = __float_as_uint(e->view.v0[ti].w);
                    if (any) {
                        best_t = t;
                        best_p = pid;
                        tg_mask = 0;
                        ng_group = 0;
                        stack.clear();
                    } else if (best_p == FND_INVALID_ID || t < best_t || (t == best_t && pid < best_p)) {
                        best_t = t;
                        best_p = pid;
                    }
                }
            }
            if (ng_group & 0xFFu) continue;
            if (stack.empty()) break;
            const uint2 g = stack.back();
            stack.pop_back();
            ng_base = g.x;
            ng_group = g.y;
        }
        hits[2 * i] = best_p;
        hits[2 * i + 1] = best_p == FND_INVALID_ID ? 0x7F800000u : __float_as_uint(best_t);
    }
    stats[0] = nodes;
    stats[1] = tris;
    stats[2] = max_sp;
    stats[3] = occupied;  // occupied child slots over the visited nodes
}

// Two-level scenes: the product's host-side top level (bvh/instances.cpp)
// over emulated bottom levels, traced with RT::trace_two_level (the
// per-thread two-level traversal of the path-tracing megakernels).
struct emu_two {
    InstanceTop top;
    std::vector<InstanceRec> recs;
    DeviceScene tlas{};
};

emu_two* emu_instances(const emu_bvh* const* blas, const float* transforms, const uint32_t* offsets, uint32_t n) {
    auto* t = new emu_two();
    std::vector<InstanceInput> in(n);
    for (uint32_t i = 0; i < n; ++i) {
        std::memcpy(in[i].transform, transforms + 12 * (size_t)i, 48);
        std::memcpy(in[i].lo, blas[i]->wide.lo, 12);
        std::memcpy(in[i].hi, blas[i]->wide.hi, 12);
    }
    BuildInstanceTop(in.data(), n, t->top);
    t->recs.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        t->recs[i].blas = blas[i]->view;
        std::memcpy(t->recs[i].inv, &t->top.inv[12 * (size_t)i], 48);
        t->recs[i].prim_offset = offsets[i];
        static const float kId[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};  // the library's identity rule
        t->recs[i].flags = std::memcmp(t->recs[i].inv, kId, sizeof(kId)) == 0 ? kInstanceIdentity : 0u;
    }
    t->tlas.nodes = reinterpret_cast<const uint4*>(t->top.wide.nodes.data());
    t->tlas.v0 = reinterpret_cast<const float4*>(t->top.wide.v0.data());
    t->tlas.v1 = reinterpret_cast<const float4*>(t->top.wide.v1.data());
    t->tlas.v2 = reinterpret_cast<const float4*>(t->top.wide.v2.data());
    t->tlas.num_nodes = (uint32_t)t->top.wide.nodes.size();
    t->tlas.num_tris = n;
    return t;
}

void emu_instances_trace(const emu_two* t, const float* rays, uint64_t n, uint32_t* hits, int any) {
    uint32_t status = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float* rp = rays + 8 * i;
        const float4 r0{rp[0], rp[1], rp[2], rp[3]}, r1{rp[4], rp[5], rp[6], rp[7]};
        float best_t = r1.w;
        uint32_t p = FND_INVALID_ID;
        const bool h = any ? trace_two_level<true>(t->tlas, t->recs.data(), (uint32_t)t->recs.size(), r0, r1, best_t, p,
                                                   &status)
                           : trace_two_level<false>(t->tlas, t->recs.data(), (uint32_t)t->recs.size(), r0, r1, best_t,
                                                    p, &status);
        hits[2 * i] = h ? p : FND_INVALID_ID;
        hits[2 * i + 1] = h ? __float_as_uint(best_t) : 0x7F800000u;
    }
}

double emu_instance_reach(const emu_two* t, uint32_t i) { return InstanceReach(&t->top.inv[12 * (size_t)i], t->top.lo, t->top.hi); }

void emu_instances_free(emu_two* t) { delete t; }

// The same rays through RT::trace_single (the per-thread traversal of the
// cache's training paths).
void emu_trace_single(const emu_bvh* e, const float* rays, uint64_t n, uint32_t* hits, int any) {
    uint32_t status = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float* rp = rays + 8 * i;
        const RayState r = setup_ray(float4{rp[0], rp[1], rp[2], rp[3]}, float4{rp[4], rp[5], rp[6], rp[7]});
        float t = r.tmax;
        uint32_t p = FND_INVALID_ID;
        const bool h = any ? trace_single<true>(e->view, r, t, p, &status) : trace_single<false>(e->view, r, t, p, &status);
        hits[2 * i] = h ? p : FND_INVALID_ID;
        hits[2 * i + 1] = h ? __float_as_uint(t) : 0x7F800000u;
    }
}

// RT::trace_single over caller-made node and triangle arrays (planes: v0[nt],
// v1[nt], v2[nt] as float4), closest hit; *status_out receives the status
// word the traversal latched (it starts at 0).
void emu_trace_single_raw(const void* nodes, uint32_t num_nodes, const float* planes, uint32_t num_tris,
                          const float* rays, uint64_t n, uint32_t* hits, uint32_t* status_out) {
    DeviceScene sc{};
    sc.nodes = static_cast<const uint4*>(nodes);
    const float4* pl = reinterpret_cast<const float4*>(planes);
    sc.v0 = pl;
    sc.v1 = pl + num_tris;
    sc.v2 = pl + 2 * (size_t)num_tris;
    sc.num_nodes = num_nodes;
    sc.num_tris = num_tris;
    uint32_t status = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float* rp = rays + 8 * i;
        const RayState r = setup_ray(float4{rp[0], rp[1], rp[2], rp[3]}, float4{rp[4], rp[5], rp[6], rp[7]});
        float t = r.tmax;
        uint32_t p = FND_INVALID_ID;
        const bool h = trace_single<false>(sc, r, t, p, &status);
        hits[2 * i] = h ? p : FND_INVALID_ID;
        hits[2 * i + 1] = h ? __float_as_uint(t) : 0x7F800000u;
    }
    *status_out = status;
}

// The fnd_status every entry point reports for a latched status word.
int emu_status_code(uint32_t bits) { return StatusCode(bits); }

}  // extern "C"
