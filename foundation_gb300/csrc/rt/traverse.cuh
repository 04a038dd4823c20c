// traverse.cuh — device-side scene view, ray set-up, watertight triangle test
// and compressed 8-wide node test shared by every traversal kernel
// (closest hit, any hit, the batched multi-scene launch and the integrator's
// extend / shadow stages).
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../../include/fnd_rt.h"
#include "../bvh/wide_bvh.hpp"
#include "device_scene.hpp"

namespace Foundation {
namespace RT {

// Per-ray state for the node test (origin, sanitised inverse direction,
// direction-sign octant) and for the watertight triangle test (shear
// constants of Woop, Benthin & Wald 2013, dominant axis kz).
struct RayState {
    float ox, oy, oz;
    float ix, iy, iz;
    float nSx, nSy, Sz;  // -Sx, -Sy, Sz
    float tmin, tmax;
    uint32_t oct;
    int kz;
};

__device__ __forceinline__ float sanitize_dir(float d) {
    // keep the sign (also of -0.0); 2^-64 keeps the inverse finite
    return fabsf(d) < 5.421010862427522e-20f ? copysignf(5.421010862427522e-20f, d) : d;
}

__device__ __forceinline__ RayState setup_ray(float4 r0, float4 r1) {
    RayState s;
    s.ox = r0.x;
    s.oy = r0.y;
    s.oz = r0.z;
    s.tmin = r0.w;
    s.tmax = r1.w;
    s.ix = __fdiv_rn(1.0f, sanitize_dir(r1.x));
    s.iy = __fdiv_rn(1.0f, sanitize_dir(r1.y));
    s.iz = __fdiv_rn(1.0f, sanitize_dir(r1.z));
    s.oct = (signbit(r1.x) ? 1u : 0u) | (signbit(r1.y) ? 2u : 0u) | (signbit(r1.z) ? 4u : 0u);
    const float ax = fabsf(r1.x), ay = fabsf(r1.y), az = fabsf(r1.z);
    const int kz = (ax >= ay) ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    s.kz = kz;
    const float dkz = kz == 0 ? r1.x : (kz == 1 ? r1.y : r1.z);
    const float dkx = kz == 0 ? r1.y : (kz == 1 ? r1.z : r1.x);
    const float dky = kz == 0 ? r1.z : (kz == 1 ? r1.x : r1.y);
    s.nSx = -__fdiv_rn(dkx, dkz);
    s.nSy = -__fdiv_rn(dky, dkz);
    s.Sz = __fdiv_rn(1.0f, dkz);
    return s;
}

// Cyclic permutation (kx, ky, kz) = (kz+1, kz+2, kz) mod 3.
__device__ __forceinline__ void permute(const RayState& r, float a0, float a1, float a2, float& x, float& y, float& z) {
    x = r.kz == 0 ? a1 : (r.kz == 1 ? a2 : a0);
    y = r.kz == 0 ? a2 : (r.kz == 1 ? a0 : a1);
    z = r.kz == 0 ? a0 : (r.kz == 1 ? a1 : a2);
}

__device__ __forceinline__ float edge_fallback(float ax, float by, float ay, float bx) {
    return __double2float_rn(__dsub_rn(__dmul_rn((double)ax, (double)by), __dmul_rn((double)ay, (double)bx)));
}

// Watertight test, non-culling, same FP32 expression tree as the CPU
// restatement: every operation is an explicit round-to-nearest intrinsic so
// the compiler cannot contract or reorder it. Returns t (NaN-free) on a hit
// with t in [tmin, tmax]; out_u/out_v/out_det for barycentrics on request.
template <bool kBary = false>
__device__ __forceinline__ bool intersect_tri(const RayState& r, float4 v0, float4 v1, float4 v2, float tmax,
                                              float& t_out, float* bary = nullptr) {
    float Ax, Ay, Az, Bx, By, Bz, Cx, Cy, Cz;
    permute(r, __fsub_rn(v0.x, r.ox), __fsub_rn(v0.y, r.oy), __fsub_rn(v0.z, r.oz), Ax, Ay, Az);
    permute(r, __fsub_rn(v1.x, r.ox), __fsub_rn(v1.y, r.oy), __fsub_rn(v1.z, r.oz), Bx, By, Bz);
    permute(r, __fsub_rn(v2.x, r.ox), __fsub_rn(v2.y, r.oy), __fsub_rn(v2.z, r.oz), Cx, Cy, Cz);
    const float ax = __fmaf_rn(r.nSx, Az, Ax), ay = __fmaf_rn(r.nSy, Az, Ay);
    const float bx = __fmaf_rn(r.nSx, Bz, Bx), by = __fmaf_rn(r.nSy, Bz, By);
    const float cx = __fmaf_rn(r.nSx, Cz, Cx), cy = __fmaf_rn(r.nSy, Cz, Cy);
    float U = __fsub_rn(__fmul_rn(cx, by), __fmul_rn(cy, bx));
    float V = __fsub_rn(__fmul_rn(ax, cy), __fmul_rn(ay, cx));
    float W = __fsub_rn(__fmul_rn(bx, ay), __fmul_rn(by, ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = edge_fallback(cx, by, cy, bx);
        V = edge_fallback(ax, cy, ay, cx);
        W = edge_fallback(bx, ay, by, ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float az = __fmul_rn(r.Sz, Az), bz = __fmul_rn(r.Sz, Bz), cz = __fmul_rn(r.Sz, Cz);
    const float T = __fmaf_rn(W, cz, __fmaf_rn(V, bz, __fmul_rn(U, az)));
    const float t = __fdiv_rn(T, det);
    if (!(t >= r.tmin && t <= tmax)) return false;
    t_out = t;
    if (kBary) {
        bary[0] = U;
        bary[1] = V;
        bary[2] = W;
        bary[3] = det;
    }
    return true;
}

// Packed FP32 pairs for the child-box test: two slots' plane FMAs in one
// fma.rm / fma.rp .f32x2 (sm_100 family). Each lane rounds exactly like the
// scalar __fmaf_rd / __fmaf_ru (tests/test_minmax_gpu.py checks it on the
// GPU); the host build evaluates the scalar forms.
struct F2 {
#if defined(__CUDA_ARCH__)
    unsigned long long v;
#else
    float x, y;
#endif
};
__device__ __forceinline__ F2 pack_f2(float a, float b) {
    F2 r;
#if defined(__CUDA_ARCH__)
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
#else
    r.x = a;
    r.y = b;
#endif
    return r;
}
// out = a * b + c per lane, rounded down (kUp false) or up (kUp true)
template <bool kUp>
__device__ __forceinline__ void fma_dir_f2(F2 a, F2 b, F2 c, float out[2]) {
#if defined(__CUDA_ARCH__)
    unsigned long long d;
    if (kUp)
        asm("fma.rp.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a.v), "l"(b.v), "l"(c.v));
    else
        asm("fma.rm.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a.v), "l"(b.v), "l"(c.v));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(out[0]), "=f"(out[1]) : "l"(d));
#else
    out[0] = kUp ? __fmaf_ru(a.x, b.x, c.x) : __fmaf_rd(a.x, b.x, c.x);
    out[1] = kUp ? __fmaf_ru(a.y, b.y, c.y) : __fmaf_rd(a.y, b.y, c.y);
#endif
}

// Two quantised planes as floats 1024 + q, exactly: one PRMT builds the
// half2 (0x64 | q) pair (a half with exponent 2^10 and q in its low mantissa
// bits), and the two halves widen to float off the integer pipe. sel picks
// the byte pair: 0x4140 for bytes 0 and 1, 0x4342 for bytes 2 and 3.
__device__ __forceinline__ void plane_pair(uint32_t word, uint32_t sel, float& a, float& b) {
#if defined(__CUDA_ARCH__)
    const uint32_t h2 = __byte_perm(word, 0x64u, sel);
    __half2 h;
    memcpy(&h, &h2, sizeof(h));
    a = __low2float(h);
    b = __high2float(h);
#else
    const uint32_t k = (sel & 0xFu) * 8u;
    a = 1024.0f + (float)((word >> k) & 0xFFu);
    b = 1024.0f + (float)((word >> (k + 8u)) & 0xFFu);
#endif
}

// max / min of three (one instruction on the sm_100 family; NaN operands
// are dropped like nested fmaxf / fminf, which tests/test_minmax_gpu.py
// checks on the GPU).
__device__ __forceinline__ float max3f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}

// Bit 7 of each byte of w gathered into bits 0..3: the product places bits
// 7, 15, 23 and 31 at 28..31 and its other partial products at distinct
// lower positions, so no carry reaches the result.
__device__ __forceinline__ uint32_t meta_leaf_bits(uint32_t w) { return ((w & 0x80808080u) * 0x00204081u) >> 28; }

// Bit s of the 8-bit mask m moved to bit s ^ oct.
__device__ __forceinline__ uint32_t xor_permute8(uint32_t m, uint32_t oct) {
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u) m = ((m & 0x0Fu) << 4) | (m >> 4);
    return m;
}

// Tests the 8 child boxes of one compressed node against the ray.
// Returns the hit mask of internal children in traversal order (bit i is
// slot i ^ oct) in bits 0..7 with the node's imask in bits 8..15, and the
// triangle mask (bit k: triangle tri_base + k) of the hit leaf children.
struct NodeHits {
    uint32_t child_base;
    uint32_t tri_base;
    uint32_t group;  // imask << 8 | ordered internal hits
    uint32_t tris;
};

// perm (optional): a table of 8 x 256 bytes, perm[oct * 256 + m] =
// xor_permute8(m, oct), in place of the bit swaps, followed by 256 words:
// the triangle mask of a leaf slot by its meta byte.
__device__ __forceinline__ NodeHits intersect_node(const RayState& r, const uint4* __restrict__ nodes, uint32_t idx,
                                                   float tfar, const uint8_t* perm = nullptr) {
    const uint4* n = nodes + 5 * (size_t)idx;
    const uint4 w0 = __ldg(n + 0);
    const uint4 w1 = __ldg(n + 1);
    const uint4 w2 = __ldg(n + 2);
    const uint4 w3 = __ldg(n + 3);
    const uint4 w4 = __ldg(n + 4);
    const float sx = __uint_as_float((w0.w & 0xFFu) << 23) * r.ix;
    const float sy = __uint_as_float(((w0.w >> 8) & 0xFFu) << 23) * r.iy;
    const float sz = __uint_as_float(((w0.w >> 16) & 0xFFu) << 23) * r.iz;
    const float bx = (__uint_as_float(w0.x) - r.ox) * r.ix;
    const float by = (__uint_as_float(w0.y) - r.oy) * r.iy;
    const float bz = (__uint_as_float(w0.z) - r.oz) * r.iz;
    const uint32_t imask = w0.w >> 24;
    // near / far plane words per axis, chosen by the direction signs
    const bool fx = r.oct & 1u, fy = r.oct & 2u, fz = r.oct & 4u;
    const uint32_t nx0 = fx ? w3.z : w2.x, nx1 = fx ? w3.w : w2.y;
    const uint32_t gx0 = fx ? w2.x : w3.z, gx1 = fx ? w2.y : w3.w;
    const uint32_t ny0 = fy ? w4.x : w2.z, ny1 = fy ? w4.y : w2.w;
    const uint32_t gy0 = fy ? w2.z : w4.x, gy1 = fy ? w2.w : w4.y;
    const uint32_t nz0 = fz ? w4.z : w3.x, nz1 = fz ? w4.w : w3.y;
    const uint32_t gz0 = fz ? w3.x : w4.z, gz1 = fz ? w3.y : w4.w;
    // A plane's t is q * s + b with q the quantised byte. The byte is read
    // as the float 1024 + q (plane_pair) and the 1024 * s is folded into the
    // offset, near planes rounded down and far planes up:
    //   near: rd((1024+q) s + rd(b - 1024 s)) <= rd(q s + b) <= rn(q s + b)
    //   far:  ru((1024+q) s + ru(b - 1024 s)) >= ru(q s + b) >= rn(q s + b)
    // so every child box is at least as wide as under round-to-nearest
    // fma(q, s, b), the culling stays conservative and the hits exact.
    const float bnx = __fmaf_rd(-1024.0f, sx, bx), bfx = __fmaf_ru(-1024.0f, sx, bx);
    const float bny = __fmaf_rd(-1024.0f, sy, by), bfy = __fmaf_ru(-1024.0f, sy, by);
    const float bnz = __fmaf_rd(-1024.0f, sz, bz), bfz = __fmaf_ru(-1024.0f, sz, bz);
    // the boxes alone: bit s of hitm for slot s (empty slots included; the
    // slot kinds below mask them out); two slots per byte pair, their plane
    // FMAs as packed pairs
    const F2 sx2 = pack_f2(sx, sx), sy2 = pack_f2(sy, sy), sz2 = pack_f2(sz, sz);
    const F2 bnx2 = pack_f2(bnx, bnx), bny2 = pack_f2(bny, bny), bnz2 = pack_f2(bnz, bnz);
    const F2 bfx2 = pack_f2(bfx, bfx), bfy2 = pack_f2(bfy, bfy), bfz2 = pack_f2(bfz, bfz);
    uint32_t hitm = 0;
#pragma unroll
    for (int pr = 0; pr < 4; ++pr) {
        const uint32_t sel = (pr & 1) ? 0x4342u : 0x4140u;
        float q0[6], q1[6];
        plane_pair(pr < 2 ? nx0 : nx1, sel, q0[0], q1[0]);
        plane_pair(pr < 2 ? ny0 : ny1, sel, q0[1], q1[1]);
        plane_pair(pr < 2 ? nz0 : nz1, sel, q0[2], q1[2]);
        plane_pair(pr < 2 ? gx0 : gx1, sel, q0[3], q1[3]);
        plane_pair(pr < 2 ? gy0 : gy1, sel, q0[4], q1[4]);
        plane_pair(pr < 2 ? gz0 : gz1, sel, q0[5], q1[5]);
        float tnx[2], tny[2], tnz[2], tfx[2], tfy[2], tfz[2];
        fma_dir_f2<false>(pack_f2(q0[0], q1[0]), sx2, bnx2, tnx);
        fma_dir_f2<false>(pack_f2(q0[1], q1[1]), sy2, bny2, tny);
        fma_dir_f2<false>(pack_f2(q0[2], q1[2]), sz2, bnz2, tnz);
        fma_dir_f2<true>(pack_f2(q0[3], q1[3]), sx2, bfx2, tfx);
        fma_dir_f2<true>(pack_f2(q0[4], q1[4]), sy2, bfy2, tfy);
        fma_dir_f2<true>(pack_f2(q0[5], q1[5]), sz2, bfz2, tfz);
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float tn = max3f(tnx[e], tny[e], fmaxf(tnz[e], r.tmin));
            const float tf = min3f(tfx[e], tfy[e], fminf(tfz[e], tfar));
            hitm |= tn <= tf ? 1u << (2 * pr + e) : 0u;
        }
    }
    // leaf slots: the 0x80 flag of their meta byte
    const uint32_t leaves = meta_leaf_bits(w1.z) | meta_leaf_bits(w1.w) << 4;
    uint32_t lh = hitm & leaves, tris = 0;
    while (lh) {  // about one hit leaf per three nodes on incoherent rays
        const uint32_t s = (uint32_t)__ffs(lh) - 1u;
        lh &= lh - 1u;
        const uint32_t meta = __byte_perm(s < 4u ? w1.z : w1.w, 0u, 0x4440u | (s & 3u));
        tris |= perm ? reinterpret_cast<const uint32_t*>(perm + 2048)[meta]
                     : ((2u << ((meta >> 5) & 3u)) - 1u) << (meta & 31u);
    }
    NodeHits out;
    out.child_base = w1.x;
    out.tri_base = w1.y;
    out.group = (imask << 8) | (perm ? (uint32_t)perm[(r.oct << 8) | (hitm & imask)] : xor_permute8(hitm & imask, r.oct));
    out.tris = tris;
    return out;
}

}  // namespace RT
}  // namespace Foundation

namespace Foundation {
namespace RT {

// Single-ray traversal with a thread-local stack and no warp refill, for
// latency-bound work where each thread follows its own path (the radiance
// cache's training paths). Same node / triangle tests and tie rule as the
// persistent kernels. Returns true on a hit (best_t / best_p updated; the
// caller initialises best_t to the ray's tmax).
template <bool kAny>
__device__ __forceinline__ bool trace_single(const DeviceScene& sc, const RayState& r, float& best_t,
                                             uint32_t& best_p, uint32_t* status) {
    best_p = FND_INVALID_ID;
    if (sc.num_nodes == 0) return false;
    uint2 stack[kMaxStack];
    int sp = 0;
    uint32_t ng_base = 0, ng_group = (1u << 8) | (1u << r.oct), tg_base = 0, tg_mask = 0;
    for (;;) {
        if (ng_group & 0xFFu) {
            const uint32_t b = (uint32_t)__ffs(ng_group & 0xFFu) - 1u;
            ng_group &= ~(1u << b);
            const uint32_t slot = b ^ r.oct;
            const uint32_t child = ng_base + (uint32_t)__popc((ng_group >> 8) & ((1u << slot) - 1u));
            if (ng_group & 0xFFu) {
                if (sp >= kMaxStack) {
                    atomicOr(status, kStatusStackOverflow);
                    break;
                }
                stack[sp++] = make_uint2(ng_base, ng_group);
            }
            if (child >= sc.num_nodes) {
                atomicOr(status, kStatusBadIndex);
                break;
            }
            const NodeHits h = intersect_node(r, sc.nodes, child, best_t);
            ng_base = h.child_base;
            ng_group = h.group;
            tg_base = h.tri_base;
            tg_mask = h.tris;
            if (tg_mask && (uint64_t)tg_base + (uint64_t)(32 - __clz(tg_mask)) > sc.num_tris) {
                atomicOr(status, kStatusBadIndex);
                break;
            }
        }
        while (tg_mask) {
            const uint32_t k = (uint32_t)__ffs(tg_mask) - 1u;
            tg_mask &= tg_mask - 1u;
            const uint32_t ti = tg_base + k;
            const float4 v0 = __ldg(sc.v0 + ti);
            float t;
            if (intersect_tri(r, v0, __ldg(sc.v1 + ti), __ldg(sc.v2 + ti), best_t, t)) {
                const uint32_t pid = __float_as_uint(v0.w);
                if (kAny) {
                    best_t = t;
                    best_p = pid;
                    return true;
                }
                if (best_p == FND_INVALID_ID || t < best_t || (t == best_t && pid < best_p)) {
                    best_t = t;
                    best_p = pid;
                }
            }
        }
        if (ng_group & 0xFFu) continue;
        if (sp == 0) break;
        const uint2 e = stack[--sp];
        ng_base = e.x;
        ng_group = e.y;
    }
    return best_p != FND_INVALID_ID;
}

// World ray -> object space of an instance: o' = inv * (o, 1), d' = inv * (d, 0),
// each component summed left to right with round-to-nearest operations (the
// oracle evaluates the same expression); t is the same parameter in both
// spaces, so tmin / tmax carry over.
__device__ __forceinline__ void instance_ray(const float* inv, float4 r0, float4 r1, float4& o0, float4& o1) {
    float o[3], d[3];
    for (int i = 0; i < 3; ++i) {
        const float* m = inv + 4 * i;
        o[i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], r0.x), __fmul_rn(m[1], r0.y)), __fmul_rn(m[2], r0.z)), m[3]);
        d[i] = __fadd_rn(__fadd_rn(__fmul_rn(m[0], r1.x), __fmul_rn(m[1], r1.y)), __fmul_rn(m[2], r1.z));
    }
    o0 = make_float4(o[0], o[1], o[2], r0.w);
    o1 = make_float4(d[0], d[1], d[2], r1.w);
}

// Two-level traversal: the top-level tree's leaves are instances (the plane
// record's index word holds the instance id); each instance's bottom level
// is traversed in object space with trace_single. Ties across instances
// break by the global id (prim_offset + bottom-level id), as within a scene.
template <bool kAny>
__device__ __forceinline__ bool trace_two_level(const DeviceScene& tlas, const InstanceRec* __restrict__ inst,
                                                uint32_t num_inst, float4 r0, float4 r1, float& best_t,
                                                uint32_t& best_p, uint32_t* status) {
    best_p = FND_INVALID_ID;
    if (tlas.num_nodes == 0) return false;
    const RayState r = setup_ray(r0, r1);
    uint2 stack[kMaxStack];
    int sp = 0;
    uint32_t ng_base = 0, ng_group = (1u << 8) | (1u << r.oct), tg_base = 0, tg_mask = 0;
    for (;;) {
        if (ng_group & 0xFFu) {
            const uint32_t b = (uint32_t)__ffs(ng_group & 0xFFu) - 1u;
            ng_group &= ~(1u << b);
            const uint32_t slot = b ^ r.oct;
            const uint32_t child = ng_base + (uint32_t)__popc((ng_group >> 8) & ((1u << slot) - 1u));
            if (ng_group & 0xFFu) {
                if (sp >= kMaxStack) {
                    atomicOr(status, kStatusStackOverflow);
                    break;
                }
                stack[sp++] = make_uint2(ng_base, ng_group);
            }
            if (child >= tlas.num_nodes) {
                atomicOr(status, kStatusBadIndex);
                break;
            }
            const NodeHits h = intersect_node(r, tlas.nodes, child, best_t);
            ng_base = h.child_base;
            ng_group = h.group;
            tg_base = h.tri_base;
            tg_mask = h.tris;
            if (tg_mask && (uint64_t)tg_base + (uint64_t)(32 - __clz(tg_mask)) > tlas.num_tris) {
                atomicOr(status, kStatusBadIndex);
                break;
            }
        }
        while (tg_mask) {
            const uint32_t k = (uint32_t)__ffs(tg_mask) - 1u;
            tg_mask &= tg_mask - 1u;
            const uint32_t id = __float_as_uint(__ldg(tlas.v0 + tg_base + k).w);
            if (id >= num_inst) {
                atomicOr(status, kStatusBadIndex);
                continue;
            }
            const InstanceRec& I = inst[id];
            RayState ro = r;  // an identity instance keeps the world ray
            if (!(__ldg(&I.flags) & kInstanceIdentity)) {
                float inv[12];
                for (int q = 0; q < 12; ++q) inv[q] = __ldg(I.inv + q);
                float4 o0, o1;
                instance_ray(inv, r0, r1, o0, o1);
                ro = setup_ray(o0, o1);
            }
            const DeviceScene blas = I.blas;
            float t = best_t;
            uint32_t p;
            if (trace_single<kAny>(blas, ro, t, p, status)) {
                const uint32_t gid = __ldg(&I.prim_offset) + p;
                if (kAny) {
                    best_t = t;
                    best_p = gid;
                    return true;
                }
                if (best_p == FND_INVALID_ID || t < best_t || (t == best_t && gid < best_p)) {
                    best_t = t;
                    best_p = gid;
                }
            }
        }
        if (ng_group & 0xFFu) continue;
        if (sp == 0) break;
        const uint2 e = stack[--sp];
        ng_base = e.x;
        ng_group = e.y;
    }
    return best_p != FND_INVALID_ID;
}

// One ray through a one- or two-level scene (per-thread traversal, for the
// path-tracing megakernels). r0 / r1: the ray in the fnd_ray layout; best_t
// starts at the ray's tmax.
template <bool kAny, bool kTwoLevel>
__device__ __forceinline__ bool trace_scene(const DeviceScene& sc, const InstanceRec* inst, uint32_t num_inst,
                                            float4 r0, float4 r1, float& best_t, uint32_t& best_p, uint32_t* status) {
    if constexpr (kTwoLevel) return trace_two_level<kAny>(sc, inst, num_inst, r0, r1, best_t, best_p, status);
    return trace_single<kAny>(sc, setup_ray(r0, r1), best_t, best_p, status);
}

}  // namespace RT
}  // namespace Foundation
