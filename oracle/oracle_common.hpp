// oracle_common.hpp — TEST INFRASTRUCTURE ONLY.
//
// Scalar CPU restatement of the ray-tracing hot path, used by tests/, by
// __graft_entry__.smoke() and by bench.py's cpu_baseline leg as the checker.
// Nothing in the product library links, loads or calls this code.
//
// Parity is UNPINNED against the reference: mos9527/Foundation has no BVH,
// traversal, intersection or path-tracing code (its only pass is a raster
// DrawIndexed of a quad, src/Renderer/Renderer.cpp:312-366), so there is no
// reference output to pin to. This oracle is written from the published
// methods named beside each function and is pinned by hand-derived
// known-answer tests and by brute-force cross-checks (tests/test_oracle_*.py).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

// Ray record as in include/fnd_rt.h (fnd_ray): org, tmin, dir, tmax.
struct Ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
};
static_assert(sizeof(Ray) == 32, "ray layout");

struct Hit {
    uint32_t prim;
    float t;
};
static_assert(sizeof(Hit) == 8, "hit layout");

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Watertight ray/triangle intersection, Woop, Benthin & Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013, without back-face culling and
// without the winding-preserving kx/ky swap (both signs of U,V,W accepted).
//
// The FP32 expression tree below is the contract shared with the device
// kernel: the same operations in the same order, single roundings where an
// fmaf is written, separate roundings everywhere else (build with
// -ffp-contract=off). The per-ray shear constants come from RayPre.
// ---------------------------------------------------------------------------
struct RayPre {
    float o[3];
    float tmin, tmax;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

inline RayPre precompute(const Ray& r) {
    RayPre p;
    for (int i = 0; i < 3; ++i) p.o[i] = r.org[i];
    p.tmin = r.tmin;
    p.tmax = r.tmax;
    const float ax = std::fabs(r.dir[0]), ay = std::fabs(r.dir[1]), az = std::fabs(r.dir[2]);
    // dominant axis; ties resolve to the lower axis index
    p.kz = (ax >= ay) ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    p.kx = p.kz == 2 ? 0 : p.kz + 1;
    p.ky = p.kx == 2 ? 0 : p.kx + 1;
    p.Sx = r.dir[p.kx] / r.dir[p.kz];
    p.Sy = r.dir[p.ky] / r.dir[p.kz];
    p.Sz = 1.0f / r.dir[p.kz];
    return p;
}

// Returns true and t (and U,V,W,det for barycentrics u=U/det, v=V/det) when
// the ray hits the triangle with t in [tmin, tmax].
inline bool intersect(const RayPre& r, const float* v0, const float* v1, const float* v2, float& t_out,
                      float* uvw_det = nullptr) {
    const float A0 = v0[0] - r.o[0], A1 = v0[1] - r.o[1], A2 = v0[2] - r.o[2];
    const float B0 = v1[0] - r.o[0], B1 = v1[1] - r.o[1], B2 = v1[2] - r.o[2];
    const float C0 = v2[0] - r.o[0], C1 = v2[1] - r.o[1], C2 = v2[2] - r.o[2];
    const float A[3] = {A0, A1, A2}, B[3] = {B0, B1, B2}, C[3] = {C0, C1, C2};
    const float Akz = A[r.kz], Bkz = B[r.kz], Ckz = C[r.kz];
    const float Ax = std::fma(-r.Sx, Akz, A[r.kx]);
    const float Ay = std::fma(-r.Sy, Akz, A[r.ky]);
    const float Bx = std::fma(-r.Sx, Bkz, B[r.kx]);
    const float By = std::fma(-r.Sy, Bkz, B[r.ky]);
    const float Cx = std::fma(-r.Sx, Ckz, C[r.kx]);
    const float Cy = std::fma(-r.Sy, Ckz, C[r.ky]);
    // edge functions: plain products so that a shared edge evaluates to the
    // exact negation in the neighbouring triangle (watertightness)
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // exact products in double, one rounding of the difference
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    const float T = std::fma(W, Cz, std::fma(V, Bz, U * Az));
    const float t = T / det;
    if (!(t >= r.tmin && t <= r.tmax)) return false;
    t_out = t;
    if (uvw_det) {
        uvw_det[0] = U;
        uvw_det[1] = V;
        uvw_det[2] = W;
        uvw_det[3] = det;
    }
    return true;
}

// (t, prim) lexicographic order: the closest-hit tie rule.
inline bool closer(float t, uint32_t prim, float best_t, uint32_t best_prim) {
    return t < best_t || (t == best_t && prim < best_prim);
}

// ---------------------------------------------------------------------------
// PCG32 (PCG-XSH-RR 64/32), M. E. O'Neill, "PCG: A Family of Simple Fast
// Space-Efficient Statistically Good Algorithms for Random Number
// Generation", 2014: LCG multiplier 6364136223846793005, odd increment,
// xorshift-high then random rotation output; seeding as in the paper's
// pcg32_srandom_r (state 0, step, add seed, step).
// ---------------------------------------------------------------------------
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    Pcg32() = default;
    Pcg32(uint64_t seed, uint64_t seq) { seed_with(seed, seq); }
    void seed_with(uint64_t seed, uint64_t seq) {
        state = 0u;
        inc = (seq << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // uniform float in [0, 1): top 24 bits
    float next_float() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
    double next_double() {
        // 53 random bits from two outputs
        const uint64_t hi = next() >> 5, lo = next() >> 6;
        return ((double)hi * 67108864.0 + (double)lo) * (1.0 / 9007199254740992.0);
    }
};

}  // namespace oracle
