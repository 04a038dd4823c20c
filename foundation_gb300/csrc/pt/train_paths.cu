// train_paths.cu — the radiance cache's training paths as one megakernel.
//
// Each thread follows one training path from the camera through a random
// pixel to its end (at most max_depth interactions) with the vertex logic of
// the wavefront stages (shade.cuh): NEE with MIS to the quad lights, the sun,
// the sky, Russian roulette. Every non-emissive vertex
// becomes a training sample whose target is the radiance the path collected
// after that vertex divided by the throughput that reached it (an unbiased
// single-path estimate of the reflected radiance there).
//
// Why a megakernel: the 65,536 training paths of a frame are too few to fill
// the GPU, and in the wavefront each bounce's kernels wait for the slowest
// ray of that bounce. The kernel is persistent (one grid of resident
// blocks) and a lane that finishes its path takes the next one, so warps
// stay full until the paths run out instead of waiting for their longest
// path. Each path's samples go out with one atomic for their slots.
#include "../../../include/fnd_rt.h"
#include "../rt/traverse.cuh"
#include "integrator.hpp"
#include "pt_math.cuh"
#include "shade.cuh"

namespace Foundation {
namespace PT {
namespace {

constexpr int kBlock = 128;
constexpr int kMaxDepthTrain = 16;
constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

__device__ __forceinline__ uint32_t hash32(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

template <bool kAny, bool kTwoLevel>
__device__ __forceinline__ bool trace(const TrainPathsArgs& A, float3 o, float3 d, float& t, uint32_t& p) {
    return RT::trace_scene<kAny, kTwoLevel>(A.scene, A.inst, A.num_inst, make_float4(o.x, o.y, o.z, 0.0f),
                                            make_float4(d.x, d.y, d.z, t), t, p, A.status);
}

// A finished path's samples: slots from one atomic, targets from the
// radiance the path collected after each sample's vertex.
__device__ __forceinline__ void write_samples(const TrainPathsArgs& A, const NRC::CachePoint* pts,
                                              const float3* before, int ns, float3 total) {
    if (ns == 0) return;
    const uint32_t base = atomicAdd(A.sample_count, (uint32_t)ns);
    for (int k = 0; k < ns; ++k) {
        const uint32_t slot = base + (uint32_t)k;
        if (slot >= A.sample_cap) break;
        NRC::TrainSample s;
        s.pt = pts[k];
        s.before = make_float4(before[k].x, before[k].y, before[k].z, 0.0f);
        A.samples[slot] = s;
        const float bt[3] = {s.pt.beta.x, s.pt.beta.y, s.pt.beta.z};
        const float df[3] = {total.x - before[k].x, total.y - before[k].y, total.z - before[k].z};
        float tg[3];
        bool ok = true;
        for (int c = 0; c < 3; ++c) {
            ok = ok && bt[c] > 1e-8f;
            tg[c] = bt[c] > 1e-8f ? fmaxf(df[c], 0.0f) / bt[c] : 0.0f;
        }
        A.targets[slot] = make_float4(tg[0], tg[1], tg[2], ok ? 1.0f : 0.0f);
    }
}

// Persistent: every lane holds one path and, each iteration, runs one
// interaction of it (closest hit, shade_vertex, its shadow rays); a lane
// whose path ended takes the next path index at the top of the iteration
// (one atomic per warp), so the warp stays full until the paths run out and
// its lanes stay at the same point of the loop.
template <bool kTwoLevel>
__global__ void __launch_bounds__(kBlock) training_paths_kernel(const TrainPathsArgs A) {
    const RenderParams& R = A.R;
    const ShadeScene& S = A.S;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t depth = min(R.max_depth, (uint32_t)kMaxDepthTrain);
    const uint32_t npix = R.width * R.height;
    NRC::CachePoint pts[kMaxDepthTrain];
    float3 before[kMaxDepthTrain];
    int ns = 0;
    float3 total = f3(0.f, 0.f, 0.f), o = total, d = total, beta = total;
    float last_pdf = 0.0f;
    uint32_t bounce = 0;
    Pcg32 rng;
    rng.state = 0;
    rng.inc = 1;
    bool have = false, exhausted = false;
    for (;;) {
        const uint32_t need = __ballot_sync(kFull, !have);
        if (need && !exhausted) {
            const uint32_t leader = (uint32_t)__ffs(need) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(A.fetch, (uint32_t)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            exhausted = base + (uint32_t)__popc(need) >= A.n;
            if (!have) {
                const uint32_t i = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
                if (i < A.n) {
                    const uint32_t pixel = hash32(A.seed ^ hash32(i)) % npix;
                    rng = training_path_rng(R.seed, pixel, i, A.seed);
                    const float a = rng.uniform(), b = rng.uniform();
                    const uint32_t px = pixel % R.width, py = pixel / R.width;
                    const float sx = (2.0f * ((float)px + a) / (float)R.width - 1.0f) * R.tan_half * R.aspect;
                    const float sy = (1.0f - 2.0f * ((float)py + b) / (float)R.height) * R.tan_half;
                    o = ld3(R.eye);
                    d = normalize(ld3(R.fwd) + ld3(R.right) * sx + ld3(R.up) * sy);
                    beta = f3(1.f, 1.f, 1.f);
                    total = f3(0.f, 0.f, 0.f);
                    last_pdf = 0.0f;
                    bounce = 0;
                    ns = 0;
                    have = depth > 0;
                }
            }
        }
        if (!__any_sync(kFull, have)) break;
        if (!have) continue;
        VertexIn in;
        float t = __int_as_float(0x7F800000);
        uint32_t prim;
        in.hit = trace<false, kTwoLevel>(A, o, d, t, prim);
        in.o = o;
        in.d = d;
        in.prim = prim;
        in.t = t;
        in.beta = beta;
        in.last_pdf = last_pdf;
        in.query_here = false;
        VertexOut v;
        shade_vertex<2u>(R, S, 0.0f, bounce, depth, in, rng, v);
        total = total + v.add;
        if (v.sample) {
            pts[ns] = v.cp;
            before[ns] = total;
            ns++;
        }
        if (v.shadow) {
            float ts = v.sh_tmax;
            uint32_t sp;
            if (!trace<true, kTwoLevel>(A, v.surf_o, v.sh_d, ts, sp)) total = total + v.sh_c;
        }
        if (v.sun) {
            float ts = __int_as_float(0x7F800000);
            uint32_t sp;
            if (!trace<true, kTwoLevel>(A, v.surf_o, ld3(R.sun_dir), ts, sp)) total = total + v.sun_c;
        }
        bounce++;
        if (v.next && bounce < depth) {
            last_pdf = v.pdf;
            beta = v.beta;
            o = v.surf_o;
            d = v.next_d;
        } else {
            write_samples(A, pts, before, ns, total);
            have = false;
        }
    }
}

}  // namespace

int TrainingPathsBlocksPerSm(bool two_level) {
    const void* f = two_level ? (const void*)&training_paths_kernel<true> : (const void*)&training_paths_kernel<false>;
    int k = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, kBlock, 0) != cudaSuccess) k = 1;
    return k > 0 ? k : 1;
}

cudaError_t LaunchTrainingPaths(const TrainPathsArgs& A, int grid, cudaStream_t s) {
    if (A.n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(A.fetch, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const uint32_t blocks_needed = (A.n + kBlock - 1) / kBlock;
    grid = grid < (int)blocks_needed ? grid : (int)blocks_needed;
    if (A.inst)
        training_paths_kernel<true><<<grid > 0 ? grid : 1, kBlock, 0, s>>>(A);
    else
        training_paths_kernel<false><<<grid > 0 ? grid : 1, kBlock, 0, s>>>(A);
    return cudaGetLastError();
}

}  // namespace PT
}  // namespace Foundation
