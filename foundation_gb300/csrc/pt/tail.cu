// tail.cu — the tail of a wavefront wave as one persistent path megakernel.
//
// Late bounces of a wave hold few paths, and every wavefront stage still
// costs a launch plus the latency of its slowest ray; with the radiance
// cache almost all paths end at their second vertex and the specular
// chains that remain would otherwise pay that per bounce. Here each lane
// takes a path from the queue, runs it bounce by bounce (closest hit,
// shade_vertex, one any-hit ray per light sample) until it ends, then takes
// the next path, so a warp stays full while paths remain.
#include <cuda_runtime.h>

#include "../../../include/fnd_rt.h"
#include "../rt/traverse.cuh"
#include "integrator.hpp"
#include "pt_math.cuh"
#include "shade.cuh"

namespace Foundation {
namespace PT {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ float3 tl_xyz(float4 v) { return f3(v.x, v.y, v.z); }

__device__ __forceinline__ void tl_add(float4* fb, uint32_t pixel, float3 L) {
    float* p = reinterpret_cast<float*>(fb + pixel);
    atomicAdd(p + 0, L.x);
    atomicAdd(p + 1, L.y);
    atomicAdd(p + 2, L.z);
}

template <bool kTwoLevel>
__device__ __forceinline__ bool tl_occluded(const TailArgs& A, float3 o, float3 d, float tmax) {
    float t = tmax;
    uint32_t p;
    return RT::trace_scene<true, kTwoLevel>(A.scene, A.inst, A.num_inst, make_float4(o.x, o.y, o.z, 0.0f),
                                            make_float4(d.x, d.y, d.z, tmax), t, p, A.status);
}

template <uint32_t kMode, bool kTwoLevel>
__global__ void __launch_bounds__(kTailBlock) tail_kernel(const TailArgs A) {
    uint32_t* counts = A.B.counts;
    const uint32_t n = counts[A.q];
    const bool take = n != 0u && n <= A.threshold;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t n_ext = 0, n_sh = 0;
    if (take) {
        const PathBuffers& B = A.B;
        bool have = false, exhausted = false;
        uint32_t pixel = 0, flags = 0, b = 0;
        float3 o = f3(0.f, 0.f, 0.f), d = o, beta = o;
        float last_pdf = 0.0f;
        Pcg32 rng;
        rng.state = 0;
        rng.inc = 1;
        for (;;) {
            // lanes without a path take the next ones (one atomic per warp)
            const uint32_t need = __ballot_sync(kFull, !have);
            if (need && !exhausted) {
                const uint32_t leader = (uint32_t)__ffs(need) - 1u;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(counts + kCountTailFetch, (uint32_t)__popc(need));
                base = __shfl_sync(kFull, base, leader);
                exhausted = base + (uint32_t)__popc(need) >= n;
                if (!have) {
                    const uint32_t j = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
                    if (j < n) {
                        const uint32_t slot = B.ext_path[A.q][j];
                        const float4 r0 = B.ext_rays[A.q][2 * (size_t)j];
                        const float4 r1 = B.ext_rays[A.q][2 * (size_t)j + 1];
                        const float4 b4 = B.beta[slot];
                        const uint4 rs = B.rng[slot];
                        rng = unpack_rng(rs);
                        pixel = rs.w & ~kQueryNextFlag;
                        flags = rs.w & kQueryNextFlag;
                        o = tl_xyz(r0);
                        d = tl_xyz(r1);
                        beta = tl_xyz(b4);
                        last_pdf = b4.w;
                        b = A.bounce;
                        have = true;
                    }
                }
            }
            if (!__any_sync(kFull, have)) break;
            if (!have) continue;
            // one interaction of this lane's path
            VertexIn in;
            float t = __int_as_float(0x7F800000);
            uint32_t prim;
            in.hit = RT::trace_scene<false, kTwoLevel>(A.scene, A.inst, A.num_inst, make_float4(o.x, o.y, o.z, 0.0f),
                                                       make_float4(d.x, d.y, d.z, t), t, prim, A.status);
            n_ext++;
            in.o = o;
            in.d = d;
            in.prim = prim;
            in.t = t;
            in.beta = beta;
            in.last_pdf = last_pdf;
            in.query_here = flags != 0u;
            VertexOut v;
            shade_vertex<kMode>(A.R, A.S, A.C.specular_alpha, b, A.R.max_depth, in, rng, v);
            if (max3(v.add) > 0.0f) tl_add(B.fb, pixel, v.add);
            if (kMode == 1u && v.query) {
                const uint32_t k = atomicAdd(A.C.query_count, 1u);
                if (k < A.C.query_cap) {
                    v.cp.wo_aux.w = __uint_as_float(pixel);
                    A.C.queries[k] = v.cp;
                }
            }
            if (v.shadow) {
                n_sh++;
                if (!tl_occluded<kTwoLevel>(A, v.surf_o, v.sh_d, v.sh_tmax)) tl_add(B.fb, pixel, v.sh_c);
            }
            if (v.sun) {
                n_sh++;
                if (!tl_occluded<kTwoLevel>(A, v.surf_o, f3(A.R.sun_dir[0], A.R.sun_dir[1], A.R.sun_dir[2]),
                                            __int_as_float(0x7F800000)))
                    tl_add(B.fb, pixel, v.sun_c);
            }
            if (v.next) {
                o = v.surf_o;
                d = v.next_d;
                beta = v.beta;
                last_pdf = v.pdf;
                if (v.query_next) flags = kQueryNextFlag;
                b++;
            } else {
                have = false;
            }
        }
    }
    // ray statistics, one atomic per warp
    const uint32_t we = __reduce_add_sync(kFull, n_ext), ws = __reduce_add_sync(kFull, n_sh);
    if (lane == 0 && we) atomicAdd(A.ray_stats + 0, (unsigned long long)we);
    if (lane == 0 && ws) atomicAdd(A.ray_stats + 1, (unsigned long long)ws);
    // the last block to finish empties the queue (every block has read n by then)
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t prev = atomicAdd(counts + kCountTailDone, 1u);
        if (prev == gridDim.x - 1u) {
            if (take) counts[A.q] = 0u;
            counts[kCountTailFetch] = 0u;
            counts[kCountTailDone] = 0u;
            __threadfence();
        }
    }
}

}  // namespace

int TailBlocksPerSm(bool two_level) {
    const void* fns[2] = {two_level ? (const void*)&tail_kernel<0u, true> : (const void*)&tail_kernel<0u, false>,
                          two_level ? (const void*)&tail_kernel<1u, true> : (const void*)&tail_kernel<1u, false>};
    int b = 1 << 30;
    for (const void* f : fns) {
        int k = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, kTailBlock, 0) != cudaSuccess) k = 1;
        b = k < b ? k : b;
    }
    return b > 0 ? b : 1;
}

cudaError_t LaunchTail(const TailArgs& A, int grid, cudaStream_t s) {
    const bool two = A.inst != nullptr;
    if (A.C.mode == 1u) {
        if (two)
            tail_kernel<1u, true><<<grid, kTailBlock, 0, s>>>(A);
        else
            tail_kernel<1u, false><<<grid, kTailBlock, 0, s>>>(A);
    } else {
        if (two)
            tail_kernel<0u, true><<<grid, kTailBlock, 0, s>>>(A);
        else
            tail_kernel<0u, false><<<grid, kTailBlock, 0, s>>>(A);
    }
    return cudaGetLastError();
}

}  // namespace PT
}  // namespace Foundation
