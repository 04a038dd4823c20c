// integrator.cu — wavefront path-tracing stages (sm_103a): generate, shade,
// shadow resolve, finalize. The extend and shadow traversals are the
// persistent trace kernels of rt/traverse.cu reading their ray counts from
// the device queues.
//
// Light transport (same definitions as the FP64 oracle, oracle/pt_oracle.cpp):
//  * pinhole camera (glm lookAt convention), one jittered sample per path;
//  * surfaces two-sided (geometric normal flipped towards the incoming ray),
//    emitters one-sided (they emit on the side their winding normal faces)
//    and black;
//  * next-event estimation at every non-emissive hit: one point on one quad
//    light (uniform light choice, uniform point on the quad) weighted by the
//    power heuristic against the BSDF pdf, plus one shadow ray towards the
//    directional sun when there is one; BSDF-sampled hits on emitters are
//    weighted by the power heuristic against the light pdf; escaping rays
//    collect the constant sky radiance;
//  * Russian roulette from bounce `rr_start` with survival probability
//    clamp(max(throughput), 0.05, 1); at most `max_depth` surface interactions.
#include "integrator.hpp"

#include "../../../include/fnd_rt.h"
#include "pt_math.cuh"
#include "shade.cuh"

namespace Foundation {
namespace PT {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr int kBlock = 256;

__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }

__device__ __forceinline__ void add_radiance(float4* fb, uint32_t pixel, float3 L) {
    float* p = reinterpret_cast<float*>(fb + pixel);
    atomicAdd(p + 0, L.x);
    atomicAdd(p + 1, L.y);
    atomicAdd(p + 2, L.z);
}

// Warp-aggregated append: every lane of `active` calls it together; lanes
// with pred get consecutive slots.
__device__ __forceinline__ uint32_t append_slot(uint32_t* counter, bool pred, uint32_t active) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t m = __ballot_sync(active, pred);
    if (m == 0u) return 0u;
    const uint32_t leader = (uint32_t)__ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(active, base, leader);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(kBlock) generate_kernel(const PathBuffers B, const RenderParams R,
                                                          uint64_t wave_base, uint32_t wave_n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        B.counts[kCountExt0] = wave_n;
        B.counts[kCountExt1] = 0;
        B.counts[kCountShadow] = 0;
        B.counts[kCountTailDone] = 0;
        B.counts[kCountTailFetch] = 0;
    }
    if (i >= wave_n) return;
    const uint64_t npix = (uint64_t)R.width * R.height;
    const uint64_t g = wave_base + i;
    const uint32_t pixel = (uint32_t)(g % npix);
    const uint32_t sample = (uint32_t)(g / npix) + R.sample_offset;
    Pcg32 rng = camera_path_rng(R.seed, pixel, sample);
    const float a = rng.uniform(), b = rng.uniform();
    const uint32_t px = pixel % R.width, py = pixel / R.width;
    const float sx = (2.0f * ((float)px + a) / (float)R.width - 1.0f) * R.tan_half * R.aspect;
    const float sy = (1.0f - 2.0f * ((float)py + b) / (float)R.height) * R.tan_half;
    const float3 d = normalize(ld3(R.fwd) + ld3(R.right) * sx + ld3(R.up) * sy);
    B.ext_rays[0][2 * (size_t)i] = make_float4(R.eye[0], R.eye[1], R.eye[2], 0.0f);
    B.ext_rays[0][2 * (size_t)i + 1] = make_float4(d.x, d.y, d.z, __int_as_float(0x7F800000));
    B.ext_path[0][i] = i;
    B.rng[i] = pack_rng(rng, sample, pixel);
    B.beta[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
}

template <uint32_t kMode>
__global__ void __launch_bounds__(kBlock) shade_kernel(const PathBuffers B, const RenderParams R, const ShadeScene S,
                                                       const CacheIO C, int cur, uint32_t bounce) {
    const uint32_t n = B.counts[cur];
    const int nxt = cur ^ 1;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t j = base + threadIdx.x;
        const bool valid = j < n;
        const uint32_t active = __ballot_sync(kFull, valid);
        if (!valid) continue;
        const uint32_t slot = B.ext_path[cur][j];
        const uint2 hit = B.hits[j];
        const float4 r0 = B.ext_rays[cur][2 * (size_t)j];
        const float4 r1 = B.ext_rays[cur][2 * (size_t)j + 1];
        const float4 beta4 = B.beta[slot];
        const uint4 rs = B.rng[slot];
        Pcg32 rng = unpack_rng(rs);
        const uint32_t pixel = rs.w & ~kQueryNextFlag;
        VertexIn in;
        in.o = xyz(r0);
        in.d = xyz(r1);
        in.hit = hit.x != FND_INVALID_ID;
        in.prim = hit.x;
        in.t = __uint_as_float(hit.y);
        in.beta = xyz(beta4);
        in.last_pdf = beta4.w;
        in.query_here = (rs.w & kQueryNextFlag) != 0u;
        VertexOut v;
        shade_vertex<kMode>(R, S, C.specular_alpha, bounce, R.max_depth, in, rng, v);
        if (max3(v.add) > 0.0f) add_radiance(B.fb, pixel, v.add);
        // queue appends (all lanes of `active` take part)
        const uint32_t ks = append_slot(B.counts + kCountShadow, v.shadow, active);
        if (v.shadow) {
            B.sh_rays[2 * (size_t)ks] = make_float4(v.surf_o.x, v.surf_o.y, v.surf_o.z, 0.0f);
            B.sh_rays[2 * (size_t)ks + 1] = make_float4(v.sh_d.x, v.sh_d.y, v.sh_d.z, v.sh_tmax);
            B.sh_pixel[ks] = pixel;
            B.sh_contrib[ks] = make_float4(v.sh_c.x, v.sh_c.y, v.sh_c.z, 0.0f);
        }
        const uint32_t kz = append_slot(B.counts + kCountShadow, v.sun, active);
        if (v.sun) {
            B.sh_rays[2 * (size_t)kz] = make_float4(v.surf_o.x, v.surf_o.y, v.surf_o.z, 0.0f);
            B.sh_rays[2 * (size_t)kz + 1] = make_float4(R.sun_dir[0], R.sun_dir[1], R.sun_dir[2],
                                                        __int_as_float(0x7F800000));
            B.sh_pixel[kz] = pixel;
            B.sh_contrib[kz] = make_float4(v.sun_c.x, v.sun_c.y, v.sun_c.z, 0.0f);
        }
        if (kMode == 1u) {
            const uint32_t kq = append_slot(C.query_count, v.query, active);
            if (v.query && kq < C.query_cap) {
                v.cp.wo_aux.w = __uint_as_float(pixel);
                C.queries[kq] = v.cp;
            }
        }
        const uint32_t kn = append_slot(B.counts + nxt, v.next, active);
        if (v.next) {
            const uint32_t flags = (rs.w & kQueryNextFlag) | (v.query_next ? kQueryNextFlag : 0u);
            B.ext_rays[nxt][2 * (size_t)kn] = make_float4(v.surf_o.x, v.surf_o.y, v.surf_o.z, 0.0f);
            B.ext_rays[nxt][2 * (size_t)kn + 1] =
                make_float4(v.next_d.x, v.next_d.y, v.next_d.z, __int_as_float(0x7F800000));
            B.ext_path[nxt][kn] = slot;
            B.beta[slot] = make_float4(v.beta.x, v.beta.y, v.beta.z, v.pdf);
            B.rng[slot] = pack_rng(rng, rs.z, pixel | flags);
        }
    }
}

__global__ void __launch_bounds__(kBlock) resolve_kernel(const PathBuffers B) {
    const uint32_t n = B.counts[kCountShadow];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        if (B.sh_occluded[k]) continue;
        const float4 c = B.sh_contrib[k];
        add_radiance(B.fb, B.sh_pixel[k], f3(c.x, c.y, c.z));
    }
}

__global__ void __launch_bounds__(kBlock) finalize_kernel(const float4* fb, float* rgb, uint32_t npix, float scale) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float4 v = fb[i];
    rgb[3 * (size_t)i + 0] = v.x * scale;
    rgb[3 * (size_t)i + 1] = v.y * scale;
    rgb[3 * (size_t)i + 2] = v.z * scale;
}

}  // namespace

cudaError_t LaunchGenerate(const PathBuffers& B, const RenderParams& R, uint64_t wave_base, uint32_t wave_n,
                           cudaStream_t s) {
    const uint32_t blocks = (wave_n + kBlock - 1) / kBlock;
    generate_kernel<<<blocks ? blocks : 1, kBlock, 0, s>>>(B, R, wave_base, wave_n);
    return cudaGetLastError();
}

cudaError_t LaunchShade(const PathBuffers& B, const RenderParams& R, const ShadeScene& S, const CacheIO& C, int cur,
                        uint32_t bounce, int grid, cudaStream_t s) {
    if (C.mode == 1u)
        shade_kernel<1u><<<grid, kBlock, 0, s>>>(B, R, S, C, cur, bounce);
    else
        shade_kernel<0u><<<grid, kBlock, 0, s>>>(B, R, S, C, cur, bounce);
    return cudaGetLastError();
}

cudaError_t LaunchResolve(const PathBuffers& B, int grid, cudaStream_t s) {
    resolve_kernel<<<grid, kBlock, 0, s>>>(B);
    return cudaGetLastError();
}

cudaError_t LaunchFinalize(const PathBuffers& B, float* rgb, uint32_t npix, float scale, cudaStream_t s) {
    finalize_kernel<<<(npix + kBlock - 1) / kBlock, kBlock, 0, s>>>(B.fb, rgb, npix, scale);
    return cudaGetLastError();
}

}  // namespace PT
}  // namespace Foundation
