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
    }
    if (i >= wave_n) return;
    const uint64_t npix = (uint64_t)R.width * R.height;
    const uint64_t g = wave_base + i;
    const uint32_t pixel = (uint32_t)(g % npix);
    const uint32_t sample = (uint32_t)(g / npix) + R.sample_offset;
    Pcg32 rng;
    rng.seed(R.seed * 0x9E3779B97F4A7C15ull + pixel, sample);
    const float a = rng.uniform(), b = rng.uniform();
    const uint32_t px = pixel % R.width, py = pixel / R.width;
    const float sx = (2.0f * ((float)px + a) / (float)R.width - 1.0f) * R.tan_half * R.aspect;
    const float sy = (1.0f - 2.0f * ((float)py + b) / (float)R.height) * R.tan_half;
    const float3 d = normalize(ld3(R.fwd) + ld3(R.right) * sx + ld3(R.up) * sy);
    B.ext_rays[0][2 * (size_t)i] = make_float4(R.eye[0], R.eye[1], R.eye[2], 0.0f);
    B.ext_rays[0][2 * (size_t)i + 1] = make_float4(d.x, d.y, d.z, __int_as_float(0x7F800000));
    B.ext_path[0][i] = i;
    B.rng[i] = make_uint4((uint32_t)rng.state, (uint32_t)(rng.state >> 32), sample, pixel);
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
        float4 beta4 = B.beta[slot];
        const uint4 rs = B.rng[slot];
        Pcg32 rng;
        rng.state = (uint64_t)rs.x | ((uint64_t)rs.y << 32);
        rng.inc = ((uint64_t)rs.z << 1) | 1u;
        const uint32_t pixel = rs.w & ~kQueryNextFlag;
        uint32_t flags = rs.w & kQueryNextFlag;
        float3 beta = xyz(beta4);
        const float3 o = xyz(r0), d = xyz(r1);

        bool want_shadow = false, want_sun = false, want_next = false, want_query = false;
        NRC::CachePoint cp;
        float3 sh_o, sh_d, sh_c, sun_c, next_d, surf_o = f3(0.f, 0.f, 0.f);
        float sh_tmax = 0.0f;
        if (hit.x == FND_INVALID_ID) {
            const float3 L = beta * ld3(R.sky);
            if (max3(L) > 0.0f) add_radiance(B.fb, pixel, L);
        } else {
            const float t = __uint_as_float(hit.y);
            const float4 sh = S.tri_shade[hit.x];
            const DevMaterial M = S.materials[min(__float_as_uint(sh.w), S.num_materials - 1u)];
            const uint32_t type = __float_as_uint(M.albedo_type.w);
            const float3 ng = xyz(sh);
            const float dn = dot(d, ng);
            const float3 p = o + d * t;
            if (type == kMatEmissive) {
                const float3 Le = xyz(M.emission_light);
                if (dn < 0.0f && max3(Le) > 0.0f) {
                    float w = 1.0f;
                    const int li = __float_as_int(M.emission_light.w);
                    if (bounce > 0 && li >= 0 && (uint32_t)li < S.num_lights) {
                        const float area = S.lights[li].corner_area.w;
                        const float pdf_l = t * t / (-dn * area * (float)S.num_lights);
                        w = power_heuristic(beta4.w, pdf_l);
                    }
                    add_radiance(B.fb, pixel, beta * Le * w);
                }
            } else if (kMode == 1u && flags) {
                // cache query: the network supplies this vertex's reflected radiance
                const float3 nrm = dn < 0.0f ? ng : -ng;
                cp.p_rough = make_float4(p.x, p.y, p.z, type == kMatLambert ? 1.0f : M.params.x);
                cp.wo_aux = make_float4(-d.x, -d.y, -d.z, __uint_as_float(pixel));
                cp.n_pad = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                cp.albedo = M.albedo_type;
                cp.beta = make_float4(beta.x, beta.y, beta.z, 0.0f);
                want_query = true;
            } else {
                const float3 nrm = dn < 0.0f ? ng : -ng;
                float3 tb, bb;
                onb(nrm, tb, bb);
                const float3 wo = f3(-dot(d, tb), -dot(d, bb), -dot(d, nrm));
                const float3 albedo = xyz(M.albedo_type);
                const float alpha = M.params.x;
                const float3 po = p + nrm * R.eps;
                surf_o = po;
                if (kMode == 1u && (type == kMatLambert || alpha >= C.specular_alpha)) flags = kQueryNextFlag;
                // next-event estimation: one quad light
                const float ul = rng.uniform(), u1 = rng.uniform(), u2 = rng.uniform();
                if (S.num_lights > 0) {
                    const uint32_t k = min((uint32_t)(ul * (float)S.num_lights), S.num_lights - 1u);
                    const DevQuadLight Lq = S.lights[k];
                    const float3 y = xyz(Lq.corner_area) + xyz(Lq.eu) * u1 + xyz(Lq.ev) * u2;
                    float3 wl = y - po;
                    const float d2 = dot(wl, wl);
                    const float dist = sqrtf(d2);
                    wl = wl * (1.0f / dist);
                    const float cos_l = -dot(wl, xyz(Lq.normal));
                    const float cos_x = dot(wl, nrm);
                    if (cos_l > 0.0f && cos_x > 0.0f) {
                        const float3 wi = f3(dot(wl, tb), dot(wl, bb), cos_x);
                        const BsdfEval ev = eval_bsdf(type, albedo, alpha, wo, wi);
                        const float pdf_l = d2 / (cos_l * Lq.corner_area.w * (float)S.num_lights);
                        const float w = power_heuristic(pdf_l, ev.pdf);
                        sh_c = beta * ev.f * xyz(Lq.radiance) * (cos_x * w / pdf_l);
                        if (max3(sh_c) > 0.0f) {
                            want_shadow = true;
                            sh_o = po;
                            sh_d = wl;
                            sh_tmax = dist * (1.0f - 1e-3f);
                        }
                    }
                }
                if (R.has_sun) {
                    const float3 sd = ld3(R.sun_dir);
                    const float cos_x = dot(sd, nrm);
                    if (cos_x > 0.0f) {
                        const float3 wi = f3(dot(sd, tb), dot(sd, bb), cos_x);
                        const BsdfEval ev = eval_bsdf(type, albedo, alpha, wo, wi);
                        sun_c = beta * ev.f * ld3(R.sun_E) * cos_x;
                        want_sun = max3(sun_c) > 0.0f;
                    }
                }
                // continuation
                const float ub1 = rng.uniform(), ub2 = rng.uniform(), urr = rng.uniform();
                if (bounce + 1 < R.max_depth) {
                    const BsdfSample bs = sample_bsdf(type, albedo, alpha, wo, ub1, ub2);
                    if (bs.ok) {
                        beta = beta * bs.weight;
                        bool alive = max3(beta) > 0.0f;
                        if (alive && bounce >= R.rr_start) {
                            const float q = fminf(fmaxf(max3(beta), 0.05f), 1.0f);
                            if (urr >= q)
                                alive = false;
                            else
                                beta = beta * (1.0f / q);
                        }
                        if (alive) {
                            want_next = true;
                            next_d = tb * bs.wi.x + bb * bs.wi.y + nrm * bs.wi.z;
                            beta4 = make_float4(beta.x, beta.y, beta.z, bs.pdf);
                        }
                    }
                }
            }
        }
        // queue appends (all lanes of `active` take part)
        const uint32_t ks = append_slot(B.counts + kCountShadow, want_shadow, active);
        if (want_shadow) {
            B.sh_rays[2 * (size_t)ks] = make_float4(sh_o.x, sh_o.y, sh_o.z, 0.0f);
            B.sh_rays[2 * (size_t)ks + 1] = make_float4(sh_d.x, sh_d.y, sh_d.z, sh_tmax);
            B.sh_pixel[ks] = pixel;
            B.sh_contrib[ks] = make_float4(sh_c.x, sh_c.y, sh_c.z, 0.0f);
        }
        const uint32_t kz = append_slot(B.counts + kCountShadow, want_sun, active);
        if (want_sun) {
            B.sh_rays[2 * (size_t)kz] = make_float4(surf_o.x, surf_o.y, surf_o.z, 0.0f);
            B.sh_rays[2 * (size_t)kz + 1] = make_float4(R.sun_dir[0], R.sun_dir[1], R.sun_dir[2],
                                                        __int_as_float(0x7F800000));
            B.sh_pixel[kz] = pixel;
            B.sh_contrib[kz] = make_float4(sun_c.x, sun_c.y, sun_c.z, 0.0f);
        }
        if (kMode == 1u) {
            const uint32_t kq = append_slot(C.query_count, want_query, active);
            if (want_query && kq < C.query_cap) C.queries[kq] = cp;
        }
        const uint32_t kn = append_slot(B.counts + nxt, want_next, active);
        if (want_next) {
            B.ext_rays[nxt][2 * (size_t)kn] = make_float4(surf_o.x, surf_o.y, surf_o.z, 0.0f);
            B.ext_rays[nxt][2 * (size_t)kn + 1] = make_float4(next_d.x, next_d.y, next_d.z, __int_as_float(0x7F800000));
            B.ext_path[nxt][kn] = slot;
            B.beta[slot] = beta4;
            B.rng[slot] = make_uint4((uint32_t)rng.state, (uint32_t)(rng.state >> 32), rs.z, pixel | flags);
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
