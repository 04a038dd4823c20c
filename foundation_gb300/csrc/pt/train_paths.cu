// train_paths.cu — the radiance cache's training paths as one megakernel.
//
// Each thread follows one training path from the camera through a random
// pixel to its end (at most max_depth interactions) with the same light
// transport as the wavefront stages (integrator.cu): NEE with MIS to the quad
// lights, the sun, the sky, Russian roulette. Every non-emissive vertex
// becomes a training sample whose target is the radiance the path collected
// after that vertex divided by the throughput that reached it (an unbiased
// single-path estimate of the reflected radiance there).
//
// Why a megakernel: the 65,536 training paths of a frame are too few to fill
// the GPU, and in the wavefront each bounce's kernels wait for the slowest
// ray of that bounce; here the kernel lasts as long as the longest path,
// not as long as the sum of every bounce's slowest ray. The samples of a warp
// are written compactly with one atomic per warp.
#include "../../../include/fnd_rt.h"
#include "../rt/traverse.cuh"
#include "integrator.hpp"
#include "pt_math.cuh"

namespace Foundation {
namespace PT {
namespace {

constexpr int kBlock = 128;
constexpr int kMaxDepthTrain = 16;

__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 xyz(float4 v) { return f3(v.x, v.y, v.z); }

__device__ __forceinline__ uint32_t hash32(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

__device__ __forceinline__ RT::RayState make_ray(float3 o, float3 d, float tmax) {
    return RT::setup_ray(make_float4(o.x, o.y, o.z, 0.0f), make_float4(d.x, d.y, d.z, tmax));
}

__global__ void __launch_bounds__(kBlock) training_paths_kernel(const TrainPathsArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < A.n;
    const RenderParams& R = A.R;
    const ShadeScene& S = A.S;
    NRC::CachePoint pts[kMaxDepthTrain];
    float3 before[kMaxDepthTrain];
    int ns = 0;
    float3 total = f3(0.f, 0.f, 0.f);
    const uint32_t depth = min(R.max_depth, (uint32_t)kMaxDepthTrain);
    if (valid) {
        const uint32_t npix = R.width * R.height;
        const uint32_t pixel = hash32(A.seed ^ hash32(i)) % npix;
        Pcg32 rng;
        rng.seed(R.seed * 0x9E3779B97F4A7C15ull + pixel + 0x5851F42D4C957F2Dull * (i + 1ull),
                 0x40000000u + (A.seed & 0x3FFFFFFFu));
        const float a = rng.uniform(), b = rng.uniform();
        const uint32_t px = pixel % R.width, py = pixel / R.width;
        const float sx = (2.0f * ((float)px + a) / (float)R.width - 1.0f) * R.tan_half * R.aspect;
        const float sy = (1.0f - 2.0f * ((float)py + b) / (float)R.height) * R.tan_half;
        float3 o = ld3(R.eye);
        float3 d = normalize(ld3(R.fwd) + ld3(R.right) * sx + ld3(R.up) * sy);
        float3 beta = f3(1.f, 1.f, 1.f);
        float last_pdf = 0.0f;
        for (uint32_t bounce = 0; bounce < depth; ++bounce) {
            const RT::RayState rs = make_ray(o, d, __int_as_float(0x7F800000));
            float t = __int_as_float(0x7F800000);
            uint32_t prim;
            if (!RT::trace_single<false>(A.scene, rs, t, prim, A.status)) {
                total = total + beta * ld3(R.sky);
                break;
            }
            const float4 sh = S.tri_shade[prim];
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
                        const float pdf_l = t * t / (-dn * S.lights[li].corner_area.w * (float)S.num_lights);
                        w = power_heuristic(last_pdf, pdf_l);
                    }
                    total = total + beta * Le * w;
                }
                break;
            }
            const float3 nrm = dn < 0.0f ? ng : -ng;
            float3 tb, bb;
            onb(nrm, tb, bb);
            const float3 wo = f3(-dot(d, tb), -dot(d, bb), -dot(d, nrm));
            const float3 albedo = xyz(M.albedo_type);
            const float alpha = M.params.x;
            const float3 po = p + nrm * R.eps;
            // training sample at this vertex
            NRC::CachePoint& cp = pts[ns];
            cp.p_rough = make_float4(p.x, p.y, p.z, type == kMatLambert ? 1.0f : alpha);
            cp.wo_aux = make_float4(-d.x, -d.y, -d.z, 0.0f);
            cp.n_pad = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
            cp.albedo = M.albedo_type;
            cp.beta = make_float4(beta.x, beta.y, beta.z, 0.0f);
            before[ns] = total;
            ns++;
            // next-event estimation
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
                    const BsdfEval ev = eval_bsdf(type, albedo, alpha, wo, f3(dot(wl, tb), dot(wl, bb), cos_x));
                    const float pdf_l = d2 / (cos_l * Lq.corner_area.w * (float)S.num_lights);
                    const float3 c = beta * ev.f * xyz(Lq.radiance) * (cos_x * power_heuristic(pdf_l, ev.pdf) / pdf_l);
                    if (max3(c) > 0.0f) {
                        float ts = dist * (1.0f - 1e-3f);
                        uint32_t sp;
                        if (!RT::trace_single<true>(A.scene, make_ray(po, wl, ts), ts, sp, A.status)) total = total + c;
                    }
                }
            }
            if (R.has_sun) {
                const float3 sd = ld3(R.sun_dir);
                const float cos_x = dot(sd, nrm);
                if (cos_x > 0.0f) {
                    const BsdfEval ev = eval_bsdf(type, albedo, alpha, wo, f3(dot(sd, tb), dot(sd, bb), cos_x));
                    const float3 c = beta * ev.f * ld3(R.sun_E) * cos_x;
                    if (max3(c) > 0.0f) {
                        float ts = __int_as_float(0x7F800000);
                        uint32_t sp;
                        if (!RT::trace_single<true>(A.scene, make_ray(po, sd, ts), ts, sp, A.status)) total = total + c;
                    }
                }
            }
            const float ub1 = rng.uniform(), ub2 = rng.uniform(), urr = rng.uniform();
            if (bounce + 1 >= depth) break;
            const BsdfSample bs = sample_bsdf(type, albedo, alpha, wo, ub1, ub2);
            if (!bs.ok) break;
            beta = beta * bs.weight;
            if (!(max3(beta) > 0.0f)) break;
            if (bounce >= R.rr_start) {
                const float q = fminf(fmaxf(max3(beta), 0.05f), 1.0f);
                if (urr >= q) break;
                beta = beta * (1.0f / q);
            }
            last_pdf = bs.pdf;
            o = po;
            d = tb * bs.wi.x + bb * bs.wi.y + nrm * bs.wi.z;
        }
    }
    // compact the warp's samples: one atomic per warp
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = (uint32_t)ns;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if ((int)lane >= o) incl += v;
    }
    const uint32_t warp_total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && warp_total) base = atomicAdd(A.sample_count, warp_total);
    base = __shfl_sync(0xFFFFFFFFu, base, 31) + incl - (uint32_t)ns;
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

}  // namespace

cudaError_t LaunchTrainingPaths(const TrainPathsArgs& A, cudaStream_t s) {
    if (A.n == 0) return cudaSuccess;
    training_paths_kernel<<<(A.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(A);
    return cudaGetLastError();
}

}  // namespace PT
}  // namespace Foundation
