// shade.cuh — what happens at one path vertex, shared by the wavefront shade
// stage (integrator.cu), the tail kernel that finishes small queues and the
// training-path megakernel (train_paths.cu). The caller traces; this decides.
//
// Light transport (the FP64 oracle, oracle/pt_oracle.cpp, states the same):
//  * misses collect the constant sky;
//  * emitters are one-sided and black; a BSDF-sampled hit on an emitter is
//    weighted by the power heuristic against the light-sampling pdf (the
//    camera ray, bounce 0, takes the emission as is);
//  * at a non-emissive vertex: one quad light sample (uniform light choice,
//    uniform point) weighted against the BSDF pdf, one sun ray if there is a
//    sun, then a BSDF sample continues the path (at most `max_depth`
//    interactions), with Russian roulette from bounce rr_start (survival
//    clamp(max(throughput), 0.05, 1));
//  * with the radiance cache (kMode 1) the vertex after the first
//    non-specular one becomes a cache query and ends the path; training
//    paths (kMode 2) record every non-emissive vertex.
// Random numbers per non-emissive, non-query vertex: light choice, two for
// the light point, two for the BSDF, one for roulette, in that order.
#pragma once

#include "../nrc/nrc.hpp"
#include "integrator.hpp"
#include "pt_math.cuh"

namespace Foundation {
namespace PT {

struct VertexIn {
    float3 o, d;       // ray of the segment that reached the vertex
    bool hit;
    uint32_t prim;
    float t;
    float3 beta;       // throughput reaching the vertex
    float last_pdf;    // solid-angle pdf of the BSDF sample that made the ray (0 for camera rays)
    bool query_here;   // cache mode: this vertex is a query
};

struct VertexOut {
    float3 add;        // radiance to add now (sky / emission), throughput applied
    bool query;        // cache query at this vertex (cp)
    bool sample;       // training sample at this vertex (cp)
    NRC::CachePoint cp;
    bool shadow;       // NEE ray to a quad light
    float3 sh_d, sh_c;
    float sh_tmax;
    bool sun;          // NEE ray to the sun
    float3 sun_c;
    float3 surf_o;     // offset origin of shadow and continuation rays
    bool next;         // continuation
    float3 next_d, beta;
    float pdf;
    bool query_next;   // cache mode: the next vertex becomes a query
};

__device__ __forceinline__ float3 sh_ld3(const float* p) { return f3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 sh_xyz(float4 v) { return f3(v.x, v.y, v.z); }

template <uint32_t kMode>
__device__ __forceinline__ void shade_vertex(const RenderParams& R, const ShadeScene& S, float specular_alpha,
                                             uint32_t bounce, uint32_t max_depth, const VertexIn& in, Pcg32& rng,
                                             VertexOut& out) {
    out.add = f3(0.f, 0.f, 0.f);
    out.query = out.sample = out.shadow = out.sun = out.next = out.query_next = false;
    out.surf_o = in.o;
    if (!in.hit) {
        out.add = in.beta * sh_ld3(R.sky);
        return;
    }
    const float4 sh = S.tri_shade[in.prim];
    const DevMaterial M = S.materials[min(__float_as_uint(sh.w), S.num_materials - 1u)];
    const uint32_t type = __float_as_uint(M.albedo_type.w);
    const float3 ng = sh_xyz(sh);
    const float3 d = in.d;
    const float dn = dot(d, ng);
    const float3 p = in.o + d * in.t;
    if (type == kMatEmissive) {
        const float3 Le = sh_xyz(M.emission_light);
        if (dn < 0.0f && max3(Le) > 0.0f) {
            float w = 1.0f;
            const int li = __float_as_int(M.emission_light.w);
            if (bounce > 0 && li >= 0 && (uint32_t)li < S.num_lights) {
                const float pdf_l = in.t * in.t / (-dn * S.lights[li].corner_area.w * (float)S.num_lights);
                w = power_heuristic(in.last_pdf, pdf_l);
            }
            out.add = in.beta * Le * w;
        }
        return;
    }
    const float3 nrm = dn < 0.0f ? ng : -ng;
    const float alpha = M.params.x;
    if (kMode != 0u) {
        out.cp.p_rough = make_float4(p.x, p.y, p.z, type == kMatLambert ? 1.0f : alpha);
        out.cp.wo_aux = make_float4(-d.x, -d.y, -d.z, 0.0f);
        out.cp.n_pad = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
        out.cp.albedo = M.albedo_type;
        out.cp.beta = make_float4(in.beta.x, in.beta.y, in.beta.z, 0.0f);
    }
    if (kMode == 1u && in.query_here) {
        out.query = true;
        return;
    }
    if (kMode == 2u) out.sample = true;
    float3 tb, bb;
    onb(nrm, tb, bb);
    const float3 wo = f3(-dot(d, tb), -dot(d, bb), -dot(d, nrm));
    const float3 albedo = sh_xyz(M.albedo_type);
    const float3 po = p + nrm * R.eps;
    out.surf_o = po;
    if (kMode == 1u) out.query_next = type == kMatLambert || alpha >= specular_alpha;
    // next-event estimation: one quad light
    const float ul = rng.uniform(), u1 = rng.uniform(), u2 = rng.uniform();
    if (S.num_lights > 0) {
        const uint32_t k = min((uint32_t)(ul * (float)S.num_lights), S.num_lights - 1u);
        const DevQuadLight Lq = S.lights[k];
        const float3 y = sh_xyz(Lq.corner_area) + sh_xyz(Lq.eu) * u1 + sh_xyz(Lq.ev) * u2;
        float3 wl = y - po;
        const float d2 = dot(wl, wl);
        const float dist = sqrtf(d2);
        wl = wl * (1.0f / dist);
        const float cos_l = -dot(wl, sh_xyz(Lq.normal));
        const float cos_x = dot(wl, nrm);
        if (cos_l > 0.0f && cos_x > 0.0f) {
            const BsdfEval ev = eval_bsdf(type, albedo, alpha, wo, f3(dot(wl, tb), dot(wl, bb), cos_x));
            const float pdf_l = d2 / (cos_l * Lq.corner_area.w * (float)S.num_lights);
            out.sh_c = in.beta * ev.f * sh_xyz(Lq.radiance) * (cos_x * power_heuristic(pdf_l, ev.pdf) / pdf_l);
            if (max3(out.sh_c) > 0.0f) {
                out.shadow = true;
                out.sh_d = wl;
                out.sh_tmax = dist * (1.0f - 1e-3f);
            }
        }
    }
    if (R.has_sun) {
        const float3 sd = sh_ld3(R.sun_dir);
        const float cos_x = dot(sd, nrm);
        if (cos_x > 0.0f) {
            const BsdfEval ev = eval_bsdf(type, albedo, alpha, wo, f3(dot(sd, tb), dot(sd, bb), cos_x));
            out.sun_c = in.beta * ev.f * sh_ld3(R.sun_E) * cos_x;
            out.sun = max3(out.sun_c) > 0.0f;
        }
    }
    // continuation
    const float ub1 = rng.uniform(), ub2 = rng.uniform(), urr = rng.uniform();
    if (bounce + 1 < max_depth) {
        const BsdfSample bs = sample_bsdf(type, albedo, alpha, wo, ub1, ub2);
        if (bs.ok) {
            float3 beta = in.beta * bs.weight;
            bool alive = max3(beta) > 0.0f;
            if (alive && bounce >= R.rr_start) {
                const float q = fminf(fmaxf(max3(beta), 0.05f), 1.0f);
                if (urr >= q)
                    alive = false;
                else
                    beta = beta * (1.0f / q);
            }
            if (alive) {
                out.next = true;
                out.next_d = tb * bs.wi.x + bb * bs.wi.y + nrm * bs.wi.z;
                out.beta = beta;
                out.pdf = bs.pdf;
            }
        }
    }
}

}  // namespace PT
}  // namespace Foundation
