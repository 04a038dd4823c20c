// capi_instances.cpp — two-level scenes (see fnd_rt_instances_upload in
// include/fnd_rt.h): per instance the FP64 inverse transform (rounded to
// FP32) and the world box of its bottom level's bounds, a top-level tree
// over those boxes (the binned-SAH builder fed one degenerate triangle per
// instance, spanning the box), the instance records on the device.
#include <algorithm>
#include <array>
#include <cmath>
#include <memory>
#include <vector>

#include "../bvh/bvh_build.hpp"
#include "../bvh/collapse.hpp"
#include "../bvh/gpu_build.hpp"
#include "context.hpp"

using namespace Foundation;
using Foundation::CApi::Guard;

namespace {

// Row-major 3x4 inverse: adjugate over the determinant, translation
// -inv(A) b, all in FP64 with the operation order of the oracle.
bool Inverse(const float* m, double inv[12]) {
    const double a00 = m[0], a01 = m[1], a02 = m[2], a10 = m[4], a11 = m[5], a12 = m[6];
    const double a20 = m[8], a21 = m[9], a22 = m[10];
    const double c00 = a11 * a22 - a12 * a21, c01 = a10 * a22 - a12 * a20, c02 = a10 * a21 - a11 * a20;
    const double det = a00 * c00 - a01 * c01 + a02 * c02;
    if (!(std::fabs(det) > 1e-30) || !std::isfinite(det)) return false;
    inv[0] = c00 / det;
    inv[1] = (a02 * a21 - a01 * a22) / det;
    inv[2] = (a01 * a12 - a02 * a11) / det;
    inv[4] = (a12 * a20 - a10 * a22) / det;
    inv[5] = (a00 * a22 - a02 * a20) / det;
    inv[6] = (a02 * a10 - a00 * a12) / det;
    inv[8] = c02 / det;
    inv[9] = (a01 * a20 - a00 * a21) / det;
    inv[10] = (a00 * a11 - a01 * a10) / det;
    for (int i = 0; i < 3; ++i)
        inv[4 * i + 3] = -((inv[4 * i] * (double)m[3] + inv[4 * i + 1] * (double)m[7]) + inv[4 * i + 2] * (double)m[11]);
    return true;
}

float Down(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
}
float Up(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}

}  // namespace

extern "C" {

int fnd_rt_instances_upload(fnd_rt_ctx* ctx, const fnd_rt_instance* instances, uint32_t n, fnd_rt_scene** out_scene) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(out_scene != nullptr && (n == 0 || instances != nullptr));
        *out_scene = nullptr;
        CHECK_CODE(n <= (1u << 24), FND_ERR_INVALID_ARG, "%u instances", n);
        std::vector<RT::InstanceRec> recs(n);
        std::vector<float> boxes(9 * (size_t)n);
        double wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
        std::vector<std::array<double, 12>> invs(n);
        for (uint32_t i = 0; i < n; ++i) {
            const fnd_rt_instance& I = instances[i];
            CHECK_CODE(I.scene && I.scene->ctx == ctx, FND_ERR_INVALID_ARG, "instance %u: scene of another context", i);
            CHECK_CODE(!I.scene->two_level, FND_ERR_INVALID_ARG, "instance %u: a two-level scene cannot be instanced",
                       i);
            for (int k = 0; k < 12; ++k)
                CHECK_CODE(std::isfinite(I.transform[k]), FND_ERR_INVALID_ARG, "instance %u: non-finite transform", i);
            CHECK_CODE(Inverse(I.transform, invs[i].data()), FND_ERR_INVALID_ARG, "instance %u: singular transform", i);
            CHECK_CODE((uint64_t)I.prim_offset + I.scene->info.num_tris <= 0xFFFFFFFFull, FND_ERR_INVALID_ARG,
                       "instance %u: prim_offset overflows the 32-bit id", i);
            RT::InstanceRec& r = recs[i];
            r.blas = I.scene->view;
            for (int k = 0; k < 12; ++k) r.inv[k] = (float)invs[i][k];
            r.prim_offset = I.prim_offset;
            // world box of the bottom level's bounds (an empty scene gets a point box)
            const fnd_rt_scene_info& b = I.scene->info;
            double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int c = 0; c < 8; ++c) {
                const double p[3] = {(c & 1) ? b.bounds_hi[0] : b.bounds_lo[0], (c & 2) ? b.bounds_hi[1] : b.bounds_lo[1],
                                     (c & 4) ? b.bounds_hi[2] : b.bounds_lo[2]};
                for (int a = 0; a < 3; ++a) {
                    const float* m = I.transform + 4 * a;
                    const double w = ((double)m[0] * p[0] + (double)m[1] * p[1]) + (double)m[2] * p[2] + (double)m[3];
                    lo[a] = std::min(lo[a], w);
                    hi[a] = std::max(hi[a], w);
                }
            }
            float* t = &boxes[9 * (size_t)i];
            for (int a = 0; a < 3; ++a) {
                t[a] = t[6 + a] = Down(lo[a]);
                t[3 + a] = Up(hi[a]);
                wlo[a] = std::min(wlo[a], lo[a]);
                whi[a] = std::max(whi[a], hi[a]);
            }
        }
        // each bottom level's margin must cover object-space origins of rays
        // that start inside the world box (its margin covers origins within
        // about 50x its own size; 32x is required here)
        for (uint32_t i = 0; i < n; ++i) {
            const fnd_rt_scene* sc = instances[i].scene;
            if (sc->info.num_tris == 0) continue;
            double reach = 0.0;
            for (int c = 0; c < 8; ++c) {
                const double p[3] = {(c & 1) ? whi[0] : wlo[0], (c & 2) ? whi[1] : wlo[1], (c & 4) ? whi[2] : wlo[2]};
                for (int a = 0; a < 3; ++a) {
                    const double* m = invs[i].data() + 4 * a;
                    reach = std::max(reach, std::fabs(((m[0] * p[0] + m[1] * p[1]) + m[2] * p[2]) + m[3]));
                }
            }
            const double covered = 32.0 * 65536.0 * (double)sc->info.box_margin;
            const double base = 32.0 * 65536.0 * (double)RT::SceneMargin(sc->info.bounds_lo, sc->info.bounds_hi);
            CHECK_CODE(reach <= covered, FND_ERR_INVALID_SCENE,
                       "instance %u: its bottom level needs margin_scale >= %.0f (object-space ray origins reach %g)",
                       i, std::ceil(reach / std::max(base, 1e-30)), reach);
        }
        CUDA_CHECK(cudaSetDevice(ctx->device));
        auto scene = std::make_unique<fnd_rt_scene>();
        scene->ctx = ctx;
        scene->two_level = true;
        scene->num_instances = n;
        uint64_t prims = 0;
        for (uint32_t i = 0; i < n; ++i) prims = std::max<uint64_t>(prims, (uint64_t)instances[i].prim_offset +
                                                                              instances[i].scene->info.num_tris);
        scene->info.num_tris = (uint32_t)prims;
        if (n) {
            RT::BuildParams bp;
            RT::BinaryBvh bin;
            RT::BuildBinaryBvh(boxes.data(), n, bp, bin);
            RT::WideBvh wide;
            RT::CollapseToWide(bin, boxes.data(), n, wide);
            CHECK_CODE(wide.depth <= (uint32_t)RT::kMaxStack / 2, FND_ERR_INVALID_SCENE, "top level too deep");
            fnd_rt_scene_info& I = scene->info;
            I.num_binary_nodes = (uint32_t)bin.nodes.size();
            I.binary_depth = bin.depth;
            I.num_leaves = bin.leaves;
            I.sah_cost = bin.sah_cost;
            I.num_wide_nodes = (uint32_t)wide.nodes.size();
            I.wide_depth = wide.depth;
            I.node_bytes = wide.nodes.size() * sizeof(RT::WideNode);
            I.num_refs = n;
            I.tri_bytes = 48ull * n;
            for (int a = 0; a < 3; ++a) {
                I.bounds_lo[a] = wide.lo[a];
                I.bounds_hi[a] = wide.hi[a];
            }
            I.box_margin = wide.margin;
            try {
                CUDA_CHECK(cudaMalloc(&scene->d_nodes, I.node_bytes));
                CUDA_CHECK(cudaMalloc(&scene->d_tris, I.tri_bytes));
                CUDA_CHECK(cudaMalloc(&scene->d_instances, sizeof(RT::InstanceRec) * n));
                char* tris = static_cast<char*>(scene->d_tris);
                CUDA_CHECK(cudaMemcpy(scene->d_nodes, wide.nodes.data(), I.node_bytes, cudaMemcpyHostToDevice));
                CUDA_CHECK(cudaMemcpy(tris, wide.v0.data(), 16ull * n, cudaMemcpyHostToDevice));
                CUDA_CHECK(cudaMemcpy(tris + 16ull * n, wide.v1.data(), 16ull * n, cudaMemcpyHostToDevice));
                CUDA_CHECK(cudaMemcpy(tris + 32ull * n, wide.v2.data(), 16ull * n, cudaMemcpyHostToDevice));
                CUDA_CHECK(cudaMemcpy(scene->d_instances, recs.data(), sizeof(RT::InstanceRec) * n,
                                      cudaMemcpyHostToDevice));
            } catch (...) {
                for (void* p : {scene->d_nodes, scene->d_tris, scene->d_instances})
                    if (p) cudaFree(p);
                throw;
            }
            char* tris = static_cast<char*>(scene->d_tris);
            scene->view.nodes = static_cast<const uint4*>(scene->d_nodes);
            scene->view.v0 = reinterpret_cast<const float4*>(tris);
            scene->view.v1 = reinterpret_cast<const float4*>(tris + 16ull * n);
            scene->view.v2 = reinterpret_cast<const float4*>(tris + 32ull * n);
            scene->view.num_nodes = I.num_wide_nodes;
            scene->view.num_tris = n;
        }
        // shading records by global id: world normals of every instance's triangles
        {
            std::vector<uint32_t> prefix(n + 1, 0), offs(n);
            std::vector<float> inv(12 * (size_t)n);
            std::vector<const float4*> shade(n);
            for (uint32_t i = 0; i < n; ++i) {
                prefix[i + 1] = prefix[i] + instances[i].scene->info.num_tris;
                CHECK_CODE((uint64_t)prefix[i] + instances[i].scene->info.num_tris < (1ull << 32), FND_ERR_INVALID_ARG,
                           "instances hold more than 2^32 triangles");
                offs[i] = instances[i].prim_offset;
                std::copy(recs[i].inv, recs[i].inv + 12, inv.begin() + 12 * (size_t)i);
                shade[i] = static_cast<const float4*>(instances[i].scene->d_tri_shade);
            }
            const uint32_t total = prefix[n];
            const size_t nshade = std::max<size_t>(1, scene->info.num_tris);
            void *d_prefix = nullptr, *d_offs = nullptr, *d_inv = nullptr, *d_ptrs = nullptr;
            try {
                CUDA_CHECK(cudaMalloc(&scene->d_tri_shade, 16 * nshade));
                CUDA_CHECK(cudaMemset(scene->d_tri_shade, 0, 16 * nshade));
                if (total) {
                    CUDA_CHECK(cudaMalloc(&d_prefix, 4ull * (n + 1)));
                    CUDA_CHECK(cudaMalloc(&d_offs, 4ull * n));
                    CUDA_CHECK(cudaMalloc(&d_inv, 48ull * n));
                    CUDA_CHECK(cudaMalloc(&d_ptrs, sizeof(void*) * n));
                    CUDA_CHECK(cudaMemcpy(d_prefix, prefix.data(), 4ull * (n + 1), cudaMemcpyHostToDevice));
                    CUDA_CHECK(cudaMemcpy(d_offs, offs.data(), 4ull * n, cudaMemcpyHostToDevice));
                    CUDA_CHECK(cudaMemcpy(d_inv, inv.data(), 48ull * n, cudaMemcpyHostToDevice));
                    CUDA_CHECK(cudaMemcpy(d_ptrs, shade.data(), sizeof(void*) * n, cudaMemcpyHostToDevice));
                    CUDA_CHECK(RT::InstanceShade(static_cast<const float*>(d_inv), static_cast<const uint32_t*>(d_prefix),
                                                 static_cast<const uint32_t*>(d_offs),
                                                 static_cast<const float4* const*>(d_ptrs), n, total,
                                                 static_cast<float4*>(scene->d_tri_shade), ctx->stream));
                    CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
                }
                CApi::DefaultMaterial(scene.get());
            } catch (...) {
                for (void* p : {d_prefix, d_offs, d_inv, d_ptrs, scene->d_tri_shade, scene->d_nodes, scene->d_tris,
                                scene->d_instances, scene->d_materials})
                    if (p) cudaFree(p);
                throw;
            }
            for (void* p : {d_prefix, d_offs, d_inv, d_ptrs})
                if (p) cudaFree(p);
        }
        for (uint32_t i = 0; i < n; ++i) {
            fnd_rt_scene* b = const_cast<fnd_rt_scene*>(instances[i].scene);
            if (std::find(scene->blas.begin(), scene->blas.end(), b) == scene->blas.end()) {
                scene->blas.push_back(b);
                b->users++;
            }
        }
        *out_scene = scene.release();
        ctx->live_scenes++;
    });
}

}  // extern "C"
