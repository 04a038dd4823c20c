// capi_instances.cpp — two-level scenes (see fnd_rt_instances_upload in
// include/fnd_rt.h): per instance the FP64 inverse transform (rounded to
// FP32) and the world box of its bottom level's bounds, a top-level tree
// over those boxes (the binned-SAH builder fed one degenerate triangle per
// instance, spanning the box), the instance records on the device.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../bvh/bvh_build.hpp"
#include "../bvh/collapse.hpp"
#include "../bvh/gpu_build.hpp"
#include "../bvh/instances.hpp"
#include "context.hpp"

using namespace Foundation;
using Foundation::CApi::Guard;

extern "C" {

int fnd_rt_instances_upload(fnd_rt_ctx* ctx, const fnd_rt_instance* instances, uint32_t n, fnd_rt_scene** out_scene) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(out_scene != nullptr && (n == 0 || instances != nullptr));
        *out_scene = nullptr;
        CHECK_CODE(n <= (1u << 24), FND_ERR_INVALID_ARG, "%u instances", n);
        std::vector<RT::InstanceInput> in(n);
        for (uint32_t i = 0; i < n; ++i) {
            const fnd_rt_instance& I = instances[i];
            CHECK_CODE(I.scene && I.scene->ctx == ctx, FND_ERR_INVALID_ARG, "instance %u: scene of another context", i);
            CHECK_CODE(!I.scene->two_level, FND_ERR_INVALID_ARG, "instance %u: a two-level scene cannot be instanced",
                       i);
            CHECK_CODE((uint64_t)I.prim_offset + I.scene->info.num_tris <= 0xFFFFFFFFull, FND_ERR_INVALID_ARG,
                       "instance %u: prim_offset overflows the 32-bit id", i);
            std::copy(I.transform, I.transform + 12, in[i].transform);
            std::copy(I.scene->info.bounds_lo, I.scene->info.bounds_lo + 3, in[i].lo);
            std::copy(I.scene->info.bounds_hi, I.scene->info.bounds_hi + 3, in[i].hi);
        }
        RT::InstanceTop top;
        RT::BuildInstanceTop(in.data(), n, top);
        std::vector<RT::InstanceRec> recs(n);
        for (uint32_t i = 0; i < n; ++i) {
            RT::InstanceRec& r = recs[i];
            r.blas = instances[i].scene->view;
            std::copy(&top.inv[12 * (size_t)i], &top.inv[12 * (size_t)i] + 12, r.inv);
            r.prim_offset = instances[i].prim_offset;
            static const float kId[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
            r.flags = std::memcmp(r.inv, kId, sizeof(kId)) == 0 ? RT::kInstanceIdentity : 0u;  // bit for bit
        }
        // each bottom level's margin must cover object-space origins of rays
        // that start inside the world box (its margin covers origins within
        // about 50x its own size; 32x is required here)
        for (uint32_t i = 0; i < n; ++i) {
            const fnd_rt_scene* sc = instances[i].scene;
            if (sc->info.num_tris == 0) continue;
            const double reach = RT::InstanceReach(&top.inv[12 * (size_t)i], top.lo, top.hi);
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
            const RT::BinaryBvh& bin = top.bin;
            const RT::WideBvh& wide = top.wide;
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
