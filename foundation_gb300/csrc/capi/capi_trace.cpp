// capi_trace.cpp — C ABI: context, scene upload, closest / any-hit traversal.
//
// Every entry point runs its body inside Guard(): C++ failures (FndError from
// CHECK / Fail, std::bad_alloc, CUDA errors) become a negative fnd_status and
// a message in fnd_rt_last_error; nothing throws across the ABI and nothing
// terminates the process (the reference's CHECK -> BugCheck -> terminate,
// src/Core/Core.cpp:7-10, is not acceptable behind a C ABI).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../bvh/bvh_build.hpp"
#include "../bvh/collapse.hpp"
#include "../bvh/gpu_build.hpp"
#include "context.hpp"

using namespace Foundation;
using Foundation::RtCore::Fail;
using Foundation::RtCore::FndError;

namespace {

double MsSince(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void UseDevice(const fnd_rt_ctx* ctx) { CUDA_CHECK(cudaSetDevice(ctx->device)); }

}  // namespace

namespace Foundation {
namespace CApi {

std::string& GlobalError() {
    thread_local std::string msg;
    return msg;
}

void CudaCheck(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    const int code = e == cudaErrorMemoryAllocation ? FND_ERR_OUT_OF_MEMORY
                     : (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) ? FND_ERR_NO_DEVICE
                                                                                 : FND_ERR_CUDA;
    Fail(code, "%s failed: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

void EnsureDevice(void*& ptr, size_t& cap, size_t bytes) {
    if (bytes <= cap) return;
    if (ptr) CUDA_CHECK(cudaFree(ptr));
    ptr = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4;
    CUDA_CHECK(cudaMalloc(&ptr, want));
    cap = want;
}

cudaError_t LaunchTraceOrdered(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, RT::TraceLaunch L, bool any, bool stats,
                               const RT::TraceConfig& cfg, int grid, cudaStream_t stream) {
    if (!stream) stream = ctx->stream;
    L.order = nullptr;
    if (cfg.sort_bits && L.n > 1 && scene->view.num_nodes) {
        const size_t m = size_t(1) << cfg.sort_bits;
        const size_t need = RT::RaySortScratchBytes(L.n, cfg.sort_bits) + 1024;  // + alignment of the parts
        EnsureDevice(ctx->d_sort, ctx->d_sort_cap, need);
        auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
        char* p = static_cast<char*>(ctx->d_sort);
        RT::RaySortBuffers B{};
        B.keys = reinterpret_cast<uint32_t*>(p);
        p += align(sizeof(uint32_t) * (size_t)L.n);
        B.order = reinterpret_cast<uint32_t*>(p);
        p += align(sizeof(uint32_t) * (size_t)L.n);
        B.hist = reinterpret_cast<uint32_t*>(p);
        p += align(sizeof(uint32_t) * m);
        B.sums = reinterpret_cast<uint32_t*>(p);
        const cudaError_t e = RT::LaunchRaySort(L.rays, L.n, L.n_dev, scene->info.bounds_lo, scene->info.bounds_hi,
                                                cfg.sort_bits, B, stream);
        if (e != cudaSuccess) return e;
        L.order = B.order;
    }
    return RT::LaunchTraceConfigured(L, any, stats, cfg, grid, stream);
}

int ReadStatus(fnd_rt_ctx* ctx) {
    CUDA_CHECK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    const uint32_t s = *ctx->h_status;
    if (s == 0) return FND_OK;
    CUDA_CHECK(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    return RT::StatusCode(s);
}

}  // namespace CApi
}  // namespace Foundation

using namespace Foundation::CApi;

namespace {

}  // namespace

namespace Foundation {
namespace CApi {

// One grey Lambertian until fnd_rt_scene_set_materials.
void DefaultMaterial(fnd_rt_scene* scene) {
    PT::DevMaterial m{};
    m.albedo_type = make_float4(0.8f, 0.8f, 0.8f, 0.0f);
    m.emission_light = make_float4(0.f, 0.f, 0.f, __builtin_bit_cast(float, (int32_t)-1));
    m.params = make_float4(1.0f, 0.f, 0.f, 0.f);
    CUDA_CHECK(cudaMalloc(&scene->d_materials, sizeof(m)));
    CUDA_CHECK(cudaMemcpy(scene->d_materials, &m, sizeof(m), cudaMemcpyHostToDevice));
    scene->num_materials = 1;
}

}  // namespace CApi
}  // namespace Foundation

namespace {

// FND_BVH_GPU_BUILD: the vertices and indices go to the device once and the
// tree is built there (bvh/gpu_build.cu).
void UploadGpuBuilt(fnd_rt_ctx* ctx, fnd_rt_scene* scene, const float* verts, uint32_t nv, const uint32_t* idx,
                    uint32_t nt, const RT::BuildParams& bp, float margin_scale, const RT::CollapseOptions& copt,
                    uint32_t cluster_radius) {
    void *d_verts = nullptr, *d_idx = nullptr;
    RT::GpuBuildOutput go;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        CUDA_CHECK(cudaMalloc(&d_verts, 12ull * std::max(nv, 1u)));
        CUDA_CHECK(cudaMalloc(&d_idx, 12ull * nt));
        if (nv) CUDA_CHECK(cudaMemcpyAsync(d_verts, verts, 12ull * nv, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(d_idx, idx, 12ull * nt, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        const double upload_ms = MsSince(t0);
        RT::GpuBuildParams gp;
        gp.max_leaf = bp.max_leaf;
        gp.trav_cost = bp.trav_cost;
        gp.margin_scale = margin_scale;
        gp.sah_collapse = copt.sah;
        gp.c_tri = (float)copt.c_tri;
        gp.ploc_radius = cluster_radius;
        gp.width = copt.width;
        RT::BuildWideGpu(static_cast<const float*>(d_verts), nv, static_cast<const uint32_t*>(d_idx), nt, gp, go,
                         ctx->stream);
        CUDA_CHECK(cudaFree(d_verts));
        CUDA_CHECK(cudaFree(d_idx));
        d_verts = d_idx = nullptr;
        scene->d_nodes = go.d_nodes;
        scene->d_tris = go.d_tris;
        scene->d_tri_shade = go.d_tri_shade;
        go.d_nodes = go.d_tris = go.d_tri_shade = nullptr;
        CApi::DefaultMaterial(scene);
        fnd_rt_scene_info& I = scene->info;
        I.num_binary_nodes = go.num_binary_nodes;
        I.binary_depth = 0;  // not tracked by the GPU build
        I.num_leaves = go.leaves;
        I.sah_cost = go.sah_cost;
        I.num_wide_nodes = go.num_nodes;
        I.wide_depth = go.depth;
        I.node_bytes = (uint64_t)go.num_nodes * sizeof(RT::WideNode);
        I.num_refs = go.num_refs;
        I.tri_bytes = 48ull * go.num_refs;
        for (int a = 0; a < 3; ++a) {
            I.bounds_lo[a] = go.lo[a];
            I.bounds_hi[a] = go.hi[a];
        }
        I.box_margin = go.margin;
        I.build_ms = go.build_ms;
        I.collapse_ms = go.collapse_ms;
        I.upload_ms = upload_ms;
    } catch (...) {
        for (void* p : {go.d_nodes, go.d_tris, go.d_tri_shade, d_verts, d_idx, scene->d_nodes, scene->d_tris,
                        scene->d_tri_shade, scene->d_materials})
            if (p) cudaFree(p);
        scene->d_nodes = scene->d_tris = scene->d_tri_shade = scene->d_materials = nullptr;
        throw;
    }
    char* tris = static_cast<char*>(scene->d_tris);
    const size_t plane = 16ull * scene->info.num_refs;
    scene->view.nodes = static_cast<const uint4*>(scene->d_nodes);
    scene->view.v0 = reinterpret_cast<const float4*>(tris);
    scene->view.v1 = reinterpret_cast<const float4*>(tris + plane);
    scene->view.v2 = reinterpret_cast<const float4*>(tris + 2 * plane);
    scene->view.num_nodes = scene->info.num_wide_nodes;
    scene->view.num_tris = scene->info.num_refs;
}

}  // namespace

extern "C" {

int fnd_rt_create(const fnd_rt_desc* desc, fnd_rt_ctx** out_ctx) {
    return Guard(nullptr, [&] {
        CHECK(desc != nullptr && out_ctx != nullptr);
        *out_ctx = nullptr;
        CHECK_CODE(desc->abi_version == FND_RT_ABI_VERSION, FND_ERR_INVALID_ARG, "ABI version %u, library has %u",
                   desc->abi_version, FND_RT_ABI_VERSION);
        int count = 0;
        CUDA_CHECK(cudaGetDeviceCount(&count));
        CHECK_CODE(desc->device >= 0 && desc->device < count, FND_ERR_NO_DEVICE, "device %d of %d", desc->device,
                   count);
        cudaDeviceProp prop;
        CUDA_CHECK(cudaGetDeviceProperties(&prop, desc->device));
        CHECK_CODE(prop.major == 10 && prop.minor == 3, FND_ERR_NO_DEVICE,
                   "device %d is sm_%d%d; this library is built for sm_103a only", desc->device, prop.major,
                   prop.minor);
        auto ctx = std::make_unique<fnd_rt_ctx>();
        ctx->device = desc->device;
        ctx->sm_count = prop.multiProcessorCount;
        CUDA_CHECK(cudaSetDevice(ctx->device));
        auto cleanup = [&](fnd_rt_ctx* c) {
            if (c->d_counter) cudaFree(c->d_counter);
            if (c->h_status) cudaFreeHost(c->h_status);
            if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
        };
        try {
            if (desc->stream) {
                ctx->stream = (cudaStream_t)desc->stream;
            } else {
                CUDA_CHECK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
                ctx->own_stream = true;
            }
            // one allocation: counter (256 B slot), status (256 B slot), stats
            char* scratch = nullptr;
            CUDA_CHECK(cudaMalloc(&scratch, 1024));
            ctx->d_counter = reinterpret_cast<uint32_t*>(scratch);
            ctx->d_status = reinterpret_cast<uint32_t*>(scratch + 256);
            ctx->d_stats = reinterpret_cast<unsigned long long*>(scratch + 512);
            ctx->d_render_stats = reinterpret_cast<unsigned long long*>(scratch + 768);
            CUDA_CHECK(cudaMemsetAsync(scratch, 0, 1024, ctx->stream));
            CUDA_CHECK(cudaMallocHost(&ctx->h_status, sizeof(uint32_t)));
            for (int v = 0; v < 4; ++v) CUDA_CHECK(RT::TraceOccupancy(v, &ctx->occupancy[v]));
            CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            cleanup(ctx.get());
            throw;
        }
        if (const char* s = std::getenv("FND_RT_REFILL_MIN")) ctx->refill_min = (uint32_t)std::atoi(s);
        *out_ctx = ctx.release();
    });
}

int fnd_rt_destroy(fnd_rt_ctx* ctx) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    const int rc = Guard(ctx, [&] {
        CHECK_CODE(ctx->live_scenes == 0, FND_ERR_INVALID_ARG, "%d scenes still alive", ctx->live_scenes);
        UseDevice(ctx);
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
    if (rc == FND_ERR_INVALID_ARG) return rc;
    // the context is freed below: keep its failure message in the global slot
    GlobalError() = ctx->last_error;
    cudaSetDevice(ctx->device);
    FreeCache(ctx);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    if (ctx->d_in) cudaFree(ctx->d_in);
    if (ctx->d_out) cudaFree(ctx->d_out);
    if (ctx->d_paths) cudaFree(ctx->d_paths);
    if (ctx->d_fb) cudaFree(ctx->d_fb);
    if (ctx->d_rgb) cudaFree(ctx->d_rgb);
    if (ctx->d_sort) cudaFree(ctx->d_sort);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    for (cudaEvent_t e : ctx->pipe_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
    if (ctx->compute2) cudaStreamDestroy(ctx->compute2);
    if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return rc;
}

const char* fnd_rt_last_error(const fnd_rt_ctx* ctx) { return ctx ? ctx->last_error.c_str() : GlobalError().c_str(); }

int fnd_rt_sync(fnd_rt_ctx* ctx) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    int status = FND_OK;
    const int rc = Guard(ctx, [&] {
        UseDevice(ctx);
        status = ReadStatus(ctx);
        if (status != FND_OK)
            Fail(status, "device status: %s",
                 status == FND_ERR_STACK_OVERFLOW   ? "traversal stack overflow"
                 : status == FND_ERR_INVALID_SCENE ? "scene index out of range"
                                                    : "bounded wait timed out");
    });
    return rc;
}

void* fnd_rt_stream(const fnd_rt_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int fnd_rt_scene_upload(fnd_rt_ctx* ctx, const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt,
                        const fnd_rt_bvh_desc* bvh, fnd_rt_scene** out_scene) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(out_scene != nullptr);
        *out_scene = nullptr;
        CHECK(nt == 0 || (verts != nullptr && idx != nullptr));
        CHECK_CODE(nt <= (1u << 30), FND_ERR_INVALID_SCENE, "%u triangles exceed the 2^30 limit", nt);
        RT::BuildParams bp;
        if (bvh) {
            if (bvh->sah_bins) bp.bins = bvh->sah_bins;
            if (bvh->max_leaf_tris) bp.max_leaf = bvh->max_leaf_tris;
            bp.threads = bvh->build_threads;
            if (bvh->traversal_cost != 0.0f) bp.trav_cost = bvh->traversal_cost;
            if (bvh->split_budget != 0.0f) bp.max_refs_factor = bvh->split_budget;
        }
        CHECK_CODE(bp.max_refs_factor >= 0.0 && bp.max_refs_factor <= 16.0, FND_ERR_INVALID_ARG,
                   "split_budget %g not in [0, 16]", bp.max_refs_factor);
        // references are indexed with 32 bits
        CHECK_CODE(!(bvh && (bvh->flags & FND_BVH_SPATIAL_SPLITS)) ||
                       (double)nt * (1.0 + bp.max_refs_factor) < 4294967295.0,
                   FND_ERR_INVALID_ARG, "split_budget %g allows more than 2^32 references for %u triangles",
                   bp.max_refs_factor, nt);
        const float margin_scale = bvh && bvh->margin_scale != 0.0f ? bvh->margin_scale : 1.0f;
        CHECK_CODE(margin_scale >= 1.0f && margin_scale <= 65536.0f, FND_ERR_INVALID_ARG,
                   "margin_scale %g not in [1, 65536]", (double)margin_scale);
        CHECK_CODE(bp.trav_cost > 0.0f && bp.trav_cost <= 64.0f, FND_ERR_INVALID_ARG, "traversal_cost %g not in (0, 64]",
                   (double)bp.trav_cost);
        CHECK_CODE(bp.bins >= 2 && bp.bins <= 64, FND_ERR_INVALID_ARG, "sah_bins %u not in [2, 64]", bp.bins);
        CHECK_CODE(bp.max_leaf >= 1 && bp.max_leaf <= 4, FND_ERR_INVALID_ARG, "max_leaf_tris %u not in [1, 4]",
                   bp.max_leaf);
        CHECK_CODE(!bvh || (bvh->flags & ~(uint32_t)(FND_BVH_SPATIAL_SPLITS | FND_BVH_GPU_BUILD |
                                                     FND_BVH_SAH_COLLAPSE | FND_BVH_GPU_CLUSTER |
                                                     FND_BVH_CLUSTER_RADIUS(255) | FND_BVH_NODE_WIDTH(15))) == 0,
                   FND_ERR_INVALID_ARG, "unknown BVH flags 0x%x", bvh ? bvh->flags : 0u);
        const uint32_t radius_bits = bvh ? (bvh->flags >> 8) & 255u : 0u;
        const uint32_t width_bits = bvh ? (bvh->flags >> 16) & 15u : 0u;
        CHECK_CODE(width_bits == 0 || (width_bits >= 2 && width_bits <= 8), FND_ERR_INVALID_ARG,
                   "node width %u not in 2..8", width_bits);
        CHECK_CODE(radius_bits <= 64, FND_ERR_INVALID_ARG, "clustering radius %u not in 1..64", radius_bits);
        CHECK_CODE(!bvh || (bvh->flags & FND_BVH_GPU_CLUSTER) || radius_bits == 0, FND_ERR_INVALID_ARG,
                   "FND_BVH_CLUSTER_RADIUS without FND_BVH_GPU_CLUSTER");
        CHECK_CODE(!bvh || !(bvh->flags & FND_BVH_GPU_CLUSTER) || (bvh->flags & FND_BVH_GPU_BUILD),
                   FND_ERR_INVALID_ARG, "FND_BVH_GPU_CLUSTER without FND_BVH_GPU_BUILD");
        const uint32_t cluster_radius =
            bvh && (bvh->flags & FND_BVH_GPU_CLUSTER) ? (radius_bits ? radius_bits : 2u) : 0u;
        RT::CollapseOptions copt;
        copt.sah = bvh && (bvh->flags & FND_BVH_SAH_COLLAPSE);
        copt.threads = bvh ? bvh->build_threads : 0u;
        copt.width = width_bits ? width_bits : 8u;
        copt.c_tri = bvh && bvh->collapse_tri_cost != 0.0f ? bvh->collapse_tri_cost : 0.3;
        CHECK_CODE(copt.c_tri > 0.0 && copt.c_tri <= 16.0, FND_ERR_INVALID_ARG, "collapse_tri_cost %g not in (0, 16]",
                   copt.c_tri);
        const bool gpu_build = bvh && (bvh->flags & FND_BVH_GPU_BUILD);
        CHECK_CODE(!(gpu_build && (bvh->flags & FND_BVH_SPATIAL_SPLITS)), FND_ERR_INVALID_ARG,
                   "FND_BVH_GPU_BUILD does not combine with FND_BVH_SPATIAL_SPLITS");
        UseDevice(ctx);
        auto scene = std::make_unique<fnd_rt_scene>();
        scene->ctx = ctx;
        scene->info.num_tris = nt;
        if (nt == 0) {
            *out_scene = scene.release();
            ctx->live_scenes++;
            return;
        }
        if (gpu_build) {
            UploadGpuBuilt(ctx, scene.get(), verts, nv, idx, nt, bp, margin_scale, copt, cluster_radius);
            *out_scene = scene.release();
            ctx->live_scenes++;
            return;
        }
        // gather + validate (parallel over triangle ranges)
        std::vector<float> tri(9 * (size_t)nt);
        {
            const unsigned threads = bp.threads ? bp.threads : std::max(1u, std::thread::hardware_concurrency());
            std::vector<std::thread> pool;
            std::vector<int> bad(threads, 0);
            const uint32_t chunk = (nt + threads - 1) / threads;
            for (unsigned w = 0; w < threads; ++w) {
                pool.emplace_back([&, w] {
                    const uint32_t s = w * chunk, e = std::min<uint64_t>(nt, (uint64_t)s + chunk);
                    for (uint32_t t = s; t < e && !bad[w]; ++t)
                        for (int k = 0; k < 3; ++k) {
                            const uint32_t vi = idx[3 * (size_t)t + k];
                            if (vi >= nv) {
                                bad[w] = 1;
                                break;
                            }
                            for (int c = 0; c < 3; ++c) {
                                const float x = verts[3 * (size_t)vi + c];
                                if (!std::isfinite(x)) bad[w] = 2;
                                tri[9 * (size_t)t + 3 * k + c] = x;
                            }
                        }
                });
            }
            for (auto& t : pool) t.join();
            for (int b : bad) {
                CHECK_CODE(b != 1, FND_ERR_INVALID_ARG, "vertex index out of range (nv = %u)", nv);
                CHECK_CODE(b != 2, FND_ERR_INVALID_ARG, "non-finite vertex coordinate");
            }
        }
        // geometric normals (winding order) for shading; material 0 until set
        scene->tri_shade.resize(4 * (size_t)nt);
        for (uint32_t t = 0; t < nt; ++t) {
            const float* v = &tri[9 * (size_t)t];
            const float e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
            const float e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
            float nx = e1[1] * e2[2] - e1[2] * e2[1], ny = e1[2] * e2[0] - e1[0] * e2[2],
                  nz = e1[0] * e2[1] - e1[1] * e2[0];
            const float l = std::sqrt(nx * nx + ny * ny + nz * nz);
            if (l > 0.0f) {
                nx /= l;
                ny /= l;
                nz /= l;
            } else {
                nx = ny = 0.0f;
                nz = 1.0f;
            }
            float* o = &scene->tri_shade[4 * (size_t)t];
            o[0] = nx;
            o[1] = ny;
            o[2] = nz;
            o[3] = 0.0f;  // material 0 (bits)
        }
        auto t0 = std::chrono::steady_clock::now();
        RT::BinaryBvh bin;
        if (bvh && (bvh->flags & FND_BVH_SPATIAL_SPLITS))
            RT::BuildBinarySbvh(tri.data(), nt, bp, bin);
        else
            RT::BuildBinaryBvh(tri.data(), nt, bp, bin);
        scene->info.build_ms = MsSince(t0);
        t0 = std::chrono::steady_clock::now();
        RT::WideBvh wide;
        RT::CollapseToWide(bin, tri.data(), nt, wide, margin_scale, copt);
        scene->info.collapse_ms = MsSince(t0);
        CHECK_CODE(wide.depth <= (uint32_t)RT::kMaxStack / 2, FND_ERR_INVALID_SCENE,
                   "wide BVH depth %u exceeds the traversal stack bound %d", wide.depth, RT::kMaxStack / 2);
        fnd_rt_scene_info& I = scene->info;
        I.num_binary_nodes = (uint32_t)bin.nodes.size();
        I.binary_depth = bin.depth;
        I.num_leaves = bin.leaves;
        I.sah_cost = bin.sah_cost;
        I.num_wide_nodes = (uint32_t)wide.nodes.size();
        I.wide_depth = wide.depth;
        I.node_bytes = wide.nodes.size() * sizeof(RT::WideNode);
        I.num_refs = (uint32_t)bin.prims.size();
        I.tri_bytes = 3ull * 16ull * I.num_refs;
        for (int a = 0; a < 3; ++a) {
            I.bounds_lo[a] = wide.lo[a];
            I.bounds_hi[a] = wide.hi[a];
        }
        I.box_margin = wide.margin;
        t0 = std::chrono::steady_clock::now();
        try {
            CUDA_CHECK(cudaMalloc(&scene->d_nodes, I.node_bytes));
            CUDA_CHECK(cudaMalloc(&scene->d_tris, I.tri_bytes));
            char* tris = static_cast<char*>(scene->d_tris);
            const size_t plane = 16ull * I.num_refs;
            CUDA_CHECK(cudaMemcpy(scene->d_nodes, wide.nodes.data(), I.node_bytes, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(tris, wide.v0.data(), plane, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(tris + plane, wide.v1.data(), plane, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(tris + 2 * plane, wide.v2.data(), plane, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMalloc(&scene->d_tri_shade, 16ull * nt));
            CUDA_CHECK(cudaMemcpy(scene->d_tri_shade, scene->tri_shade.data(), 16ull * nt, cudaMemcpyHostToDevice));
            std::vector<float>().swap(scene->tri_shade);  // the device copy is the only one kept
            CApi::DefaultMaterial(scene.get());
        } catch (...) {
            if (scene->d_nodes) cudaFree(scene->d_nodes);
            if (scene->d_tris) cudaFree(scene->d_tris);
            if (scene->d_tri_shade) cudaFree(scene->d_tri_shade);
            if (scene->d_materials) cudaFree(scene->d_materials);
            throw;
        }
        I.upload_ms = MsSince(t0);
        char* tris = static_cast<char*>(scene->d_tris);
        const size_t plane = 16ull * I.num_refs;
        scene->view.nodes = static_cast<const uint4*>(scene->d_nodes);
        scene->view.v0 = reinterpret_cast<const float4*>(tris);
        scene->view.v1 = reinterpret_cast<const float4*>(tris + plane);
        scene->view.v2 = reinterpret_cast<const float4*>(tris + 2 * plane);
        scene->view.num_nodes = I.num_wide_nodes;
        scene->view.num_tris = I.num_refs;
        *out_scene = scene.release();
        ctx->live_scenes++;
    });
}

int fnd_rt_scene_info_get(const fnd_rt_scene* scene, fnd_rt_scene_info* out_info) {
    if (!scene || !out_info) return FND_ERR_INVALID_ARG;
    *out_info = scene->info;
    return FND_OK;
}

int fnd_rt_scene_destroy(fnd_rt_scene* scene) {
    if (!scene) return FND_ERR_INVALID_ARG;
    fnd_rt_ctx* ctx = scene->ctx;
    if (scene->users > 0) {
        if (ctx) ctx->last_error = "scene is instanced by a live two-level scene";
        return FND_ERR_INVALID_ARG;
    }
    const int rc = Guard(ctx, [&] {
        UseDevice(ctx);
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        for (fnd_rt_scene* b : scene->blas) b->users--;
        scene->blas.clear();
        if (scene->d_instances) CUDA_CHECK(cudaFree(scene->d_instances));
        if (scene->d_nodes) CUDA_CHECK(cudaFree(scene->d_nodes));
        if (scene->d_tris) CUDA_CHECK(cudaFree(scene->d_tris));
        if (scene->d_tri_shade) CUDA_CHECK(cudaFree(scene->d_tri_shade));
        if (scene->d_materials) CUDA_CHECK(cudaFree(scene->d_materials));
        if (scene->d_lights) CUDA_CHECK(cudaFree(scene->d_lights));
    });
    ctx->live_scenes--;
    delete scene;
    return rc;
}

}  // extern "C"

namespace {

// Host-buffer traces of at least two chunks run as a pipeline: chunk k's rays
// go in on one copy stream while chunk k - 1 is traced and chunk k - 2's hits
// come back on another, so the copies hide under the traversal. In input
// order the chunks alternate between the context stream and a second compute
// stream, each with its own work counter, so a chunk's blocks start on the
// SMs the previous chunk's last blocks leave; in coherence order (which
// shares the sort scratch) they all run on the context stream. Chunks of at
// least 2^19 rays, 8 per call at 2^22 rays and above, plus a first chunk of a
// quarter of that size, so at most 17 per call.
// Per chunk the launch, its tail and the stream waits cost more than the
// shorter uncovered first copy saves below 2^20 rays per chunk (measured:
// 8.4M rays in 8 chunks 2.74 ms, in 16 chunks 2.91 ms per call).
constexpr uint32_t kPipeMinChunk = 1u << 19;
constexpr uint32_t kPipeMaxChunks = 16;

uint32_t PipelineChunk(uint32_t n) {
    uint32_t chunk = std::max(kPipeMinChunk, (n + 7u) / 8u);
    chunk = std::max(chunk, (uint32_t)(((uint64_t)n + kPipeMaxChunks - 1) / kPipeMaxChunks));
    return chunk;
}

void EnsurePipeline(fnd_rt_ctx* ctx) {
    if (!ctx->copy_in) CUDA_CHECK(cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
    if (!ctx->copy_out) CUDA_CHECK(cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
    if (!ctx->compute2) CUDA_CHECK(cudaStreamCreateWithFlags(&ctx->compute2, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ctx->pipe_ev)
        if (!e) CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

int TraceImpl(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n, void* out, int mem,
              bool any, fnd_rt_trace_stats* stats) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(scene != nullptr && scene->ctx == ctx);
        CHECK(mem == FND_MEM_HOST || mem == FND_MEM_DEVICE);
        CHECK(n == 0 || (rays != nullptr && out != nullptr));
        CHECK_CODE(n <= (1u << 31), FND_ERR_INVALID_ARG, "%u rays exceed the 2^31 limit per call", n);
        CHECK_CODE(!(scene->two_level && stats), FND_ERR_INVALID_ARG,
                   "trace statistics are not kept for two-level scenes");
        UseDevice(ctx);
        const size_t hit_bytes = any ? 1 : sizeof(fnd_hit);
        // one traversal launch over `cnt` device-resident rays on `st` with
        // work counter `counter`
        auto launch = [&](const float4* d_rays, uint32_t cnt, void* d_out, cudaStream_t st, uint32_t* counter) {
            RT::TraceLaunch L{};
            L.scene = scene->view;
            L.n = cnt;
            L.counter = counter;
            L.status = ctx->d_status;
            L.stats = ctx->d_stats;
            L.refill_min = ctx->refill_min;
            L.rays = d_rays;
            if (any)
                L.occluded = static_cast<uint8_t*>(d_out);
            else
                L.hits = d_out;
            if (scene->two_level) {
                RT::InstancedLaunch I{};
                I.tlas = scene->view;
                I.inst = static_cast<const RT::InstanceRec*>(scene->d_instances);
                I.num_inst = scene->num_instances;
                I.rays = L.rays;
                I.n = cnt;
                I.hits = L.hits;
                I.occluded = L.occluded;
                I.counter = counter;
                I.status = ctx->d_status;
                if (scene->num_instances == 0) {
                    RT::TraceLaunch E = L;  // no instances: every ray misses
                    E.scene = RT::DeviceScene{};
                    CUDA_CHECK(RT::LaunchTraceConfigured(E, any, false, ctx->trace_cfg, 1, st));
                } else {
                    CUDA_CHECK(RT::LaunchInstanced(I, any, ctx->sm_count, st));
                }
            } else {
                const int variant = (any ? 1 : 0) + (stats ? 2 : 0);
                const int grid = TraceGrid(ctx, ctx->trace_cfg, variant);
                CUDA_CHECK(LaunchTraceOrdered(ctx, scene, L, any, stats != nullptr, ctx->trace_cfg, grid, st));
            }
        };
        if (stats) CUDA_CHECK(cudaMemsetAsync(ctx->d_stats, 0, 4 * sizeof(unsigned long long), ctx->stream));
        bool copied_back = false;
        if (mem == FND_MEM_DEVICE) {
            CHECK_CODE(((uintptr_t)rays & 15u) == 0 && ((uintptr_t)out & (any ? 0u : 7u)) == 0, FND_ERR_INVALID_ARG,
                       "device rays must be 16-byte aligned and hits 8-byte aligned");
            launch(reinterpret_cast<const float4*>(rays), n, out, ctx->stream, ctx->d_counter);
        } else if (n > 0) {
            EnsureDevice(ctx->d_in, ctx->d_in_cap, sizeof(fnd_ray) * (size_t)n);
            EnsureDevice(ctx->d_out, ctx->d_out_cap, hit_bytes * (size_t)n);
            auto* d_in = static_cast<char*>(ctx->d_in);
            auto* d_out = static_cast<char*>(ctx->d_out);
            const uint32_t chunk = PipelineChunk(n);
            if (stats || n <= chunk) {
                CUDA_CHECK(cudaMemcpyAsync(d_in, rays, sizeof(fnd_ray) * (size_t)n, cudaMemcpyHostToDevice,
                                           ctx->stream));
                launch(reinterpret_cast<const float4*>(d_in), n, d_out, ctx->stream, ctx->d_counter);
            } else {
                EnsurePipeline(ctx);
                // on a failure part-way, the copies already queued on the
                // library's streams still read and write the caller's host
                // buffers: let them finish before the error returns
                auto drain = [&] {
                    cudaStreamSynchronize(ctx->copy_in);
                    cudaStreamSynchronize(ctx->compute2);
                    cudaStreamSynchronize(ctx->stream);
                    cudaStreamSynchronize(ctx->copy_out);
                };
                try {
                    cudaEvent_t* ev = ctx->pipe_ev;
                    const bool two = ctx->trace_cfg.sort_bits == 0;
                    // the copy and compute streams start after the context
                    // stream's earlier work
                    CUDA_CHECK(cudaEventRecord(ev[0], ctx->stream));
                    CUDA_CHECK(cudaStreamWaitEvent(ctx->copy_in, ev[0], 0));
                    CUDA_CHECK(cudaStreamWaitEvent(ctx->copy_out, ev[0], 0));
                    if (two) CUDA_CHECK(cudaStreamWaitEvent(ctx->compute2, ev[0], 0));
                    // chunk 0 is a quarter of the others: its copy in is
                    // the part of the copies no traversal covers
                    const uint32_t c0 = chunk / 4;
                    const uint32_t chunks = 1 + (n - c0 + chunk - 1) / chunk;
                    CHECK(2 + 2 * (size_t)chunks <= sizeof(ctx->pipe_ev) / sizeof(ctx->pipe_ev[0]));
                    for (uint32_t k = 0; k < chunks; ++k) {
                        const size_t first = k == 0 ? 0 : (size_t)c0 + (size_t)(k - 1) * chunk;
                        const uint32_t cnt = (uint32_t)std::min<size_t>(k == 0 ? c0 : chunk, n - first);
                        cudaEvent_t in_done = ev[2 + 2 * k], traced = ev[3 + 2 * k];
                        CUDA_CHECK(cudaMemcpyAsync(d_in + sizeof(fnd_ray) * first, rays + first,
                                                   sizeof(fnd_ray) * cnt, cudaMemcpyHostToDevice, ctx->copy_in));
                        CUDA_CHECK(cudaEventRecord(in_done, ctx->copy_in));
                        // odd chunks on the second compute stream, with the
                        // counter 32 bytes further in the counter slot
                        const bool odd = two && (k & 1u);
                        cudaStream_t cs = odd ? ctx->compute2 : ctx->stream;
                        CUDA_CHECK(cudaStreamWaitEvent(cs, in_done, 0));
                        launch(reinterpret_cast<const float4*>(d_in + sizeof(fnd_ray) * first), cnt,
                               d_out + hit_bytes * first, cs, ctx->d_counter + (odd ? 8 : 0));
                        CUDA_CHECK(cudaEventRecord(traced, cs));
                        CUDA_CHECK(cudaStreamWaitEvent(ctx->copy_out, traced, 0));
                        CUDA_CHECK(cudaMemcpyAsync(static_cast<char*>(out) + hit_bytes * first,
                                                   d_out + hit_bytes * first, hit_bytes * cnt,
                                                   cudaMemcpyDeviceToHost, ctx->copy_out));
                    }
                    // the context stream (which the status read below waits
                    // on) covers the last copy back
                    CUDA_CHECK(cudaEventRecord(ev[1], ctx->copy_out));
                    CUDA_CHECK(cudaStreamWaitEvent(ctx->stream, ev[1], 0));
                } catch (...) {
                    drain();
                    throw;
                }
                copied_back = true;
            }
        }
        if (stats) {
            unsigned long long h[4] = {0, 0, 0, 0};
            CUDA_CHECK(cudaMemcpyAsync(h, ctx->d_stats, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
            stats->rays = n;
            stats->node_fetches = h[0];
            stats->tri_tests = h[1];
            stats->warp_node_steps = h[2];
            stats->warp_tri_steps = h[3];
        }
        if (mem == FND_MEM_HOST) {
            if (n && !copied_back)
                CUDA_CHECK(cudaMemcpyAsync(out, ctx->d_out, hit_bytes * (size_t)n, cudaMemcpyDeviceToHost,
                                           ctx->stream));
            const int s = ReadStatus(ctx);
            if (s != FND_OK)
                Fail(s, "device status: %s",
                     s == FND_ERR_STACK_OVERFLOW ? "traversal stack overflow" : "scene index out of range");
        }
    });
}

}  // namespace

extern "C" {

int fnd_rt_trace_closest(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n, fnd_hit* out,
                         int mem) {
    return TraceImpl(ctx, scene, rays, n, out, mem, false, nullptr);
}

int fnd_rt_trace_any(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n, uint8_t* out,
                     int mem) {
    return TraceImpl(ctx, scene, rays, n, out, mem, true, nullptr);
}

int fnd_rt_trace_closest_stats(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n,
                               fnd_hit* out, int mem, fnd_rt_trace_stats* stats) {
    if (!stats) return FND_ERR_INVALID_ARG;
    return TraceImpl(ctx, scene, rays, n, out, mem, false, stats);
}

}  // extern "C"

extern "C" {

int fnd_rt_host_alloc(size_t bytes, void** out_ptr) {
    if (!out_ptr) return FND_ERR_INVALID_ARG;
    *out_ptr = nullptr;
    const cudaError_t e = cudaMallocHost(out_ptr, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        GlobalError() = cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FND_ERR_OUT_OF_MEMORY : FND_ERR_CUDA;
    }
    return FND_OK;
}

int fnd_rt_host_free(void* ptr) {
    if (!ptr) return FND_OK;
    return cudaFreeHost(ptr) == cudaSuccess ? FND_OK : FND_ERR_CUDA;
}

}  // extern "C"
