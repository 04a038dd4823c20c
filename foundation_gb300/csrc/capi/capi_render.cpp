// capi_render.cpp — C ABI of the path tracer: materials, lights and the
// per-frame render call (the counterpart of Renderer::Draw,
// src/Renderer/Renderer.cpp:367-401, with a caller-owned output buffer in
// place of the swapchain).
//
// A call renders width*height*spp paths in waves of `capacity` paths. Each
// wave is a fixed kernel sequence on the context stream; queue lengths stay
// on the device, so the host never waits inside a frame.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../bvh/gpu_build.hpp"
#include "context.hpp"

using namespace Foundation;
using Foundation::CApi::Guard;
using Foundation::RtCore::Fail;

namespace {

// Paths in flight per wave: 33,554,432 (7.3 GB of path state). Every wave
// pays its bounces' launches and the latency of each bounce's last rays, so
// fewer, larger waves are faster: 1920x1080 x 64 spp takes 166.7 ms in waves
// of 2^22 paths, 150.6 ms at 2^23, 142.1 ms at 2^24 and 137.2 ms at 2^25.
// A render of fewer paths allocates only what it needs.
constexpr uint32_t kDefaultWave = 1u << 25;

size_t Align256(size_t x) { return (x + 255) & ~size_t(255); }

// Carves the path buffers out of one allocation.
void EnsurePathBuffers(fnd_rt_ctx* ctx, uint32_t capacity) {
    if (ctx->d_paths && ctx->paths.capacity >= capacity) return;
    if (ctx->d_paths) CUDA_CHECK(cudaFree(ctx->d_paths));
    ctx->d_paths = nullptr;
    ctx->paths = PT::PathBuffers{};
    const size_t c = capacity;
    const size_t sizes[] = {
        16 * c,      // rng
        16 * c,      // beta
        32 * c,      // ext_rays[0]
        32 * c,      // ext_rays[1]
        4 * c,       // ext_path[0]
        4 * c,       // ext_path[1]
        8 * c,       // hits
        2 * 32 * c,  // sh_rays (two per path)
        2 * 4 * c,   // sh_pixel
        2 * 16 * c,  // sh_contrib
        2 * c,       // sh_occluded
        256,         // counts
    };
    size_t total = 0;
    for (size_t s : sizes) total += Align256(s);
    char* base = nullptr;
    CUDA_CHECK(cudaMalloc(&base, total));
    ctx->d_paths = base;
    ctx->paths_bytes = total;
    char* p = base;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += Align256(bytes);
        return r;
    };
    PT::PathBuffers& B = ctx->paths;
    B.capacity = capacity;
    B.rng = reinterpret_cast<uint4*>(take(sizes[0]));
    B.beta = reinterpret_cast<float4*>(take(sizes[1]));
    B.ext_rays[0] = reinterpret_cast<float4*>(take(sizes[2]));
    B.ext_rays[1] = reinterpret_cast<float4*>(take(sizes[3]));
    B.ext_path[0] = reinterpret_cast<uint32_t*>(take(sizes[4]));
    B.ext_path[1] = reinterpret_cast<uint32_t*>(take(sizes[5]));
    B.hits = reinterpret_cast<uint2*>(take(sizes[6]));
    B.sh_rays = reinterpret_cast<float4*>(take(sizes[7]));
    B.sh_pixel = reinterpret_cast<uint32_t*>(take(sizes[8]));
    B.sh_contrib = reinterpret_cast<float4*>(take(sizes[9]));
    B.sh_occluded = reinterpret_cast<uint8_t*>(take(sizes[10]));
    B.counts = reinterpret_cast<uint32_t*>(take(sizes[11]));
    CUDA_CHECK(cudaMemsetAsync(B.counts, 0, 256, ctx->stream));
}

void Sub(const double a[3], const double b[3], double o[3]) {
    for (int i = 0; i < 3; ++i) o[i] = a[i] - b[i];
}
void Cross(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
bool Normalize(double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (!(l > 0.0) || !std::isfinite(l)) return false;
    for (int i = 0; i < 3; ++i) v[i] /= l;
    return true;
}

// One wave's bounce loop: extend -> shade -> shadow -> resolve, max_depth
// times. After each bounce but the last, the tail megakernel finishes the
// wave when at most `tail_paths` paths continue (tail_paths 0: never).
void RunBounces(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const PT::PathBuffers& B, const PT::RenderParams& R,
                const PT::ShadeScene& S, const PT::CacheIO& C, uint32_t max_depth, int grid_shade,
                uint32_t tail_paths) {
    const int g_closest = CApi::TraceGrid(ctx, ctx->trace_cfg, 0);
    const int g_any = CApi::TraceGrid(ctx, ctx->trace_cfg, 1);
    const bool two = scene->two_level;
    int& tail_occ = ctx->tail_blocks_per_sm[two ? 1 : 0];
    if (tail_paths && tail_occ == 0) tail_occ = PT::TailBlocksPerSm(two);
    const int g_tail = ctx->sm_count * std::max(1, tail_occ);
    RT::TraceConfig cfg0 = ctx->trace_cfg;
    cfg0.sort_bits = 0;
    // cache paths end in queries at the second interaction: what continues
    // after it are specular chains, which the tail megakernel finishes
    // whatever their number, so the later bounces are not enqueued at all
    // (they would find empty queues)
    const bool cache_tail = C.mode == 1 && tail_paths != 0;
    // two-level scenes: the instanced persistent kernel on the device queues
    auto trace = [&](RT::TraceLaunch& L, bool any, const RT::TraceConfig& cfg, int grid) -> cudaError_t {
        if (!two) return CApi::LaunchTraceOrdered(ctx, scene, L, any, false, cfg, grid);
        if (scene->num_instances == 0) {
            RT::TraceLaunch E = L;
            E.scene = RT::DeviceScene{};
            return RT::LaunchTraceConfigured(E, any, false, cfg, 1, ctx->stream);
        }
        RT::InstancedLaunch I{};
        I.tlas = scene->view;
        I.inst = static_cast<const RT::InstanceRec*>(scene->d_instances);
        I.num_inst = scene->num_instances;
        I.rays = L.rays;
        I.n = L.n;
        I.n_dev = L.n_dev;
        I.ray_total = L.ray_total;
        I.hits = L.hits;
        I.occluded = L.occluded;
        I.counter = L.counter;
        I.status = L.status;
        return RT::LaunchInstanced(I, any, ctx->sm_count, ctx->stream);
    };
    for (uint32_t b = 0; b < max_depth; ++b) {
        const int cur = (int)(b & 1u), nxt = cur ^ 1;
        RT::TraceLaunch L{};
        L.scene = scene->view;
        L.rays = B.ext_rays[cur];
        L.n = B.capacity;
        L.n_dev = B.counts + cur;
        L.ray_total = ctx->d_render_stats + 0;
        L.hits = B.hits;
        L.counter = ctx->d_counter;
        L.status = ctx->d_status;
        L.refill_min = ctx->refill_min;
        // camera rays keep their (already coherent) order; later bounces and
        // shadow rays take the context's coherence ordering, if any
        CUDA_CHECK(trace(L, false, b == 0 ? cfg0 : ctx->trace_cfg, g_closest));
        CUDA_CHECK(cudaMemsetAsync(B.counts + nxt, 0, sizeof(uint32_t), ctx->stream));
        CUDA_CHECK(cudaMemsetAsync(B.counts + PT::kCountShadow, 0, sizeof(uint32_t), ctx->stream));
        CUDA_CHECK(PT::LaunchShade(B, R, S, C, cur, b, grid_shade, ctx->stream));
        RT::TraceLaunch A{};
        A.scene = scene->view;
        A.rays = B.sh_rays;
        A.n = 2 * B.capacity;
        A.n_dev = B.counts + PT::kCountShadow;
        A.ray_total = ctx->d_render_stats + 1;
        A.occluded = B.sh_occluded;
        A.counter = ctx->d_counter;
        A.status = ctx->d_status;
        A.refill_min = ctx->refill_min;
        CUDA_CHECK(trace(A, true, ctx->trace_cfg, g_any));
        CUDA_CHECK(PT::LaunchResolve(B, grid_shade, ctx->stream));
        if (tail_paths && b + 1 < max_depth) {
            PT::TailArgs T{};
            T.scene = scene->view;
            T.inst = two && scene->num_instances ? static_cast<const RT::InstanceRec*>(scene->d_instances) : nullptr;
            T.num_inst = scene->num_instances;
            T.B = B;
            T.R = R;
            T.S = S;
            T.C = C;
            T.q = nxt;
            T.bounce = b + 1;
            T.threshold = cache_tail && b == 1 ? 0xFFFFFFFFu : tail_paths;
            T.status = ctx->d_status;
            T.ray_stats = ctx->d_render_stats;
            CUDA_CHECK(PT::LaunchTail(T, g_tail, ctx->stream));
            if (cache_tail && b == 1) break;
        }
    }
}

uint32_t Mix32(uint64_t a, uint64_t b) {
    uint64_t x = a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull);
    x ^= x >> 31;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 29;
    return (uint32_t)x;
}

}  // namespace

extern "C" {

int fnd_rt_scene_set_materials(fnd_rt_scene* scene, const uint32_t* tri_material, uint32_t nt,
                               const fnd_material* materials, uint32_t nm) {
    if (!scene) return FND_ERR_INVALID_ARG;
    fnd_rt_ctx* ctx = scene->ctx;
    return Guard(ctx, [&] {
        CHECK_CODE(nt == scene->info.num_tris, FND_ERR_INVALID_ARG, "%u material ids for %u triangles", nt,
                   scene->info.num_tris);
        CHECK(nm >= 1 && materials != nullptr && (nt == 0 || tri_material != nullptr));
        std::vector<PT::DevMaterial> dm(nm);
        for (uint32_t i = 0; i < nm; ++i) {
            const fnd_material& m = materials[i];
            CHECK_CODE(m.type <= FND_MAT_EMISSIVE, FND_ERR_INVALID_ARG, "material %u has unknown type %u", i, m.type);
            for (int c = 0; c < 3; ++c)
                CHECK_CODE(std::isfinite(m.albedo[c]) && std::isfinite(m.emission[c]) && m.emission[c] >= 0.0f,
                           FND_ERR_INVALID_ARG, "material %u has a non-finite or negative value", i);
            CHECK_CODE(m.type != FND_MAT_GGX || (m.roughness > 0.0f && m.roughness <= 1.0f), FND_ERR_INVALID_ARG,
                       "GGX material %u needs roughness in (0, 1]", i);
            uint32_t tb = m.type;
            int32_t lb = m.light;
            std::memcpy(&dm[i].albedo_type.w, &tb, 4);
            dm[i].albedo_type.x = m.albedo[0];
            dm[i].albedo_type.y = m.albedo[1];
            dm[i].albedo_type.z = m.albedo[2];
            dm[i].emission_light = make_float4(m.emission[0], m.emission[1], m.emission[2], 0.0f);
            std::memcpy(&dm[i].emission_light.w, &lb, 4);
            dm[i].params = make_float4(m.roughness, 0.f, 0.f, 0.f);
        }
        for (uint32_t t = 0; t < nt; ++t)
            CHECK_CODE(tri_material[t] < nm, FND_ERR_INVALID_ARG, "triangle %u uses material %u of %u", t,
                       tri_material[t], nm);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        if (nt) {
            // material ids into the w of the device shading records
            void* d_ids = nullptr;
            CUDA_CHECK(cudaMalloc(&d_ids, 4ull * nt));
            cudaError_t e = cudaMemcpyAsync(d_ids, tri_material, 4ull * nt, cudaMemcpyHostToDevice, ctx->stream);
            if (e == cudaSuccess)
                e = RT::WriteMaterialIds(static_cast<float4*>(scene->d_tri_shade), static_cast<const uint32_t*>(d_ids),
                                         nt, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            cudaFree(d_ids);
            CUDA_CHECK(e);
        }
        if (scene->d_materials) CUDA_CHECK(cudaFree(scene->d_materials));
        scene->d_materials = nullptr;
        scene->num_materials = 0;
        CUDA_CHECK(cudaMalloc(&scene->d_materials, sizeof(PT::DevMaterial) * nm));
        CUDA_CHECK(cudaMemcpy(scene->d_materials, dm.data(), sizeof(PT::DevMaterial) * nm, cudaMemcpyHostToDevice));
        scene->num_materials = nm;
    });
}

int fnd_rt_scene_set_lights(fnd_rt_scene* scene, const fnd_quad_light* lights, uint32_t nl) {
    if (!scene) return FND_ERR_INVALID_ARG;
    fnd_rt_ctx* ctx = scene->ctx;
    return Guard(ctx, [&] {
        CHECK(nl == 0 || lights != nullptr);
        std::vector<PT::DevQuadLight> dl(nl);
        for (uint32_t i = 0; i < nl; ++i) {
            const fnd_quad_light& q = lights[i];
            double eu[3] = {q.edge_u[0], q.edge_u[1], q.edge_u[2]}, ev[3] = {q.edge_v[0], q.edge_v[1], q.edge_v[2]};
            double n[3];
            Cross(eu, ev, n);
            const double area = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            CHECK_CODE(area > 0.0 && std::isfinite(area), FND_ERR_INVALID_ARG, "light %u has zero area", i);
            for (int c = 0; c < 3; ++c) n[c] /= area;
            dl[i].corner_area = make_float4(q.corner[0], q.corner[1], q.corner[2], (float)area);
            dl[i].eu = make_float4(q.edge_u[0], q.edge_u[1], q.edge_u[2], 0.f);
            dl[i].ev = make_float4(q.edge_v[0], q.edge_v[1], q.edge_v[2], 0.f);
            dl[i].normal = make_float4((float)n[0], (float)n[1], (float)n[2], 0.f);
            dl[i].radiance = make_float4(q.radiance[0], q.radiance[1], q.radiance[2], 0.f);
        }
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        if (scene->d_lights) CUDA_CHECK(cudaFree(scene->d_lights));
        scene->d_lights = nullptr;
        scene->num_lights = 0;
        if (nl) {
            CUDA_CHECK(cudaMalloc(&scene->d_lights, sizeof(PT::DevQuadLight) * nl));
            CUDA_CHECK(cudaMemcpy(scene->d_lights, dl.data(), sizeof(PT::DevQuadLight) * nl, cudaMemcpyHostToDevice));
        }
        scene->num_lights = nl;
    });
}

int fnd_rt_render(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_render_desc* desc, float* rgb, int mem) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(scene != nullptr && scene->ctx == ctx && desc != nullptr);
        CHECK(mem == FND_MEM_HOST || mem == FND_MEM_DEVICE);
        const fnd_render_desc& D = *desc;
        const bool train_only = (D.flags & FND_RENDER_TRAIN_ONLY) != 0;
        CHECK_CODE(rgb != nullptr || train_only, FND_ERR_INVALID_ARG, "rgb is NULL");
        CHECK_CODE(!train_only || (D.flags & FND_RENDER_CACHE), FND_ERR_INVALID_ARG,
                   "FND_RENDER_TRAIN_ONLY needs FND_RENDER_CACHE");
        CHECK_CODE(D.width > 0 && D.height > 0 && (uint64_t)D.width * D.height <= (1ull << 26), FND_ERR_INVALID_ARG,
                   "image %ux%u out of range", D.width, D.height);
        CHECK_CODE(D.spp >= 1 && D.max_depth >= 1 && D.max_depth <= 64, FND_ERR_INVALID_ARG,
                   "spp %u / max_depth %u out of range", D.spp, D.max_depth);
        CHECK_CODE(D.camera.vfov_deg > 0.0f && D.camera.vfov_deg < 180.0f, FND_ERR_INVALID_ARG, "vfov %f",
                   D.camera.vfov_deg);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const uint32_t npix = D.width * D.height;
        const uint64_t total = (uint64_t)npix * D.spp;
        uint32_t cap = D.wave_paths ? D.wave_paths : kDefaultWave;
        if (cap > total) cap = (uint32_t)total;
        CHECK_CODE(cap >= 1 && cap <= (1u << 28), FND_ERR_INVALID_ARG, "wave_paths %u out of range", cap);
        const bool use_cache = (D.flags & FND_RENDER_CACHE) != 0;
        CHECK_CODE(!use_cache || ctx->cache != nullptr, FND_ERR_INVALID_ARG,
                   "FND_RENDER_CACHE needs a cache (fnd_rt_cache_create)");
        const uint32_t train_paths = use_cache ? ctx->cache->desc.train_paths : 0u;
        if (!train_only) EnsurePathBuffers(ctx, cap);
        if (use_cache) CApi::EnsureCacheBuffers(ctx, cap, D.max_depth);
        // frame buffer (restart unless accumulating into a frame of the same size)
        const bool keep_fb = train_only;
        const bool accumulate = (D.flags & FND_RENDER_ACCUMULATE) && ctx->d_fb && ctx->fb_width == D.width &&
                                ctx->fb_height == D.height;
        if (!keep_fb && ctx->fb_pixels < npix) {
            if (ctx->d_fb) CUDA_CHECK(cudaFree(ctx->d_fb));
            ctx->d_fb = nullptr;
            ctx->fb_pixels = 0;
            CUDA_CHECK(cudaMalloc(&ctx->d_fb, sizeof(float4) * (size_t)npix));
            ctx->fb_pixels = npix;
        }
        if (!keep_fb) {
            if (!accumulate) {
                CUDA_CHECK(cudaMemsetAsync(ctx->d_fb, 0, sizeof(float4) * (size_t)npix, ctx->stream));
                ctx->fb_samples = 0;
            }
            ctx->fb_width = D.width;
            ctx->fb_height = D.height;
            ctx->paths.fb = ctx->d_fb;
        }
        // camera basis (lookAt convention)
        double eye[3] = {D.camera.eye[0], D.camera.eye[1], D.camera.eye[2]};
        double tgt[3] = {D.camera.target[0], D.camera.target[1], D.camera.target[2]};
        double up[3] = {D.camera.up[0], D.camera.up[1], D.camera.up[2]};
        double fwd[3], right[3], u[3];
        Sub(tgt, eye, fwd);
        CHECK_CODE(Normalize(fwd), FND_ERR_INVALID_ARG, "camera eye equals target");
        Cross(fwd, up, right);
        CHECK_CODE(Normalize(right), FND_ERR_INVALID_ARG, "camera up is parallel to the view direction");
        Cross(right, fwd, u);
        PT::RenderParams R{};
        R.width = D.width;
        R.height = D.height;
        R.spp = D.spp;
        R.max_depth = D.max_depth;
        R.rr_start = D.rr_start;
        R.sample_offset = ctx->fb_samples;
        R.seed = D.seed;
        for (int i = 0; i < 3; ++i) {
            R.eye[i] = (float)eye[i];
            R.fwd[i] = (float)fwd[i];
            R.right[i] = (float)right[i];
            R.up[i] = (float)u[i];
            R.sky[i] = D.sky[i];
            R.sun_E[i] = D.sun_irradiance[i];
        }
        R.tan_half = (float)std::tan((double)D.camera.vfov_deg * 3.14159265358979323846 / 360.0);
        R.aspect = (float)D.width / (float)D.height;
        double sd[3] = {D.sun_dir[0], D.sun_dir[1], D.sun_dir[2]};
        R.has_sun = Normalize(sd) && (D.sun_irradiance[0] > 0 || D.sun_irradiance[1] > 0 || D.sun_irradiance[2] > 0);
        for (int i = 0; i < 3; ++i) R.sun_dir[i] = (float)sd[i];
        R.eps = 1e-4f;
        PT::ShadeScene S{};
        S.tri_shade = static_cast<const float4*>(scene->d_tri_shade);
        S.materials = static_cast<const PT::DevMaterial*>(scene->d_materials);
        S.lights = static_cast<const PT::DevQuadLight*>(scene->d_lights);
        S.num_lights = scene->num_lights;
        S.num_materials = scene->num_materials;
        CHECK_CODE(scene->info.num_tris == 0 || S.tri_shade != nullptr, FND_ERR_INVALID_SCENE, "scene has no shading data");
        PT::PathBuffers& B = ctx->paths;
        const int grid_shade = std::max(1, std::min<int>((int)((cap + 255) / 256), ctx->sm_count * 8));
        CUDA_CHECK(cudaMemsetAsync(ctx->d_render_stats, 0, 2 * sizeof(unsigned long long), ctx->stream));
        // tail megakernel threshold: by default two paths per resident tail thread
        int& tail_occ = ctx->tail_blocks_per_sm[scene->two_level ? 1 : 0];
        if (tail_occ == 0) tail_occ = PT::TailBlocksPerSm(scene->two_level);
        const uint32_t tail_paths =
            (D.flags & FND_RENDER_WAVEFRONT)
                ? 0u
                : (D.tail_paths ? D.tail_paths : 2u * (uint32_t)ctx->sm_count * (uint32_t)tail_occ * PT::kTailBlock);
        PT::CacheIO C{};
        if (use_cache) {
            // 1) training, on the cache's own stream so it overlaps the render
            //    wave: full training paths through random pixels (one thread
            //    each, one sample + target per vertex), then the optimiser
            //    steps. The render wave's cache queries wait for it (event).
            FndCacheState& cs = *ctx->cache;
            const fnd_cache_desc& cd = cs.desc;
            cudaStream_t ts = cs.train_stream;
            CUDA_CHECK(cudaEventRecord(cs.ev_start, ctx->stream));
            CUDA_CHECK(cudaStreamWaitEvent(ts, cs.ev_start, 0));
            CUDA_CHECK(cudaMemsetAsync(cs.counters + 1, 0, sizeof(uint32_t), ts));
            PT::TrainPathsArgs T{};
            T.scene = scene->view;
            T.inst = scene->two_level && scene->num_instances
                         ? static_cast<const RT::InstanceRec*>(scene->d_instances)
                         : nullptr;
            T.num_inst = scene->num_instances;
            T.R = R;
            T.S = S;
            T.n = train_paths;
            const uint32_t tseed = Mix32(cd.seed ^ D.seed, cs.frames);
            T.seed = tseed;
            T.samples = cs.samples;
            T.targets = cs.targets;
            T.sample_count = cs.counters + 1;
            T.sample_cap = cs.sample_cap;
            T.status = ctx->d_status;
            T.fetch = cs.counters + 2;
            int& occ = ctx->train_paths_blocks_per_sm[scene->two_level ? 1 : 0];
            if (occ == 0) occ = PT::TrainingPathsBlocksPerSm(scene->two_level);
            CUDA_CHECK(PT::LaunchTrainingPaths(T, ctx->sm_count * occ, ts));
            for (uint32_t st = 0; st < cd.train_steps; ++st)
                CUDA_CHECK(NRC::TrainStep(cs.net, cs.samples, cs.targets, cs.counters + 1, cd.batch,
                                          Mix32(tseed, st + 1), cd.learning_rate, ctx->d_status, ts));
            CUDA_CHECK(cudaEventRecord(cs.ev_trained, ts));
            cs.frames++;
            if (train_only) {
                // later work on the context stream sees the trained network
                CUDA_CHECK(cudaStreamWaitEvent(ctx->stream, cs.ev_trained, 0));
                ctx->last_render = fnd_render_stats{};
                ctx->last_render.samples_accumulated = ctx->fb_samples;
                return;
            }
            // 2) render waves end their paths in cache queries
            C.mode = 1;
            C.specular_alpha = cd.specular_alpha;
            C.queries = cs.queries;
            C.query_count = cs.counters + 0;
            C.query_cap = cs.query_cap;
        }
        uint32_t waves = 0;
        for (uint64_t wave_base = 0; wave_base < total; wave_base += cap, ++waves) {
            const uint32_t wave_n = (uint32_t)std::min<uint64_t>(cap, total - wave_base);
            if (use_cache) CUDA_CHECK(cudaMemsetAsync(C.query_count, 0, sizeof(uint32_t), ctx->stream));
            CUDA_CHECK(PT::LaunchGenerate(B, R, wave_base, wave_n, ctx->stream));
            RunBounces(ctx, scene, B, R, S, C, D.max_depth, grid_shade, tail_paths);
            if (use_cache) {
                CUDA_CHECK(cudaStreamWaitEvent(ctx->stream, ctx->cache->ev_trained, 0));
                CUDA_CHECK(NRC::Infer(ctx->cache->net, C.queries, C.query_count, C.query_cap, B.fb,
                                      ctx->sm_count * 2, ctx->stream));
            }
        }
        ctx->fb_samples += D.spp;
        const float scale = 1.0f / (float)ctx->fb_samples;
        float* target = rgb;
        if (mem == FND_MEM_HOST) {
            const size_t bytes = sizeof(float) * 3 * (size_t)npix;
            if (ctx->rgb_cap < bytes) {
                if (ctx->d_rgb) CUDA_CHECK(cudaFree(ctx->d_rgb));
                ctx->d_rgb = nullptr;
                ctx->rgb_cap = 0;
                CUDA_CHECK(cudaMalloc(&ctx->d_rgb, bytes));
                ctx->rgb_cap = bytes;
            }
            target = ctx->d_rgb;
        }
        CUDA_CHECK(PT::LaunchFinalize(B, target, npix, scale, ctx->stream));
        ctx->last_render = fnd_render_stats{};
        ctx->last_render.paths = total;
        ctx->last_render.waves = waves;
        ctx->last_render.samples_accumulated = ctx->fb_samples;
        if (mem == FND_MEM_HOST) {
            CUDA_CHECK(cudaMemcpyAsync(rgb, ctx->d_rgb, sizeof(float) * 3 * (size_t)npix, cudaMemcpyDeviceToHost,
                                       ctx->stream));
            const int s = CApi::ReadStatus(ctx);
            if (s != FND_OK) Fail(s, "device status after render: %d", s);
        }
    });
}

int fnd_rt_tonemap(fnd_rt_ctx* ctx, const float* rgb, uint32_t width, uint32_t height, int mem_in, float exposure,
                   uint32_t mode, uint8_t* rgba, int mem_out) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(rgb != nullptr && rgba != nullptr);
        CHECK((mem_in == FND_MEM_HOST || mem_in == FND_MEM_DEVICE) && (mem_out == FND_MEM_HOST || mem_out == FND_MEM_DEVICE));
        CHECK_CODE(mode <= FND_TONEMAP_ACES, FND_ERR_INVALID_ARG, "tonemap mode %u", mode);
        CHECK_CODE(std::isfinite(exposure) && exposure >= 0.0f, FND_ERR_INVALID_ARG, "exposure %g", (double)exposure);
        CHECK_CODE((uint64_t)width * height <= (1ull << 28), FND_ERR_INVALID_ARG, "image %ux%u", width, height);
        const uint32_t npix = width * height;
        if (npix == 0) return;
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CHECK_CODE(mem_out == FND_MEM_HOST || ((uintptr_t)rgba & 3u) == 0, FND_ERR_INVALID_ARG,
                   "device rgba must be 4-byte aligned");
        const float* src = rgb;
        if (mem_in == FND_MEM_HOST) {
            CApi::EnsureDevice(ctx->d_in, ctx->d_in_cap, 12ull * npix);
            CUDA_CHECK(cudaMemcpyAsync(ctx->d_in, rgb, 12ull * npix, cudaMemcpyHostToDevice, ctx->stream));
            src = static_cast<const float*>(ctx->d_in);
        }
        uint32_t* dst = reinterpret_cast<uint32_t*>(rgba);
        if (mem_out == FND_MEM_HOST) {
            CApi::EnsureDevice(ctx->d_out, ctx->d_out_cap, 4ull * npix);
            dst = static_cast<uint32_t*>(ctx->d_out);
        }
        CUDA_CHECK(PT::LaunchTonemap(src, npix, exposure, mode, dst, ctx->stream));
        if (mem_out == FND_MEM_HOST) {
            CUDA_CHECK(cudaMemcpyAsync(rgba, dst, 4ull * npix, cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        }
    });
}

int fnd_rt_render_stats_get(fnd_rt_ctx* ctx, fnd_render_stats* out) {
    if (!ctx || !out) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CUDA_CHECK(cudaSetDevice(ctx->device));
        unsigned long long h[2] = {0, 0};
        CUDA_CHECK(cudaMemcpyAsync(h, ctx->d_render_stats, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        *out = ctx->last_render;
        out->extension_rays = h[0];
        out->shadow_rays = h[1];
    });
}

}  // extern "C"
