// capi_cache.cpp — C ABI of the radiance cache: session create / destroy,
// weights, checkpoints, and the test hooks that run the network kernels on
// explicit features (forward, gradient, Adam).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "context.hpp"

using namespace Foundation;
using Foundation::CApi::Guard;
using Foundation::RtCore::Fail;

namespace Foundation {
namespace CApi {

size_t Align256(size_t x) { return (x + 255) & ~size_t(255); }

void FreeCache(fnd_rt_ctx* ctx) {
    if (!ctx->cache) return;
    if (ctx->cache->train_stream) cudaStreamSynchronize(ctx->cache->train_stream);
    if (ctx->cache->ev_start) cudaEventDestroy(ctx->cache->ev_start);
    if (ctx->cache->ev_trained) cudaEventDestroy(ctx->cache->ev_trained);
    if (ctx->cache->train_stream) cudaStreamDestroy(ctx->cache->train_stream);
    if (ctx->cache->d_block) cudaFree(ctx->cache->d_block);
    delete ctx->cache;
    ctx->cache = nullptr;
}

// Grows the training / query buffers of the cache for `query_cap` queries.
void EnsureCacheBuffers(fnd_rt_ctx* ctx, uint32_t query_cap, uint32_t max_depth) {
    FndCacheState& c = *ctx->cache;
    const uint32_t train = c.desc.train_paths;
    const uint32_t samples = train * std::min(max_depth, 16u);
    if (c.d_block && c.query_cap >= query_cap && c.sample_cap >= samples && c.train_cap >= train) return;
    const uint32_t qcap = std::max(query_cap, c.query_cap), scap = std::max(samples, c.sample_cap);
    const size_t P = NRC::kNumParams;
    const size_t sizes[] = {
        sizeof(uint16_t) * NRC::kFwdElems, sizeof(uint16_t) * NRC::kUFwdElems,
        4 * P, 4 * P, 4 * P, 4 * P,            // master, m, v, grad
        sizeof(double) * 4,                    // loss
        sizeof(NRC::TrainSample) * scap, sizeof(float4) * scap, sizeof(NRC::CachePoint) * qcap, 256,
        sizeof(uint16_t) * NRC::kFwdElems, 4 * P,  // weight average: query image, fp32 average
        sizeof(uint16_t) * NRC::kUBwdElems,        // tcgen05 backward images
    };
    size_t total = 0;
    for (size_t sz : sizes) total += Align256(sz);
    char* base = nullptr;
    CUDA_CHECK(cudaMalloc(&base, total));
    char* p = base;
    auto take = [&](size_t b) {
        char* r = p;
        p += Align256(b);
        return r;
    };
    NRC::Net net = c.net;
    net.fwd = reinterpret_cast<uint16_t*>(take(sizes[0]));
    net.ufwd = reinterpret_cast<uint16_t*>(take(sizes[1]));
    net.master = reinterpret_cast<float*>(take(sizes[2]));
    net.adam_m = reinterpret_cast<float*>(take(sizes[3]));
    net.adam_v = reinterpret_cast<float*>(take(sizes[4]));
    net.grad = reinterpret_cast<float*>(take(sizes[5]));
    net.loss = reinterpret_cast<double*>(take(sizes[6]));
    const bool averaging = c.desc.weight_average > 0.0f;
    net.fwd_avg = averaging ? reinterpret_cast<uint16_t*>(take(sizes[11])) : nullptr;
    net.avg = averaging ? reinterpret_cast<float*>(take(sizes[12])) : nullptr;
    net.avg_decay = c.desc.weight_average;
    net.ubwd = reinterpret_cast<uint16_t*>(take(sizes[13]));
    if (c.d_block) {
        if (c.train_stream) CUDA_CHECK(cudaStreamSynchronize(c.train_stream));
        // keep the trained state: copy the network, moments and images across
        CUDA_CHECK(cudaMemcpyAsync(net.fwd, c.net.fwd, sizes[0], cudaMemcpyDeviceToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(net.ufwd, c.net.ufwd, sizes[1], cudaMemcpyDeviceToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(net.ubwd, c.net.ubwd, sizes[13], cudaMemcpyDeviceToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(net.master, c.net.master, 4 * P, cudaMemcpyDeviceToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(net.adam_m, c.net.adam_m, 4 * P, cudaMemcpyDeviceToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(net.adam_v, c.net.adam_v, 4 * P, cudaMemcpyDeviceToDevice, ctx->stream));
        CUDA_CHECK(cudaMemsetAsync(net.grad, 0, 4 * P, ctx->stream));
        if (averaging) {
            CUDA_CHECK(cudaMemcpyAsync(net.fwd_avg, c.net.fwd_avg, sizes[11], cudaMemcpyDeviceToDevice, ctx->stream));
            CUDA_CHECK(cudaMemcpyAsync(net.avg, c.net.avg, 4 * P, cudaMemcpyDeviceToDevice, ctx->stream));
        }
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        CUDA_CHECK(cudaFree(c.d_block));
    }
    c.net = net;
    c.samples = reinterpret_cast<NRC::TrainSample*>(take(sizes[7]));
    c.targets = reinterpret_cast<float4*>(take(sizes[8]));
    c.queries = reinterpret_cast<NRC::CachePoint*>(take(sizes[9]));
    c.counters = reinterpret_cast<uint32_t*>(take(sizes[10]));
    c.d_block = base;
    c.block_bytes = total;
    c.query_cap = qcap;
    c.sample_cap = scap;
    c.train_cap = train;
    CUDA_CHECK(cudaMemsetAsync(c.counters, 0, 256, ctx->stream));
}

}  // namespace CApi
}  // namespace Foundation

using namespace Foundation::CApi;

namespace {

FndCacheState& NeedCache(fnd_rt_ctx* ctx) {
    CHECK_CODE(ctx->cache != nullptr, FND_ERR_INVALID_ARG, "no radiance cache on this context (fnd_rt_cache_create)");
    return *ctx->cache;
}

constexpr char kMagic[8] = {'F', 'N', 'D', 'N', 'R', 'C', '0', '1'};

}  // namespace

extern "C" {

int fnd_rt_cache_create(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_cache_desc* desc) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(scene != nullptr && scene->ctx == ctx && desc != nullptr);
        CHECK_CODE(desc->train_paths >= 1 && desc->train_paths <= (1u << 24), FND_ERR_INVALID_ARG,
                   "train_paths %u out of range", desc->train_paths);
        CHECK_CODE(desc->batch >= 1 && desc->batch <= (1u << 24) && desc->train_steps <= 1024, FND_ERR_INVALID_ARG,
                   "batch / train_steps out of range");
        CHECK_CODE(desc->learning_rate > 0.0f && desc->learning_rate < 1.0f, FND_ERR_INVALID_ARG,
                   "learning rate %g out of range", desc->learning_rate);
        CHECK_CODE(desc->weight_average >= 0.0f && desc->weight_average < 1.0f, FND_ERR_INVALID_ARG,
                   "weight_average %g not in [0, 1)", desc->weight_average);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        FreeCache(ctx);
        ctx->cache = new FndCacheState();
        ctx->cache->desc = *desc;
        for (int a = 0; a < 3; ++a) {
            // the encoding box: the scene bounds, slightly enlarged
            const float lo = scene->info.bounds_lo[a], hi = scene->info.bounds_hi[a];
            const float pad = 1e-3f * (hi - lo) + 1e-6f;
            ctx->cache->net.lo[a] = lo - pad;
            ctx->cache->net.hi[a] = hi + pad;
        }
        try {
            // the highest priority: the training kernels take SMs at the render
            // wave's kernel boundaries instead of waiting for the wave to end
            int lo_prio = 0, hi_prio = 0;
            CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
            CUDA_CHECK(cudaStreamCreateWithPriority(&ctx->cache->train_stream, cudaStreamNonBlocking, hi_prio));
            CUDA_CHECK(cudaEventCreateWithFlags(&ctx->cache->ev_start, cudaEventDisableTiming));
            CUDA_CHECK(cudaEventCreateWithFlags(&ctx->cache->ev_trained, cudaEventDisableTiming));
            EnsureCacheBuffers(ctx, 1024, 8);
            CUDA_CHECK(NRC::InitNet(ctx->cache->net, desc->seed, ctx->stream));
            CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            FreeCache(ctx);
            throw;
        }
    });
}

int fnd_rt_cache_destroy(fnd_rt_ctx* ctx) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        FreeCache(ctx);
    });
}

int fnd_rt_cache_stats_get(fnd_rt_ctx* ctx, fnd_cache_stats* out) {
    if (!ctx || !out) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        double loss = 0.0;
        uint32_t counters[2] = {0, 0};
        CUDA_CHECK(cudaMemcpyAsync(&loss, c.net.loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(counters, c.counters, sizeof(counters), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        out->steps = c.net.step;
        out->samples_last = counters[1];
        out->queries_last = counters[0];
        out->loss_last = loss / (3.0 * (double)std::max<uint32_t>(1u, c.desc.batch));
    });
}

int fnd_rt_cache_get_weights(fnd_rt_ctx* ctx, float* out, uint32_t n) {
    if (!ctx || !out) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CHECK_CODE(n == (uint32_t)NRC::kNumParams, FND_ERR_INVALID_ARG, "%u weights, the network has %d", n,
                   NRC::kNumParams);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaMemcpyAsync(out, c.net.master, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int fnd_rt_cache_set_weights(fnd_rt_ctx* ctx, const float* w, uint32_t n) {
    if (!ctx || !w) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CHECK_CODE(n == (uint32_t)NRC::kNumParams, FND_ERR_INVALID_ARG, "%u weights, the network has %d", n,
                   NRC::kNumParams);
        for (uint32_t i = 0; i < n; ++i) CHECK_CODE(std::isfinite(w[i]), FND_ERR_INVALID_ARG, "weight %u not finite", i);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaMemcpyAsync(c.net.master, w, 4ull * n, cudaMemcpyHostToDevice, ctx->stream));
        c.net.avg_steps = 0;
        CUDA_CHECK(NRC::RewriteImages(c.net, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int fnd_rt_cache_save(fnd_rt_ctx* ctx, const char* path) {
    if (!ctx || !path) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        const size_t P = NRC::kNumParams;
        std::vector<float> buf(3 * P);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaMemcpyAsync(buf.data(), c.net.master, 4 * P, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(buf.data() + P, c.net.adam_m, 4 * P, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(buf.data() + 2 * P, c.net.adam_v, 4 * P, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        FILE* f = std::fopen(path, "wb");
        CHECK_CODE(f != nullptr, FND_ERR_IO, "cannot write %s", path);
        const uint32_t hdr[3] = {1u, (uint32_t)P, c.net.step};
        bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(hdr, 4, 3, f) == 3 &&
                  std::fwrite(c.net.lo, 4, 3, f) == 3 && std::fwrite(c.net.hi, 4, 3, f) == 3 &&
                  std::fwrite(buf.data(), 4, buf.size(), f) == buf.size();
        ok = (std::fclose(f) == 0) && ok;
        CHECK_CODE(ok, FND_ERR_IO, "write to %s failed", path);
    });
}

int fnd_rt_cache_load(fnd_rt_ctx* ctx, const char* path) {
    if (!ctx || !path) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        const size_t P = NRC::kNumParams;
        FILE* f = std::fopen(path, "rb");
        CHECK_CODE(f != nullptr, FND_ERR_IO, "cannot open %s", path);
        char magic[8];
        uint32_t hdr[3];
        float lo[3], hi[3];
        std::vector<float> buf(3 * P);
        bool ok = std::fread(magic, 1, 8, f) == 8 && std::fread(hdr, 4, 3, f) == 3 && std::fread(lo, 4, 3, f) == 3 &&
                  std::fread(hi, 4, 3, f) == 3 && std::fread(buf.data(), 4, buf.size(), f) == buf.size();
        std::fclose(f);
        CHECK_CODE(ok && std::memcmp(magic, kMagic, 8) == 0, FND_ERR_IO, "%s is not a cache checkpoint", path);
        CHECK_CODE(hdr[0] == 1u && hdr[1] == (uint32_t)P, FND_ERR_IO, "checkpoint version %u / %u params unsupported",
                   hdr[0], hdr[1]);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaMemcpyAsync(c.net.master, buf.data(), 4 * P, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(c.net.adam_m, buf.data() + P, 4 * P, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(c.net.adam_v, buf.data() + 2 * P, 4 * P, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemsetAsync(c.net.grad, 0, 4 * P, ctx->stream));
        c.net.step = hdr[2];
        for (int a = 0; a < 3; ++a) {
            c.net.lo[a] = lo[a];
            c.net.hi[a] = hi[a];
        }
        c.net.avg_steps = 0;
        CUDA_CHECK(NRC::RewriteImages(c.net, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int fnd_rt_cache_eval(fnd_rt_ctx* ctx, const float* features, uint32_t n, float* out) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CHECK(n == 0 || (features && out));
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const size_t in_b = 4ull * n * NRC::kIn, out_b = 4ull * n * 3;
        EnsureDevice(ctx->d_in, ctx->d_in_cap, in_b);
        EnsureDevice(ctx->d_out, ctx->d_out_cap, out_b);
        if (!n) return;
        CUDA_CHECK(cudaMemcpyAsync(ctx->d_in, features, in_b, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(NRC::InferRaw(c.net, static_cast<const float*>(ctx->d_in), n, static_cast<float*>(ctx->d_out),
                                 ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(out, ctx->d_out, out_b, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int fnd_rt_cache_gradient(fnd_rt_ctx* ctx, const float* features, const float* targets, uint32_t n, float* grad,
                          double* loss) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CHECK(n >= 1 && features && targets && grad);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const size_t in_b = 4ull * n * NRC::kIn, t_b = 4ull * n * 3;
        EnsureDevice(ctx->d_in, ctx->d_in_cap, in_b + t_b);
        char* d = static_cast<char*>(ctx->d_in);
        CUDA_CHECK(cudaMemcpyAsync(d, features, in_b, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(d + in_b, targets, t_b, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(NRC::GradRaw(c.net, reinterpret_cast<const float*>(d), reinterpret_cast<const float*>(d + in_b), n,
                                ctx->d_status, ctx->stream));
        double l = 0.0;
        CUDA_CHECK(cudaMemcpyAsync(grad, c.net.grad, 4ull * NRC::kNumParams, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(&l, c.net.loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        if (loss) *loss = l / (3.0 * n);
    });
}

int fnd_rt_cache_encode(fnd_rt_ctx* ctx, const float* points, uint32_t n, float* out) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CHECK(n == 0 || (points && out));
        if (!n) return;
        std::vector<NRC::CachePoint> pts(n);
        for (uint32_t i = 0; i < n; ++i) {
            const float* r = points + 13 * (size_t)i;
            pts[i].p_rough = make_float4(r[0], r[1], r[2], r[9]);
            pts[i].wo_aux = make_float4(r[3], r[4], r[5], 0.f);
            pts[i].n_pad = make_float4(r[6], r[7], r[8], 0.f);
            pts[i].albedo = make_float4(r[10], r[11], r[12], 0.f);
            pts[i].beta = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const size_t pb = sizeof(NRC::CachePoint) * n, ob = 4ull * n * NRC::kIn;
        EnsureDevice(ctx->d_in, ctx->d_in_cap, pb);
        EnsureDevice(ctx->d_out, ctx->d_out_cap, ob);
        CUDA_CHECK(cudaMemcpyAsync(ctx->d_in, pts.data(), pb, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(NRC::EncodeRaw(c.net, static_cast<const NRC::CachePoint*>(ctx->d_in), n,
                                  static_cast<float*>(ctx->d_out), ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(out, ctx->d_out, ob, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int fnd_rt_cache_adam_step(fnd_rt_ctx* ctx, const float* grad, float learning_rate) {
    if (!ctx || !grad) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        FndCacheState& c = NeedCache(ctx);
        CHECK(learning_rate > 0.0f);
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaMemcpyAsync(c.net.grad, grad, 4ull * NRC::kNumParams, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(NRC::AdamRaw(c.net, learning_rate, ctx->stream));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

}  // extern "C"
