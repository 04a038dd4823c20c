// capi_batch.cpp — C ABI of the launch-shape autotuner and of batched
// multi-scene traversal (one persistent launch over a job table, captured in
// a CUDA graph).
#include <algorithm>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "context.hpp"

using namespace Foundation;
using Foundation::CApi::Guard;

struct fnd_rt_batch {
    fnd_rt_ctx* ctx = nullptr;
    void* d_block = nullptr;  // job table, prefix sums, work counter
    RT::BatchLaunch launch{};
    RT::TraceConfig cfg{};
    bool use_graph = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace Foundation {
namespace CApi {

int TraceGrid(fnd_rt_ctx* ctx, const RT::TraceConfig& cfg, int variant) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, int>, int> cache;  // (device, block, short, variant) -> blocks/SM
    const auto key = std::make_tuple(ctx->device, cfg.block, cfg.short_stack, variant);
    int blocks = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) blocks = it->second;
    }
    if (!blocks) {
        CUDA_CHECK(RT::TraceOccupancyFor(cfg, variant, &blocks));
        blocks = std::max(1, blocks);
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = blocks;
    }
    if (cfg.blocks_per_sm > 0) blocks = std::min(blocks, cfg.blocks_per_sm);
    return ctx->sm_count * blocks;
}

}  // namespace CApi
}  // namespace Foundation

namespace {

std::vector<RT::TraceConfig> Candidates() {
    std::vector<RT::TraceConfig> out;
    for (int block : {64, 128, 256})
        for (int st : {4, 8, 16})
            for (uint32_t refill : {4u, 8u, 16u, 24u})
                for (uint32_t postpone : {0u, 8u}) {
                    RT::TraceConfig c;
                    c.block = block;
                    c.short_stack = st;
                    c.refill_min = refill;
                    c.postpone_min = postpone;
                    out.push_back(c);
                }
    return out;
}

fnd_rt_trace_config ToAbi(const RT::TraceConfig& c) {
    return fnd_rt_trace_config{(uint32_t)c.block, (uint32_t)c.short_stack, c.refill_min, c.postpone_min,
                               c.sort_bits};
}

RT::TraceConfig FromAbi(const fnd_rt_trace_config& a) {
    RT::TraceConfig c;
    c.block = (int)a.block;
    c.short_stack = (int)a.short_stack;
    c.refill_min = a.refill_min;
    c.postpone_min = a.postpone_min;
    c.sort_bits = a.sort_bits;
    return c;
}

// Times every candidate shape: one warm-up launch, then the best of `reps`
// CUDA-event-timed launches on the context stream. With `sort_stage`, the
// winning shape is then timed with every coherence-order key width.
RT::TraceConfig RunTuner(fnd_rt_ctx* ctx, uint32_t reps,
                         const std::function<cudaError_t(const RT::TraceConfig&)>& launch, fnd_rt_tune_entry* table,
                         uint32_t table_cap, uint32_t* table_n, bool sort_stage = false) {
    cudaEvent_t e0, e1;
    CUDA_CHECK(cudaEventCreate(&e0));
    CUDA_CHECK(cudaEventCreate(&e1));
    RT::TraceConfig best{};
    float best_ms = 1e30f;
    uint32_t k = 0;
    try {
        auto time_one = [&](const RT::TraceConfig& c) {
            CUDA_CHECK(launch(c));
            float ms = 1e30f;
            for (uint32_t r = 0; r < std::max(1u, reps); ++r) {
                CUDA_CHECK(cudaEventRecord(e0, ctx->stream));
                CUDA_CHECK(launch(c));
                CUDA_CHECK(cudaEventRecord(e1, ctx->stream));
                CUDA_CHECK(cudaEventSynchronize(e1));
                float t = 0.0f;
                CUDA_CHECK(cudaEventElapsedTime(&t, e0, e1));
                ms = std::min(ms, t);
            }
            if (table && k < table_cap) table[k] = fnd_rt_tune_entry{ToAbi(c), ms};
            ++k;
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        };
        for (const RT::TraceConfig& c : Candidates()) time_one(c);
        if (sort_stage) {
            const RT::TraceConfig shape = best;
            for (uint32_t bits : {9u, 12u, 15u, 18u, 21u}) {
                RT::TraceConfig c = shape;
                c.sort_bits = bits;
                time_one(c);
            }
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (table_n) *table_n = std::min(k, table_cap);
    const int s = CApi::ReadStatus(ctx);
    if (s != FND_OK) RtCore::Fail(s, "device status %d while tuning", s);
    return best;
}

void Capture(fnd_rt_batch* b) {
    fnd_rt_ctx* ctx = b->ctx;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (!b->use_graph) return;
    cudaStream_t cs = nullptr;
    CUDA_CHECK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    const int grid = CApi::TraceGrid(ctx, b->cfg, 4);
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t le = RT::LaunchBatch(b->launch, b->cfg, grid, cs);
        e = cudaStreamEndCapture(cs, &b->graph);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    cudaStreamDestroy(cs);
    CUDA_CHECK(e);
}

}  // namespace

extern "C" {

int fnd_rt_set_trace_config(fnd_rt_ctx* ctx, const fnd_rt_trace_config* config) {
    if (!ctx || !config) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        const RT::TraceConfig c = FromAbi(*config);
        CHECK_CODE(RT::ValidTraceConfig(c), FND_ERR_INVALID_ARG,
                   "launch shape block %u / short stack %u / refill %u / postpone %u / sort bits %u", config->block,
                   config->short_stack, config->refill_min, config->postpone_min, config->sort_bits);
        ctx->trace_cfg = c;
        ctx->refill_min = c.refill_min;
    });
}

int fnd_rt_get_trace_config(const fnd_rt_ctx* ctx, fnd_rt_trace_config* out) {
    if (!ctx || !out) return FND_ERR_INVALID_ARG;
    *out = ToAbi(ctx->trace_cfg);
    return FND_OK;
}

int fnd_rt_tune(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n, uint32_t kind,
                uint32_t reps, fnd_rt_tune_entry* table, uint32_t table_cap, uint32_t* table_n,
                fnd_rt_trace_config* best) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(scene && scene->ctx == ctx && rays && n > 0 && kind <= FND_QUERY_ANY);
        CHECK_CODE(!scene->two_level, FND_ERR_INVALID_ARG, "two-level scenes are not tuned");
        CHECK_CODE(((uintptr_t)rays & 15u) == 0, FND_ERR_INVALID_ARG, "device rays must be 16-byte aligned");
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const bool any = kind == FND_QUERY_ANY;
        CApi::EnsureDevice(ctx->d_out, ctx->d_out_cap, any ? n : 8ull * n);
        RT::TraceLaunch L{};
        L.scene = scene->view;
        L.rays = reinterpret_cast<const float4*>(rays);
        L.n = n;
        if (any)
            L.occluded = static_cast<uint8_t*>(ctx->d_out);
        else
            L.hits = ctx->d_out;
        L.counter = ctx->d_counter;
        L.status = ctx->d_status;
        const RT::TraceConfig b = RunTuner(
            ctx, reps,
            [&](const RT::TraceConfig& c) {
                return CApi::LaunchTraceOrdered(ctx, scene, L, any, false, c, CApi::TraceGrid(ctx, c, any ? 1 : 0));
            },
            table, table_cap, table_n, true);
        if (best) *best = ToAbi(b);
    });
}

int fnd_rt_batch_create(fnd_rt_ctx* ctx, const fnd_rt_batch_job* jobs, uint32_t njobs, uint32_t flags,
                        fnd_rt_batch** out_batch) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(out_batch != nullptr && (njobs == 0 || jobs != nullptr));
        *out_batch = nullptr;
        CHECK_CODE(njobs >= 1 && njobs <= (1u << 20), FND_ERR_INVALID_ARG, "%u jobs", njobs);
        std::vector<RT::BatchJob> table(njobs);
        std::vector<uint32_t> prefix(njobs + 1, 0);
        uint64_t total = 0;
        for (uint32_t i = 0; i < njobs; ++i) {
            const fnd_rt_batch_job& j = jobs[i];
            CHECK_CODE(j.scene && j.scene->ctx == ctx, FND_ERR_INVALID_ARG, "job %u: scene of another context", i);
            CHECK_CODE(!j.scene->two_level, FND_ERR_INVALID_ARG, "job %u: two-level scenes are not batched", i);
            CHECK_CODE(j.kind <= FND_QUERY_ANY, FND_ERR_INVALID_ARG, "job %u: kind %u", i, j.kind);
            CHECK_CODE(j.n == 0 || (j.rays && j.out), FND_ERR_INVALID_ARG, "job %u: null buffer", i);
            CHECK_CODE(((uintptr_t)j.rays & 15u) == 0 && ((uintptr_t)j.out & (j.kind ? 0u : 7u)) == 0,
                       FND_ERR_INVALID_ARG, "job %u: rays must be 16-byte and hits 8-byte aligned", i);
            table[i].scene = j.scene->view;
            table[i].rays = reinterpret_cast<const float4*>(j.rays);
            table[i].out = j.out;
            table[i].n = j.n;
            table[i].any = j.kind;
            prefix[i] = (uint32_t)total;
            total += j.n;
            CHECK_CODE(total < (1ull << 32) - 64, FND_ERR_INVALID_ARG, "batch exceeds 2^32 rays");
        }
        prefix[njobs] = (uint32_t)total;
        CUDA_CHECK(cudaSetDevice(ctx->device));
        auto b = std::make_unique<fnd_rt_batch>();
        b->ctx = ctx;
        b->cfg = ctx->trace_cfg;
        b->use_graph = !(flags & FND_BATCH_NO_GRAPH);
        const size_t tbytes = sizeof(RT::BatchJob) * njobs;
        const size_t pbytes = sizeof(uint32_t) * (njobs + 1);
        const size_t poff = (tbytes + 255) & ~size_t(255), coff = (poff + pbytes + 255) & ~size_t(255);
        char* base = nullptr;
        CUDA_CHECK(cudaMalloc(&base, coff + 256));
        b->d_block = base;
        try {
            CUDA_CHECK(cudaMemcpy(base, table.data(), tbytes, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(base + poff, prefix.data(), pbytes, cudaMemcpyHostToDevice));
            b->launch.jobs = reinterpret_cast<const RT::BatchJob*>(base);
            b->launch.prefix = reinterpret_cast<const uint32_t*>(base + poff);
            b->launch.njobs = njobs;
            b->launch.total = (uint32_t)total;
            b->launch.counter = reinterpret_cast<uint32_t*>(base + coff);
            b->launch.status = ctx->d_status;
            b->launch.refill_min = ctx->refill_min;
            Capture(b.get());
        } catch (...) {
            if (b->exec) cudaGraphExecDestroy(b->exec);
            if (b->graph) cudaGraphDestroy(b->graph);
            cudaFree(base);
            throw;
        }
        *out_batch = b.release();
    });
}

int fnd_rt_batch_launch(fnd_rt_batch* b) {
    if (!b) return FND_ERR_INVALID_ARG;
    fnd_rt_ctx* ctx = b->ctx;
    return Guard(ctx, [&] {
        CUDA_CHECK(cudaSetDevice(ctx->device));
        if (b->exec)
            CUDA_CHECK(cudaGraphLaunch(b->exec, ctx->stream));
        else
            CUDA_CHECK(RT::LaunchBatch(b->launch, b->cfg, CApi::TraceGrid(ctx, b->cfg, 4), ctx->stream));
    });
}

int fnd_rt_batch_tune(fnd_rt_batch* b, uint32_t reps, fnd_rt_tune_entry* table, uint32_t table_cap,
                      uint32_t* table_n, fnd_rt_trace_config* best) {
    if (!b) return FND_ERR_INVALID_ARG;
    fnd_rt_ctx* ctx = b->ctx;
    return Guard(ctx, [&] {
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const RT::TraceConfig c = RunTuner(
            ctx, reps,
            [&](const RT::TraceConfig& cfg) {
                return RT::LaunchBatch(b->launch, cfg, CApi::TraceGrid(ctx, cfg, 4), ctx->stream);
            },
            table, table_cap, table_n);
        b->cfg = c;
        Capture(b);
        if (best) *best = ToAbi(c);
    });
}

int fnd_rt_batch_destroy(fnd_rt_batch* b) {
    if (!b) return FND_ERR_INVALID_ARG;
    fnd_rt_ctx* ctx = b->ctx;
    const int rc = Guard(ctx, [&] {
        CUDA_CHECK(cudaSetDevice(ctx->device));
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_block) cudaFree(b->d_block);
    delete b;
    return rc;
}

}  // extern "C"
