// capi_noalloc.cu — closest-hit tracing for callers that cannot allocate
// device memory.
//
// Who needs it: a renderer plugin that runs inside a host application's
// frame callback (where the host forbids device allocations mid-frame, or
// has partitioned all device memory up front), or a caller that must not
// add cudaMalloc / cudaFree calls that synchronise the device. Such a caller
// can upload a scene during set-up and later trace ray batches from plain
// host memory through this entry point, which allocates nothing: the ray and
// hit staging, the work-queue counter and the status word all live in one
// fixed file-scope device array, g_noalloc_scratch.
//
// Costs and rules:
//  * the array (kNoAllocBytes, about 2.5 MiB) is held by every GPU that loads
//    this library, from module load until process exit;
//  * at most kNoAllocMaxRays rays per call; larger batches are rejected with
//    FND_ERR_INVALID_ARG (split them, or use fnd_rt_trace_closest);
//  * every call reuses the same array and it keeps the previous call's
//    contents, so the counter and status word are cleared at the start of
//    each call; calls whose work overlaps on the GPU (from several threads,
//    or on several streams) race on the array and must be serialised by the
//    caller;
//  * the first call on a device resolves the array's device address
//    (cudaGetSymbolAddress). Under lazy module loading that is also when the
//    driver loads the module and reserves the array, so make the first call
//    at set-up time, while device memory is still free, and before any
//    stream capture begins. A failed set-up is not remembered: the next call
//    tries again;
//  * it launches with the context's launch shape (fnd_rt_set_trace_config /
//    fnd_rt_tune) without the coherence sort, whose scratch would need an
//    allocation; results do not depend on the shape;
//  * the call is synchronous (it returns once the hits are in `out`) and
//    leaves the caller's current device as it found it.
#include <cuda_runtime.h>

#include <mutex>

#include "context.hpp"

namespace {

constexpr uint32_t kNoAllocMaxRays = 65536;
constexpr size_t kHeaderBytes = 256;  // [0] work counter, [1] status word
constexpr size_t kRayBytes = (size_t)kNoAllocMaxRays * sizeof(fnd_ray);
constexpr size_t kHitBytes = (size_t)kNoAllocMaxRays * sizeof(fnd_hit);
constexpr size_t kNoAllocBytes = kHeaderBytes + kRayBytes + kHitBytes;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch, resolved once per device with that
// device current. Host code must not use the symbol itself as a pointer: on
// the host it names a stand-in, not device memory.
struct DeviceScratch {
    std::mutex mu;
    bool ready = false;
    unsigned char* ptr = nullptr;
};
DeviceScratch g_scratch[kMaxDevices];

// Only a successful set-up is kept; a failure (for example no device memory
// left for the array when the module loads) clears the CUDA error it left
// and throws, and the next call tries again.
unsigned char* ScratchFor(int device) {
    DeviceScratch& s = g_scratch[device];
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.ready) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            Foundation::CApi::CudaCheck(e, "no-allocation scratch set-up (cudaGetSymbolAddress)");
        }
        s.ptr = static_cast<unsigned char*>(p);
        s.ready = true;
    }
    return s.ptr;
}

// Restores the calling thread's current device on scope exit.
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            (void)cudaGetLastError();
            prev = -1;
        }
    }
    ~DeviceRestore() {
        if (prev >= 0) (void)cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int fnd_rt_trace_closest_noalloc(const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n,
                                            fnd_hit* out, void* stream) {
    using namespace Foundation;
    if (!scene) {
        CApi::GlobalError() = "scene is NULL";
        return FND_ERR_INVALID_ARG;
    }
    fnd_rt_ctx* ctx = scene->ctx;
    return CApi::Guard(ctx, [&] {
        CHECK(n == 0 || (rays != nullptr && out != nullptr));
        CHECK_CODE(!scene->two_level, FND_ERR_INVALID_ARG, "two-level scenes are traced with fnd_rt_trace_closest");
        CHECK_CODE(n <= kNoAllocMaxRays, FND_ERR_INVALID_ARG,
                   "%u rays exceed the no-allocation limit of %u rays per call; split the batch or use "
                   "fnd_rt_trace_closest",
                   n, kNoAllocMaxRays);
        CHECK_CODE(ctx->device >= 0 && ctx->device < kMaxDevices, FND_ERR_NO_DEVICE, "device ordinal %d",
                   ctx->device);
        DeviceRestore restore;
        CUDA_CHECK(cudaSetDevice(ctx->device));
        unsigned char* scratch = ScratchFor(ctx->device);
        if (n == 0) return;
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
        uint32_t* counter = reinterpret_cast<uint32_t*>(scratch);
        uint32_t* status = counter + 1;
        unsigned char* d_rays = scratch + kHeaderBytes;
        unsigned char* d_hits = d_rays + kRayBytes;
        // the context's launch shape, in input order (the coherence sort
        // needs scratch of its own)
        RT::TraceConfig cfg = ctx->trace_cfg;
        cfg.sort_bits = 0;
        int blocks = 0;
        CUDA_CHECK(RT::TraceOccupancyFor(cfg, 0, &blocks));
        blocks = blocks > 0 ? blocks : 1;
        if (cfg.blocks_per_sm > 0 && cfg.blocks_per_sm < blocks) blocks = cfg.blocks_per_sm;
        const int grid = ctx->sm_count * blocks;
        // the previous call's counter and status must not leak into this one
        CUDA_CHECK(cudaMemsetAsync(scratch, 0, kHeaderBytes, st));
        CUDA_CHECK(cudaMemcpyAsync(d_rays, rays, sizeof(fnd_ray) * (size_t)n, cudaMemcpyHostToDevice, st));
        RT::TraceLaunch L{};
        L.scene = scene->view;
        L.rays = reinterpret_cast<const float4*>(d_rays);
        L.n = n;
        L.hits = d_hits;
        L.counter = counter;
        L.status = status;
        L.refill_min = ctx->refill_min;
        CUDA_CHECK(RT::LaunchTraceConfigured(L, false, false, cfg, grid, st));
        CUDA_CHECK(cudaMemcpyAsync(out, d_hits, sizeof(fnd_hit) * (size_t)n, cudaMemcpyDeviceToHost, st));
        uint32_t h_status = 0;
        CUDA_CHECK(cudaMemcpyAsync(&h_status, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        const int code = RT::StatusCode(h_status);
        CHECK_CODE(code == FND_OK, code, "device status 0x%x after the no-allocation trace", h_status);
    });
}
