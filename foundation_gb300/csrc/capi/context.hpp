// context.hpp — internal definitions of the opaque C-ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <new>
#include <stdexcept>
#include <string>

#include "../../../include/fnd_rt.h"
#include "../core/core.hpp"
#include "../pt/integrator.hpp"
#include "../rt/ray_sort.hpp"
#include "../rt/traverse_launch.hpp"

#include <vector>

// Radiance-cache session of a context.
struct FndCacheState {
    fnd_cache_desc desc{};
    Foundation::NRC::Net net{};
    void* d_block = nullptr;  // one allocation for everything below
    size_t block_bytes = 0;
    Foundation::NRC::TrainSample* samples = nullptr;
    float4* targets = nullptr;
    Foundation::NRC::CachePoint* queries = nullptr;
    uint32_t* counters = nullptr;  // [0] queries, [1] samples
    uint32_t sample_cap = 0;
    uint32_t query_cap = 0;
    uint32_t train_cap = 0;
    uint64_t frames = 0;
    // training runs on its own stream, overlapping the render wave
    cudaStream_t train_stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_trained = nullptr;
};

struct fnd_rt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 0;
    int occupancy[4] = {0, 0, 0, 0};  // blocks/SM of the trace kernel variants
    uint32_t refill_min = 8;
    // device scratch owned by the context
    uint32_t* d_counter = nullptr;
    uint32_t* d_status = nullptr;
    unsigned long long* d_stats = nullptr;
    uint32_t* h_status = nullptr;  // pinned
    // staging buffers for FND_MEM_HOST calls
    void* d_in = nullptr;
    size_t d_in_cap = 0;
    void* d_out = nullptr;
    size_t d_out_cap = 0;
    // pipelined FND_MEM_HOST traces: copy streams (created on first use) and
    // events: [0] start, [1] end, then per chunk "rays in" and "traced"
    // (at most 17 chunks: a short first chunk and 16 more)
    cudaStream_t copy_in = nullptr, copy_out = nullptr, compute2 = nullptr;
    cudaEvent_t pipe_ev[2 + 2 * 17] = {};
    int live_scenes = 0;
    Foundation::RT::TraceConfig trace_cfg{};  // launch shape of the traversal kernels
    // path-tracing state: path buffers (capacity paths) and the frame buffer
    Foundation::PT::PathBuffers paths{};
    void* d_paths = nullptr;
    size_t paths_bytes = 0;
    float4* d_fb = nullptr;
    size_t fb_pixels = 0;
    uint32_t fb_width = 0, fb_height = 0, fb_samples = 0;
    float* d_rgb = nullptr;  // finalize target for host outputs
    size_t rgb_cap = 0;
    unsigned long long* d_render_stats = nullptr;  // [0] extension rays, [1] shadow rays
    int tail_blocks_per_sm[2] = {0, 0};            // occupancy of the tail megakernel, one- / two-level (0: not queried)
    int train_paths_blocks_per_sm[2] = {0, 0};     // occupancy of the training-path megakernel (0: not queried)
    void* d_sort = nullptr;                        // coherence-order scratch (rt/ray_sort.hpp)
    size_t d_sort_cap = 0;
    fnd_render_stats last_render{};
    FndCacheState* cache = nullptr;
    std::string last_error;
};

struct fnd_rt_scene {
    fnd_rt_ctx* ctx = nullptr;
    void* d_nodes = nullptr;
    void* d_tris = nullptr;
    Foundation::RT::DeviceScene view{};
    fnd_rt_scene_info info{};
    // shading data (original triangle order)
    std::vector<float> tri_shade;  // host staging of the shading records during upload (released after)
    void* d_tri_shade = nullptr;
    void* d_materials = nullptr;
    uint32_t num_materials = 0;
    void* d_lights = nullptr;
    uint32_t num_lights = 0;
    // two-level scenes (fnd_rt_instances_upload): d_nodes / d_tris hold the
    // top level over the instances' world boxes
    bool two_level = false;
    void* d_instances = nullptr;  // RT::InstanceRec[num_instances]
    uint32_t num_instances = 0;
    std::vector<fnd_rt_scene*> blas;  // the bottom levels (each counts this scene in `users`)
    int users = 0;                    // two-level scenes that instance this one
};

namespace Foundation {
namespace CApi {

// Message slot for failures that have no context (fnd_rt_last_error(NULL)).
std::string& GlobalError();

// Runs an entry point body: C++ failures become a negative fnd_status and a
// message in the context's (or the global) error slot.
template <typename F>
int Guard(fnd_rt_ctx* ctx, F&& body) {
    std::string* err = ctx ? &ctx->last_error : &GlobalError();
    try {
        body();
        err->clear();
        return FND_OK;
    } catch (const Foundation::RtCore::FndError& e) {
        *err = e.what();
        LOG_RUNTIME(FndRt, ERR, "%s", e.what());
        return e.code();
    } catch (const std::bad_alloc&) {
        *err = "host allocation failed";
        return FND_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        *err = e.what();
        return FND_ERR_INVALID_ARG;
    }
}

void CudaCheck(cudaError_t e, const char* what);
#define CUDA_CHECK(expr) ::Foundation::CApi::CudaCheck((expr), #expr)

// Grows a device staging buffer to at least `bytes`.
void EnsureDevice(void*& ptr, size_t& cap, size_t bytes);

// Reads and clears the latched device status; returns FND_OK or an error code.
int ReadStatus(fnd_rt_ctx* ctx);

// Persistent grid (SMs x resident blocks) of a traversal variant under a
// launch shape (variant as in RT::TraceOccupancyFor).
int TraceGrid(fnd_rt_ctx* ctx, const Foundation::RT::TraceConfig& cfg, int variant);

// Launches a traversal under a launch shape; with cfg.sort_bits the rays
// (L.n, or *L.n_dev when set) are first put in coherence order over the
// scene box (context scratch), otherwise taken in input order.
// `stream` null: the context stream.
cudaError_t LaunchTraceOrdered(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, Foundation::RT::TraceLaunch L, bool any,
                               bool stats, const Foundation::RT::TraceConfig& cfg, int grid,
                               cudaStream_t stream = nullptr);

// One grey Lambertian material table on a new scene (capi_trace.cpp).
void DefaultMaterial(fnd_rt_scene* scene);

// Radiance-cache session storage (capi_cache.cpp).
void FreeCache(fnd_rt_ctx* ctx);
void EnsureCacheBuffers(fnd_rt_ctx* ctx, uint32_t query_cap, uint32_t max_depth);

}  // namespace CApi
}  // namespace Foundation
