// integrator.hpp — host-visible interface of the wavefront path tracer.
//
// A frame is processed in waves of at most `capacity` paths. Per wave:
//   generate -> [extend (closest hit) -> shade -> shadow (any hit + resolve)] x max_depth
// Queues live in device memory and their lengths are device counters, so no
// stage needs a host round trip; the host only enqueues the fixed sequence.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../nrc/nrc.hpp"
#include "../rt/device_scene.hpp"

namespace Foundation {
namespace PT {

constexpr uint32_t kMatLambert = 0;
constexpr uint32_t kMatGGX = 1;
constexpr uint32_t kMatEmissive = 2;

struct DevMaterial {
    float4 albedo_type;     // rgb albedo / specular colour, w = type bits
    float4 emission_light;  // rgb emission, w = light index bits (int, -1 = none)
    float4 params;          // x = GGX alpha
};

struct DevQuadLight {
    float4 corner_area;  // xyz corner, w = area
    float4 eu;           // edge u
    float4 ev;           // edge v
    float4 normal;       // unit emitting-side normal (cross(eu, ev))
    float4 radiance;     // rgb
};

struct ShadeScene {
    const float4* tri_shade;  // per original triangle: unit geometric normal (winding), w = material id bits
    const DevMaterial* materials;
    const DevQuadLight* lights;
    uint32_t num_lights;
    uint32_t num_materials;
};

struct RenderParams {
    uint32_t width, height;
    uint32_t spp;            // samples per pixel of this call
    uint32_t max_depth;      // surface interactions per path
    uint32_t rr_start;       // first bounce index that applies Russian roulette
    uint32_t sample_offset;  // sample index of the first sample of this call (accumulation)
    uint64_t seed;
    float eye[3], fwd[3], right[3], up[3];
    float tan_half, aspect;
    float sky[3];
    float sun_dir[3];  // unit, towards the sun
    float sun_E[3];    // irradiance of the directional sun
    uint32_t has_sun;
    float eps;         // ray-origin offset along the normal
};

struct PathBuffers {
    uint32_t capacity;
    uint4* rng;          // x,y = PCG state (lo, hi), z = sequence (sample index), w = pixel
    float4* beta;        // rgb throughput, w = solid-angle pdf of the last BSDF sample (0 at the camera)
    float4* ext_rays[2]; // 2 float4 per ray (fnd_ray layout), ping-pong by bounce parity
    uint32_t* ext_path[2];
    uint2* hits;
    float4* sh_rays;     // 2 float4 per shadow ray; up to 2 per path per bounce
    uint32_t* sh_pixel;
    float4* sh_contrib;
    uint8_t* sh_occluded;
    uint32_t* counts;    // [0], [1] extension queues, [2] shadow queue, [3..] statistics
    float4* fb;          // per-pixel radiance sums
};

// Radiance-cache hook of the shade stage.
//  mode 0: plain path tracing;
//  mode 1: render with the cache: after the first non-specular bounce the
//          next non-emissive vertex becomes a cache query (its reflected
//          radiance comes from the network) and the path ends there.
struct CacheIO {
    uint32_t mode;
    float specular_alpha;  // GGX alpha below which a vertex counts as specular
    NRC::CachePoint* queries;
    uint32_t* query_count;
    uint32_t query_cap;
};

// The cache's training paths (train_paths.cu): n full paths through random
// pixels, one thread each; every non-emissive vertex becomes a training
// sample with its target.
struct TrainPathsArgs {
    RT::DeviceScene scene;
    const RT::InstanceRec* inst;  // two-level scene: its instances (scene is the top level), else null
    uint32_t num_inst;
    RenderParams R;
    ShadeScene S;
    uint32_t n;
    uint32_t seed;
    NRC::TrainSample* samples;
    float4* targets;
    uint32_t* sample_count;
    uint32_t sample_cap;
    uint32_t* status;
    uint32_t* fetch;  // path-fetch counter (zeroed by the launch)
};
// grid: the persistent grid (SMs x TrainingPathsBlocksPerSm), capped at the
// blocks the paths need.
cudaError_t LaunchTrainingPaths(const TrainPathsArgs& A, int grid, cudaStream_t s);
int TrainingPathsBlocksPerSm(bool two_level);

constexpr uint32_t kQueryNextFlag = 0x80000000u;  // in PathBuffers::rng.w

// Device counters of a wave (PathBuffers::counts): the two extension queue
// lengths, the shadow queue length, and the tail kernel's block-completion
// and path-fetch counters (all reset by generate).
constexpr int kCountExt0 = 0, kCountExt1 = 1, kCountShadow = 2;
constexpr int kCountTailDone = 8, kCountTailFetch = 9;

// The tail of a wave: once the extension queue `q` (the paths that continue
// to interaction `bounce`) holds at most `threshold` paths, one persistent
// megakernel finishes every one of them (lanes fetch paths dynamically and
// run them to the end with single-ray traversal and the shade stage's
// vertex logic) and empties the queue, so the remaining wavefront stages of
// the wave find nothing to do. Above the threshold it returns at once.
// Results are those of the wavefront stages: same random numbers per path,
// same hits; only the order of the frame-buffer additions differs.
struct TailArgs {
    RT::DeviceScene scene;
    const RT::InstanceRec* inst;  // two-level scene: its instances (scene is the top level), else null
    uint32_t num_inst;
    PathBuffers B;
    RenderParams R;
    ShadeScene S;
    CacheIO C;
    int q;
    uint32_t bounce;
    uint32_t threshold;
    uint32_t* status;
    unsigned long long* ray_stats;  // [0] extension rays, [1] shadow rays
};
cudaError_t LaunchTail(const TailArgs& A, int grid, cudaStream_t s);
int TailBlocksPerSm(bool two_level);  // resident tail blocks per SM (occupancy of that variant)
constexpr int kTailBlock = 128;

cudaError_t LaunchGenerate(const PathBuffers& B, const RenderParams& R, uint64_t wave_base, uint32_t wave_n,
                           cudaStream_t s);
cudaError_t LaunchShade(const PathBuffers& B, const RenderParams& R, const ShadeScene& S, const CacheIO& C, int cur,
                        uint32_t bounce, int grid, cudaStream_t s);
cudaError_t LaunchResolve(const PathBuffers& B, int grid, cudaStream_t s);
cudaError_t LaunchFinalize(const PathBuffers& B, float* rgb, uint32_t npix, float scale, cudaStream_t s);
// tonemap.cu: linear RGB floats -> R8G8B8A8_UNORM words (FND_TONEMAP_* mode)
cudaError_t LaunchTonemap(const float* rgb, uint32_t npix, float exposure, uint32_t mode, uint32_t* rgba,
                          cudaStream_t s);

}  // namespace PT
}  // namespace Foundation
