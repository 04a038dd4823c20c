// PathTracerPass.hpp — the path-tracer pass for Foundation's Renderer layer.
//
// Shape of the reference renderer (src/Renderer/Renderer.hpp:10-44): built
// from a device and a Core::Allocator*, non-copyable, one per-frame Draw(),
// waits for the GPU in its destructor (src/Renderer/Renderer.cpp:402-406),
// CHECK on misuse (src/Core/Core.hpp:17). Under it sits the C ABI of
// include/fnd_rt.h; this class is what src/Renderer would hold in place of
// (or beside) the raster Renderer. Presenting is replaced by Readback into a
// caller buffer: there is no swapchain on a compute-only GPU.
#pragma once

#include <cstdint>
#include <span>
#include <string>

#include <fnd_rt.h>

#include "FoundationCore.hpp"

namespace Foundation {
namespace Renderer {

struct PathTracerDesc {
    int device = 0;
    void* stream = nullptr;  // cudaStream_t; null: the pass owns one
    uint32_t width = 1920;
    uint32_t height = 1080;
    uint32_t spp_per_draw = 1;  // samples per pixel added by each Draw()
    uint32_t max_depth = 8;
    uint32_t rr_start = 3;
    uint64_t seed = 1;
};

struct SceneDesc {
    std::span<const float> verts;           // xyz per vertex
    std::span<const uint32_t> indices;      // 3 per triangle
    std::span<const uint32_t> tri_material; // 1 per triangle (empty: all material 0)
    std::span<const fnd_material> materials;
    std::span<const fnd_quad_light> lights;
    uint32_t sah_bins = 32;
    uint32_t max_leaf_tris = 4;
    // FND_BVH_* flags of the upload. The SAH-optimal collapse costs little at
    // build time and traces faster; add FND_BVH_SPATIAL_SPLITS (with a split
    // budget, 8 lets the SAH decide) for scenes of long, overlapping triangles.
    uint32_t bvh_flags = FND_BVH_SAH_COLLAPSE;
    float split_budget = 0.0f;
};

class PathTracerPass {
public:
    PathTracerPass(const PathTracerDesc& desc, Core::Allocator* allocator);
    ~PathTracerPass();
    PathTracerPass(const PathTracerPass&) = delete;
    PathTracerPass& operator=(const PathTracerPass&) = delete;

    void SetScene(const SceneDesc& scene);
    void SetCamera(const fnd_camera& camera);
    void SetEnvironment(const float sky[3], const float sun_dir[3], const float sun_irradiance[3]);

    // Adds spp_per_draw samples per pixel to the running frame; the first
    // Draw() after a scene / camera / environment change restarts it.
    void Draw();
    uint32_t SamplesAccumulated() const { return m_samples; }

    // Mean radiance so far, width*height*3 floats (row-major from the top).
    void Readback(std::span<float> rgb);
    // The same frame in the reference's colour-target format R8G8B8A8_UNORM
    // (width*height*4 bytes, fnd_rt_tonemap with `mode` and `exposure`).
    void ReadbackRGBA8(std::span<uint8_t> rgba, float exposure = 1.0f, uint32_t mode = FND_TONEMAP_ACES);

    void TraceClosest(std::span<const fnd_ray> rays, std::span<fnd_hit> hits);
    void TraceAny(std::span<const fnd_ray> rays, std::span<uint8_t> occluded);

    const fnd_rt_scene_info& SceneInfo() const { return m_info; }

private:
    void Check(int rc, const char* what) const;

    Core::Allocator* m_allocator{nullptr};
    PathTracerDesc m_desc;
    fnd_rt_ctx* m_ctx{nullptr};
    fnd_rt_scene* m_scene{nullptr};
    fnd_rt_scene_info m_info{};
    fnd_camera m_camera{};
    float m_sky[3] = {0, 0, 0}, m_sun_dir[3] = {0, 0, 0}, m_sun_e[3] = {0, 0, 0};
    float* m_frame{nullptr};  // host copy of the last frame, from the allocator
    size_t m_frame_bytes{0};
    uint32_t m_samples{0};
    bool m_restart{true};
};

}  // namespace Renderer
}  // namespace Foundation
