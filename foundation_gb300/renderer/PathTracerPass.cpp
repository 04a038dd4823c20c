// PathTracerPass.cpp — see PathTracerPass.hpp.
#include "PathTracerPass.hpp"

#include <cstring>
#include <stdexcept>
#include <string>

namespace Foundation {
namespace Renderer {

PathTracerPass::PathTracerPass(const PathTracerDesc& desc, Core::Allocator* allocator)
    : m_allocator(allocator), m_desc(desc) {
    CHECK(allocator != nullptr);
    CHECK(desc.width > 0 && desc.height > 0 && desc.spp_per_draw > 0);
    fnd_rt_desc d{FND_RT_ABI_VERSION, desc.device, desc.stream, 0};
    Check(fnd_rt_create(&d, &m_ctx), "fnd_rt_create");
    m_frame_bytes = sizeof(float) * 3 * (size_t)desc.width * desc.height;
    m_frame = static_cast<float*>(m_allocator->Allocate(m_frame_bytes, alignof(float)));
    m_camera = fnd_camera{{0, 0, 5}, {0, 0, 0}, {0, 1, 0}, 45.0f};
}

PathTracerPass::~PathTracerPass() {
    // like Renderer::~Renderer: the GPU is idle before anything is released
    if (m_ctx) fnd_rt_sync(m_ctx);
    if (m_scene) fnd_rt_scene_destroy(m_scene);
    if (m_ctx) fnd_rt_destroy(m_ctx);
    if (m_frame) m_allocator->Deallocate(m_frame, m_frame_bytes);
}

// A failed library call is a failed check in the application's idiom:
// BugCheck with the call, its fnd_status and the library's message.
void PathTracerPass::Check(int rc, const char* what) const {
    if (rc != FND_OK)
        Core::BugCheck(std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) +
                                          "): " + fnd_rt_last_error(m_ctx)));
}

void PathTracerPass::SetScene(const SceneDesc& s) {
    CHECK(s.verts.size() % 3 == 0 && s.indices.size() % 3 == 0);
    const uint32_t nt = (uint32_t)(s.indices.size() / 3);
    if (m_scene) {
        Check(fnd_rt_scene_destroy(m_scene), "fnd_rt_scene_destroy");
        m_scene = nullptr;
    }
    fnd_rt_bvh_desc b{};
    b.sah_bins = s.sah_bins;
    b.max_leaf_tris = s.max_leaf_tris;
    b.flags = s.bvh_flags;
    b.split_budget = s.split_budget;
    Check(fnd_rt_scene_upload(m_ctx, s.verts.data(), (uint32_t)(s.verts.size() / 3), s.indices.data(), nt, &b, &m_scene),
          "fnd_rt_scene_upload");
    Check(fnd_rt_scene_info_get(m_scene, &m_info), "fnd_rt_scene_info_get");
    if (!s.materials.empty()) {
        CHECK(s.tri_material.empty() || s.tri_material.size() == nt);
        if (s.tri_material.empty()) {
            // every triangle uses material 0: a zero-filled id array from the allocator
            const size_t bytes = sizeof(uint32_t) * (size_t)nt;
            auto* ids = static_cast<uint32_t*>(m_allocator->Allocate(bytes, alignof(uint32_t)));
            std::memset(ids, 0, bytes);
            const int rc = fnd_rt_scene_set_materials(m_scene, ids, nt, s.materials.data(), (uint32_t)s.materials.size());
            m_allocator->Deallocate(ids, bytes);
            Check(rc, "fnd_rt_scene_set_materials");
        } else {
            Check(fnd_rt_scene_set_materials(m_scene, s.tri_material.data(), nt, s.materials.data(),
                                             (uint32_t)s.materials.size()),
                  "fnd_rt_scene_set_materials");
        }
    }
    Check(fnd_rt_scene_set_lights(m_scene, s.lights.data(), (uint32_t)s.lights.size()), "fnd_rt_scene_set_lights");
    m_restart = true;
}

void PathTracerPass::SetCamera(const fnd_camera& camera) {
    m_camera = camera;
    m_restart = true;
}

void PathTracerPass::SetEnvironment(const float sky[3], const float sun_dir[3], const float sun_irradiance[3]) {
    for (int i = 0; i < 3; ++i) {
        m_sky[i] = sky[i];
        m_sun_dir[i] = sun_dir[i];
        m_sun_e[i] = sun_irradiance[i];
    }
    m_restart = true;
}

void PathTracerPass::Draw() {
    CHECK(m_scene != nullptr);
    fnd_render_desc r{};
    r.width = m_desc.width;
    r.height = m_desc.height;
    r.spp = m_desc.spp_per_draw;
    r.max_depth = m_desc.max_depth;
    r.rr_start = m_desc.rr_start;
    r.flags = m_restart ? 0u : FND_RENDER_ACCUMULATE;
    r.seed = m_desc.seed;
    r.camera = m_camera;
    for (int i = 0; i < 3; ++i) {
        r.sky[i] = m_sky[i];
        r.sun_dir[i] = m_sun_dir[i];
        r.sun_irradiance[i] = m_sun_e[i];
    }
    Check(fnd_rt_render(m_ctx, m_scene, &r, m_frame, FND_MEM_HOST), "fnd_rt_render");
    m_samples = m_restart ? m_desc.spp_per_draw : m_samples + m_desc.spp_per_draw;
    m_restart = false;
}

void PathTracerPass::Readback(std::span<float> rgb) {
    CHECK(rgb.size() * sizeof(float) >= m_frame_bytes);
    std::memcpy(rgb.data(), m_frame, m_frame_bytes);
}

void PathTracerPass::ReadbackRGBA8(std::span<uint8_t> rgba, float exposure, uint32_t mode) {
    CHECK(m_frame != nullptr && rgba.size() >= 4ull * m_desc.width * m_desc.height);
    Check(fnd_rt_tonemap(m_ctx, m_frame, m_desc.width, m_desc.height, FND_MEM_HOST, exposure, mode, rgba.data(),
                         FND_MEM_HOST),
          "fnd_rt_tonemap");
}

void PathTracerPass::TraceClosest(std::span<const fnd_ray> rays, std::span<fnd_hit> hits) {
    CHECK(m_scene != nullptr && hits.size() >= rays.size());
    Check(fnd_rt_trace_closest(m_ctx, m_scene, rays.data(), (uint32_t)rays.size(), hits.data(), FND_MEM_HOST),
          "fnd_rt_trace_closest");
}

void PathTracerPass::TraceAny(std::span<const fnd_ray> rays, std::span<uint8_t> occluded) {
    CHECK(m_scene != nullptr && occluded.size() >= rays.size());
    Check(fnd_rt_trace_any(m_ctx, m_scene, rays.data(), (uint32_t)rays.size(), occluded.data(), FND_MEM_HOST),
          "fnd_rt_trace_any");
}

}  // namespace Renderer
}  // namespace Foundation
