// FrameLoop.hpp — the per-frame use of the path-tracer pass by a Foundation
// application, in the shape of its Editor loop (src/Editor/Editor.cpp:14-28:
// construct the renderer with the application's allocator, then Draw() once
// per frame): construct the pass, set the scene, camera and environment,
// draw, read the frame back.
#pragma once

#include <cstdint>
#include <span>

#include "PathTracerPass.hpp"

namespace Foundation {
namespace Renderer {

struct FrameLoopDesc {
    PathTracerDesc pass;
    fnd_camera camera{{0, 0, 5}, {0, 0, 0}, {0, 1, 0}, 45.0f};
    float sky[3] = {0, 0, 0};
    uint32_t draws = 1;
};

// Renders desc.draws frames of `scene` (each adds pass.spp_per_draw samples
// per pixel) with host memory from `allocator`, then reads the mean radiance
// into rgb (width * height * 3 floats) and, when rgba8 is not empty, the
// display pixels (R8G8B8A8_UNORM, ACES, exposure 1) into rgba8. Returns the
// samples per pixel accumulated. Failures go through CHECK / BugCheck.
uint32_t RenderFrames(Core::Allocator* allocator, const FrameLoopDesc& desc, const SceneDesc& scene,
                      std::span<float> rgb, std::span<uint8_t> rgba8 = {});

}  // namespace Renderer
}  // namespace Foundation
