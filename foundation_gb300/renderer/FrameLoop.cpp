// FrameLoop.cpp — see FrameLoop.hpp.
#include "FrameLoop.hpp"

namespace Foundation {
namespace Renderer {

uint32_t RenderFrames(Core::Allocator* allocator, const FrameLoopDesc& desc, const SceneDesc& scene,
                      std::span<float> rgb, std::span<uint8_t> rgba8) {
    CHECK(allocator != nullptr && desc.draws > 0);
    PathTracerPass pass(desc.pass, allocator);
    pass.SetScene(scene);
    pass.SetCamera(desc.camera);
    const float none[3] = {0, 0, 0};
    pass.SetEnvironment(desc.sky, none, none);
    for (uint32_t i = 0; i < desc.draws; ++i) pass.Draw();
    pass.Readback(rgb);
    if (!rgba8.empty()) pass.ReadbackRGBA8(rgba8);
    return pass.SamplesAccumulated();
}

}  // namespace Renderer
}  // namespace Foundation
