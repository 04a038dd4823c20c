// ImageIO.hpp — headless image files for the path-tracer pass (the swapchain
// of Renderer::Draw, src/Renderer/Renderer.cpp:395-399, has no counterpart on
// a compute-only GPU; frames go to files instead).
#pragma once

#include <cstdint>
#include <span>

namespace Foundation {
namespace Renderer {

// Linear float RGB, width*height*3, row-major from the top row; PFM stores
// rows bottom to top.
void WritePfm(const char* path, std::span<const float> rgb, uint32_t width, uint32_t height);

// 8-bit RGBA (the R8G8B8A8_UNORM layout of fnd_rt_tonemap), width*height*4,
// top row first. PNG (ISO/IEC 15948) with filter type 0 and stored
// (uncompressed) deflate blocks, so no compression library is needed.
void WritePng(const char* path, std::span<const uint8_t> rgba, uint32_t width, uint32_t height);

}  // namespace Renderer
}  // namespace Foundation
