// raster.hpp — CUDA restatement of the reference renderer's raster pass
// (src/Renderer/Renderer.cpp:312-366 with src/Renderer/Triangle.slang): an
// indexed triangle list transformed by proj * view * model, back faces
// culled (front faces counter-clockwise), no depth test, each fragment
// colour = texture(uv) * vertex colour, written to an R8G8B8A8_UNORM target
// cleared first. Rules made explicit where the graphics API leaves them to
// the implementation: vertex positions snapped to 1/256 pixel, pixel centres
// at +0.5, the top-left fill rule, perspective-correct interpolation, and a
// bilinear texture lookup with repeat addressing (the isotropic case of the
// reference's sampler: linear filters, repeat, one mip level), all in
// double precision so a scalar restatement reproduces every byte.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace Foundation {
namespace Raster {

struct Vertex {
    float pos[2];
    float color[3];
    float uv[2];
};

struct Uniforms {
    float model[16], view[16], proj[16];  // column-major (m[c * 4 + r])
};

struct DrawArgs {
    uint32_t width, height;
    Uniforms u;
    float clear[4];
    uint32_t cull_back;
    const Vertex* verts;
    uint32_t nv;
    const uint16_t* idx;
    uint32_t ntri;
    const uint32_t* texture;  // RGBA8 texels, row-major
    uint32_t tex_w, tex_h;
    uint32_t* target;         // RGBA8 pixels, row-major from the top row
    double4* clip;            // scratch: nv clip-space positions
    uint32_t* status;
};

cudaError_t LaunchDraw(const DrawArgs& a, cudaStream_t s);

}  // namespace Raster
}  // namespace Foundation
