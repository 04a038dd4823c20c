// tonemap.cu — linear radiance to the display format of the reference
// renderer's colour target, R8G8B8A8_UNORM (src/Renderer/Renderer.cpp:40,81).
//
// Per channel: x = exposure * L, then the tone curve
//   FND_TONEMAP_CLAMP     x
//   FND_TONEMAP_REINHARD  x / (1 + x)
//   FND_TONEMAP_ACES      (x (2.51 x + 0.03)) / (x (2.43 x + 0.59) + 0.14)
//                         (Narkowicz 2015, fit of the ACES reference curve)
// clamped to [0, 1], encoded with the sRGB transfer function (IEC 61966-2-1:
// 12.92 x below 0.0031308, else 1.055 x^(1/2.4) - 0.055) because the target
// is UNORM, not an sRGB format, and rounded to 8 bits; alpha is 255. NaN
// radiance maps to 0.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../../include/fnd_rt.h"
#include "integrator.hpp"

namespace Foundation {
namespace PT {
namespace {

__device__ __forceinline__ uint32_t encode(float L, float exposure, uint32_t mode) {
    float x = exposure * L;
    if (!(x > 0.0f)) return 0u;  // negative, zero and NaN
    if (mode == FND_TONEMAP_REINHARD)
        x = x / (1.0f + x);
    else if (mode == FND_TONEMAP_ACES)
        x = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
    x = fminf(x, 1.0f);
    const float s = x <= 0.0031308f ? 12.92f * x : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
    return (uint32_t)fminf(fmaxf(s * 255.0f + 0.5f, 0.0f), 255.0f);
}

__global__ void __launch_bounds__(256) tonemap_kernel(const float* __restrict__ rgb, uint32_t npix, float exposure,
                                                      uint32_t mode, uint32_t* __restrict__ rgba) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const uint32_t r = encode(rgb[3 * (size_t)i + 0], exposure, mode);
    const uint32_t g = encode(rgb[3 * (size_t)i + 1], exposure, mode);
    const uint32_t b = encode(rgb[3 * (size_t)i + 2], exposure, mode);
    rgba[i] = r | (g << 8) | (b << 16) | (255u << 24);  // bytes R, G, B, A in memory
}

}  // namespace

cudaError_t LaunchTonemap(const float* rgb, uint32_t npix, float exposure, uint32_t mode, uint32_t* rgba,
                          cudaStream_t s) {
    if (npix == 0) return cudaSuccess;
    tonemap_kernel<<<(npix + 255) / 256, 256, 0, s>>>(rgb, npix, exposure, mode, rgba);
    return cudaGetLastError();
}

}  // namespace PT
}  // namespace Foundation
