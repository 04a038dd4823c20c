// mlp_common.cuh — device helpers shared by the radiance cache's kernels
// (mlp.cu: inference, Adam, images; train_umma.cu: training): BF16
// rounding, the 96-feature input encoding and the sample hash.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "nrc.hpp"

namespace Foundation {
namespace NRC {

constexpr float kLossEps = 0.01f;  // relative-L2 loss: (y - t)^2 / (y^2 + eps)

__device__ __forceinline__ uint16_t bf16_bits(float x) {
    __nv_bfloat16 b = __float2bfloat16_rn(x);
    return *reinterpret_cast<uint16_t*>(&b);
}

__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

// ---- input encoding ------------------------------------------------------
// 12 sine/cosine bands per normalised position axis (sin / cos of 2^k pi p),
// then outgoing direction, normal, roughness, albedo, zero padding to 96.
// `half` 0 writes features 0..47, `half` 1 features 48..95.
__device__ __forceinline__ void encode_axis(float u, uint16_t* out) {
    // bands k = 0..11: sin / cos of 2^k pi u. Bands 0, 4, 8 come from
    // sincospif; the three after each from the double-angle identities
    // (at most three doublings: error below 1e-6, far under a bf16 step).
#pragma unroll
    for (int k0 = 0; k0 < 12; k0 += 4) {
        float s, c;
        sincospif(ldexpf(u, k0), &s, &c);
#pragma unroll
        for (int k = k0; k < k0 + 4; ++k) {
            out[2 * k] = bf16_bits(s);
            out[2 * k + 1] = bf16_bits(c);
            const float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
}

__device__ __forceinline__ void encode_half(const CachePoint& c, const float lo[3], const float hi[3], int half,
                                            uint16_t* row) {
    const float p[3] = {c.p_rough.x, c.p_rough.y, c.p_rough.z};
    if (half == 0) {
        for (int a = 0; a < 2; ++a) {
            const float ext = hi[a] - lo[a];
            encode_axis(ext > 0.0f ? (p[a] - lo[a]) / ext : 0.0f, row + 24 * a);
        }
    } else {
        const float ext = hi[2] - lo[2];
        encode_axis(ext > 0.0f ? (p[2] - lo[2]) / ext : 0.0f, row + 48);
        const float rest[10] = {c.wo_aux.x, c.wo_aux.y, c.wo_aux.z, c.n_pad.x, c.n_pad.y, c.n_pad.z,
                                c.p_rough.w, c.albedo.x, c.albedo.y, c.albedo.z};
        for (int i = 0; i < 10; ++i) row[72 + i] = bf16_bits(rest[i]);
        for (int i = 82; i < 96; ++i) row[i] = 0;
    }
}

}  // namespace NRC
}  // namespace Foundation
