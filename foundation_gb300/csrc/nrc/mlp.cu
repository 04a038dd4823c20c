// mlp.cu — fused BF16 tensor-core MLP of the radiance cache (sm_103a):
// inference, training (forward + relative-L2 loss + backward + weight
// gradients) and Adam.
//
// Tensor-core path: mma.sync.m16n8k16 BF16 x BF16 -> FP32, operands staged
// in shared memory and fetched with ldmatrix (.trans for the transposed
// operands of the weight-gradient GEMMs). A warp owns 16 rows; activations
// of every layer stay in shared memory for the backward pass. The layers are
// only 64 wide, so the kernels are latency-bound: everything a row needs is
// fused into one launch.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "nrc.hpp"

namespace Foundation {
namespace NRC {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = 32 * kWarps;
constexpr int kTileRows = 16 * kWarps;  // rows per training tile
constexpr int kStrideX = kIn + kPad;    // 104
constexpr int kStrideH = kWidth + kPad; // 72
constexpr float kLossEps = 0.01f;

__device__ __forceinline__ uint32_t sptr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm4(uint32_t* r, uint32_t a) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm4t(uint32_t* r, uint32_t a) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm2(uint32_t* r, uint32_t a) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}
__device__ __forceinline__ void ldsm2t(uint32_t* r, uint32_t a) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}
__device__ __forceinline__ void mma(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float2 unpack2(uint32_t u) {
    __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162*>(&u);
    return __bfloat1622float2(v);
}
__device__ __forceinline__ uint16_t bf16_bits(float x) {
    __nv_bfloat16 b = __float2bfloat16_rn(x);
    return *reinterpret_cast<uint16_t*>(&b);
}

// Address of the ldmatrix row this lane supplies for an A-operand 16x16 tile
// of a row-major matrix (rows r0.., cols c0..): matrices ordered
// (rows 0-7, cols 0-7), (rows 8-15, cols 0-7), (rows 0-7, cols 8-15),
// (rows 8-15, cols 8-15) -> a0..a3 of mma.m16n8k16.
__device__ __forceinline__ uint32_t a_addr(const uint16_t* m, int stride, int r0, int c0, int lane) {
    const int j = lane >> 3, r = lane & 7;
    return sptr(m + (size_t)(r0 + ((j & 1) ? 8 : 0) + r) * stride + c0 + ((j & 2) ? 8 : 0));
}
// B operand from a row-major [n][k] image: two n-tiles (rows 8*nt..) of one
// k16 chunk: matrices (nt, k lo), (nt, k hi), (nt+1, k lo), (nt+1, k hi).
__device__ __forceinline__ uint32_t b_addr(const uint16_t* m, int stride, int n0, int k0, int lane) {
    const int j = lane >> 3, r = lane & 7;
    return sptr(m + (size_t)(n0 + 8 * (j >> 1) + r) * stride + k0 + ((j & 1) ? 8 : 0));
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

// ---- forward of one warp's 16 rows --------------------------------------
// act[l]: row-major activations (act[0] stride 104, others 72); weights:
// forward images. Hidden layers write ReLU(bf16) into act[l+1]; the output
// layer returns its 16x8 tile (cols 0..2 valid) in y.
__device__ __forceinline__ void forward16(const uint16_t* fwd, uint16_t* const* act, int r0, int lane, float* y) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll 1
    for (int l = 0; l < kLayers; ++l) {
        const int K = LayerK(l);
        const int sa = l == 0 ? kStrideX : kStrideH;
        const uint16_t* W = fwd + FwdOffset(l);
        const int sw = K + kPad;
        if (l + 1 < kLayers) {
            float acc[8][4];
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
            for (int kk = 0; kk < K / 16; ++kk) {
                uint32_t a[4];
                ldsm4(a, a_addr(act[l], sa, r0, 16 * kk, lane));
#pragma unroll
                for (int np = 0; np < 4; ++np) {
                    uint32_t b[4];
                    ldsm4(b, b_addr(W, sw, 16 * np, 16 * kk, lane));
                    mma(acc[2 * np], a, b[0], b[1]);
                    mma(acc[2 * np + 1], a, b[2], b[3]);
                }
            }
            uint16_t* out = act[l + 1];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int col = 8 * nt + 2 * t;
                *reinterpret_cast<uint32_t*>(out + (size_t)(r0 + g) * kStrideH + col) =
                    pack2(fmaxf(acc[nt][0], 0.0f), fmaxf(acc[nt][1], 0.0f));
                *reinterpret_cast<uint32_t*>(out + (size_t)(r0 + g + 8) * kStrideH + col) =
                    pack2(fmaxf(acc[nt][2], 0.0f), fmaxf(acc[nt][3], 0.0f));
            }
        } else {
            y[0] = y[1] = y[2] = y[3] = 0.0f;
            for (int kk = 0; kk < K / 16; ++kk) {
                uint32_t a[4], b[2];
                ldsm4(a, a_addr(act[l], sa, r0, 16 * kk, lane));
                ldsm2(b, b_addr(W, sw, 0, 16 * kk, lane & 15));
                mma(y, a, b[0], b[1]);
            }
        }
        __syncwarp();
    }
}

// Inference forward of one warp's 16 rows with the activations kept in
// registers: the FP32 accumulator fragment of one layer, after ReLU and
// BF16 rounding, is exactly the A fragment of the next (same values as the
// shared-memory round trip of forward16). x: input rows (stride 104).
__device__ __forceinline__ void forward16_reg(const uint16_t* fwd, const uint16_t* x, int lane, float* y) {
    uint32_t a[4][4];
    float acc[8][4];
    // layer 0 from shared memory
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
    {
        const uint16_t* W = fwd + FwdOffset(0);
#pragma unroll
        for (int kk = 0; kk < kIn / 16; ++kk) {
            uint32_t af[4];
            ldsm4(af, a_addr(x, kStrideX, 0, 16 * kk, lane));
#pragma unroll
            for (int np = 0; np < 4; ++np) {
                uint32_t b[4];
                ldsm4(b, b_addr(W, kIn + kPad, 16 * np, 16 * kk, lane));
                mma(acc[2 * np], af, b[0], b[1]);
                mma(acc[2 * np + 1], af, b[2], b[3]);
            }
        }
    }
#pragma unroll 1
    for (int l = 1; l < kLayers; ++l) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            a[kk][0] = pack2(fmaxf(acc[2 * kk][0], 0.f), fmaxf(acc[2 * kk][1], 0.f));
            a[kk][1] = pack2(fmaxf(acc[2 * kk][2], 0.f), fmaxf(acc[2 * kk][3], 0.f));
            a[kk][2] = pack2(fmaxf(acc[2 * kk + 1][0], 0.f), fmaxf(acc[2 * kk + 1][1], 0.f));
            a[kk][3] = pack2(fmaxf(acc[2 * kk + 1][2], 0.f), fmaxf(acc[2 * kk + 1][3], 0.f));
        }
        const uint16_t* W = fwd + FwdOffset(l);
        if (l + 1 < kLayers) {
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int np = 0; np < 4; ++np) {
                    uint32_t b[4];
                    ldsm4(b, b_addr(W, kWidth + kPad, 16 * np, 16 * kk, lane));
                    mma(acc[2 * np], a[kk], b[0], b[1]);
                    mma(acc[2 * np + 1], a[kk], b[2], b[3]);
                }
        } else {
            y[0] = y[1] = y[2] = y[3] = 0.0f;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                uint32_t b[2];
                ldsm2(b, b_addr(W, kWidth + kPad, 0, 16 * kk, lane & 15));
                mma(y, a[kk], b[0], b[1]);
            }
        }
    }
}

__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

// ---- training: forward, loss, backward, weight gradients ----------------
struct TrainArgs {
    Net net;
    const TrainSample* samples;  // sampled mode
    const float4* targets;
    const uint32_t* count;
    const float* raw_feats;      // raw mode (tests): n x 96 features
    const float* raw_targets;    // n x 3
    uint32_t rows;               // rows of this step (batch)
    uint32_t seed;
    float inv_norm;              // 1 / (3 * rows)
};

template <bool kRaw>
__global__ void __launch_bounds__(kThreads) train_kernel(const TrainArgs A) {
    extern __shared__ __align__(16) uint16_t smem[];
    uint16_t* s_fwd = smem;
    uint16_t* s_bwd = s_fwd + kFwdElems;
    uint16_t* s_x = s_bwd + kBwdElems;
    uint16_t* s_h = s_x + kTileRows * kStrideX;           // 5 hidden activations
    uint16_t* s_dz = s_h + 5 * kTileRows * kStrideH;      // one gradient buffer
    float* s_tgt = reinterpret_cast<float*>(s_dz + kTileRows * kStrideH);  // kTileRows x 4
    uint16_t* act[kLayers];
    act[0] = s_x;
    for (int l = 1; l < kLayers; ++l) act[l] = s_h + (l - 1) * kTileRows * kStrideH;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    // weights -> shared (16-byte copies)
    {
        const int4* src = reinterpret_cast<const int4*>(A.net.fwd);
        int4* dst = reinterpret_cast<int4*>(s_fwd);
        for (int i = tid; i < kFwdElems / 8; i += kThreads) dst[i] = src[i];
        const int4* src2 = reinterpret_cast<const int4*>(A.net.bwd);
        int4* dst2 = reinterpret_cast<int4*>(s_bwd);
        for (int i = tid; i < kBwdElems / 8; i += kThreads) dst2[i] = src2[i];
    }
    const uint32_t count = kRaw ? A.rows : (A.count ? *A.count : 0u);
    const uint32_t ntiles = (A.rows + kTileRows - 1) / kTileRows;
    double loss_sum = 0.0;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        __syncthreads();
        // ---- inputs and targets of the tile's rows
        {
            const int row = tid >> 1, half = tid & 1;
            const uint32_t b = tile * kTileRows + row;
            const bool valid = b < A.rows && count > 0;
            uint16_t* xr = s_x + (size_t)row * kStrideX;
            if (!valid) {
                for (int i = half * 48; i < half * 48 + 48; ++i) xr[i] = 0;
                if (half == 0) s_tgt[4 * row] = s_tgt[4 * row + 1] = s_tgt[4 * row + 2] = s_tgt[4 * row + 3] = 0.0f;
            } else if (kRaw) {
                for (int i = half * 48; i < half * 48 + 48; ++i) xr[i] = bf16_bits(A.raw_feats[(size_t)b * kIn + i]);
                if (half == 0) {
                    for (int c = 0; c < 3; ++c) s_tgt[4 * row + c] = A.raw_targets[(size_t)b * 3 + c];
                    s_tgt[4 * row + 3] = 1.0f;
                }
            } else {
                const uint32_t si = pcg_hash(A.seed ^ pcg_hash(b)) % count;
                const TrainSample sm = A.samples[si];
                encode_half(sm.pt, A.net.lo, A.net.hi, half, xr);
                if (half == 0) {
                    const float4 tg = A.targets[si];
                    s_tgt[4 * row] = tg.x;
                    s_tgt[4 * row + 1] = tg.y;
                    s_tgt[4 * row + 2] = tg.z;
                    s_tgt[4 * row + 3] = tg.w;  // 1: valid target
                }
            }
        }
        __syncthreads();
        const int r0 = 16 * warp;
        float y[4];
        forward16(s_fwd, act, r0, lane, y);
        // ---- relative L2 loss and its gradient (bf16) into dz (stride 72)
        {
            const int rows2[2] = {r0 + g, r0 + g + 8};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = rows2[h];
                float gv[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int c = 2 * t + e;
                    const float yy = y[2 * h + e];
                    gv[e] = 0.0f;
                    if (c < kOut && s_tgt[4 * row + 3] > 0.0f) {
                        const float tt = s_tgt[4 * row + c];
                        const float den = yy * yy + kLossEps;
                        const float d = yy - tt;
                        loss_sum += (double)(d * d / den);
                        gv[e] = 2.0f * d / den * A.inv_norm;
                    }
                }
                *reinterpret_cast<uint32_t*>(s_dz + (size_t)row * kStrideH + 2 * t) = pack2(gv[0], gv[1]);
                *reinterpret_cast<uint32_t*>(s_dz + (size_t)row * kStrideH + 8 + 2 * t) = 0u;
            }
        }
        __syncthreads();
        // ---- backward
#pragma unroll 1
        for (int l = kLayers - 1; l >= 0; --l) {
            const int K = LayerK(l), N = LayerN(l), NT = LayerNpad(l) / 8, Nb = LayerNb(l);
            const int sa = l == 0 ? kStrideX : kStrideH;
            // weight gradient dW_l = act_l^T dz_l over the tile's rows
            const int mts = K / 16, tiles = mts * NT;
            for (int tt = warp; tt < tiles; tt += kWarps) {
                const int mt = tt / NT, nt = tt % NT;
                float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int rc = 0; rc < kTileRows / 16; ++rc) {
                    uint32_t a[4], b[2];
                    {   // act^T tile: matrices (rows lo, k lo), (rows lo, k hi), (rows hi, k lo), (rows hi, k hi)
                        const int j = lane >> 3, r = lane & 7;
                        ldsm4t(a, sptr(act[l] + (size_t)(16 * rc + ((j & 2) ? 8 : 0) + r) * sa + 16 * mt +
                                       ((j & 1) ? 8 : 0)));
                    }
                    {   // dz tile (rows lo / hi of one n-tile)
                        const int j = (lane >> 3) & 1, r = lane & 7;
                        ldsm2t(b, sptr(s_dz + (size_t)(16 * rc + 8 * j + r) * kStrideH + 8 * nt));
                    }
                    mma(c, a, b[0], b[1]);
                }
                float* G = A.net.grad + ParamOffset(l);
                const int k0 = 16 * mt + g, n0 = 8 * nt + 2 * t;
                if (n0 < N) {
                    atomicAdd(G + (size_t)k0 * N + n0, c[0]);
                    atomicAdd(G + (size_t)(k0 + 8) * N + n0, c[2]);
                }
                if (n0 + 1 < N) {
                    atomicAdd(G + (size_t)k0 * N + n0 + 1, c[1]);
                    atomicAdd(G + (size_t)(k0 + 8) * N + n0 + 1, c[3]);
                }
            }
            if (l == 0) break;
            // data gradient dA = dz_l W_l^T for this warp's rows, masked by ReLU'
            float acc[8][4];
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
            const uint16_t* Wb = s_bwd + BwdOffset(l);
            const int sw = Nb + kPad;
            for (int nn = 0; nn < Nb / 16; ++nn) {
                uint32_t a[4];
                ldsm4(a, a_addr(s_dz, kStrideH, r0, 16 * nn, lane));
#pragma unroll
                for (int kp = 0; kp < 4; ++kp) {
                    uint32_t b[4];
                    ldsm4(b, b_addr(Wb, sw, 16 * kp, 16 * nn, lane));
                    mma(acc[2 * kp], a, b[0], b[1]);
                    mma(acc[2 * kp + 1], a, b[2], b[3]);
                }
            }
            __syncthreads();  // every warp is done reading dz_l
            const uint16_t* al = act[l];
#pragma unroll
            for (int kt = 0; kt < 8; ++kt) {
                const int col = 8 * kt + 2 * t;
                const float2 m0 = unpack2(*reinterpret_cast<const uint32_t*>(al + (size_t)(r0 + g) * kStrideH + col));
                const float2 m1 =
                    unpack2(*reinterpret_cast<const uint32_t*>(al + (size_t)(r0 + g + 8) * kStrideH + col));
                *reinterpret_cast<uint32_t*>(s_dz + (size_t)(r0 + g) * kStrideH + col) =
                    pack2(m0.x > 0.f ? acc[kt][0] : 0.f, m0.y > 0.f ? acc[kt][1] : 0.f);
                *reinterpret_cast<uint32_t*>(s_dz + (size_t)(r0 + g + 8) * kStrideH + col) =
                    pack2(m1.x > 0.f ? acc[kt][2] : 0.f, m1.y > 0.f ? acc[kt][3] : 0.f);
            }
            __syncthreads();
        }
    }
    // loss: warp sum, one double atomic per warp
    for (int o = 16; o > 0; o >>= 1) loss_sum += __shfl_down_sync(0xFFFFFFFFu, loss_sum, o);
    if (lane == 0 && A.net.loss) atomicAdd(A.net.loss, loss_sum);
}

// ---- inference ----------------------------------------------------------
constexpr int kInferWarps = 8;

template <bool kRaw>
__global__ void __launch_bounds__(32 * kInferWarps) infer_kernel(const Net net, const CachePoint* pts,
                                                                 const uint32_t* count, uint32_t capacity,
                                                                 float4* fb, const float* raw_feats, uint32_t raw_n,
                                                                 float* raw_out) {
    extern __shared__ __align__(16) uint16_t smem[];
    uint16_t* s_fwd = smem;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    uint16_t* xbuf = s_fwd + kFwdElems + warp * (16 * kStrideX);
    {
        const int4* src = reinterpret_cast<const int4*>(net.fwd_avg ? net.fwd_avg : net.fwd);
        int4* dst = reinterpret_cast<int4*>(s_fwd);
        for (int i = tid; i < kFwdElems / 8; i += 32 * kInferWarps) dst[i] = src[i];
    }
    __syncthreads();
    const uint32_t n = kRaw ? raw_n : min(*count, capacity);
    const uint32_t tiles = (n + 15) / 16;
    for (uint32_t tile = blockIdx.x * kInferWarps + warp; tile < tiles; tile += gridDim.x * kInferWarps) {
        const int row = lane >> 1, half = lane & 1;
        const uint32_t q = tile * 16 + row;
        uint16_t* xr = xbuf + row * kStrideX;
        if (q >= n) {
            for (int i = half * 48; i < half * 48 + 48; ++i) xr[i] = 0;
        } else if (kRaw) {
            for (int i = half * 48; i < half * 48 + 48; ++i) xr[i] = bf16_bits(raw_feats[(size_t)q * kIn + i]);
        } else {
            encode_half(pts[q], net.lo, net.hi, half, xr);
        }
        __syncwarp();
        float y[4];
        forward16_reg(s_fwd, xbuf, lane, y);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t qr = tile * 16 + g + 8 * h;
            if (qr >= n) continue;
            if (kRaw) {
                for (int e = 0; e < 2; ++e)
                    if (2 * t + e < kOut) raw_out[(size_t)qr * kOut + 2 * t + e] = y[2 * h + e];
            } else {
                const CachePoint& c = pts[qr];
                const uint32_t pixel = __float_as_uint(c.wo_aux.w);
                const float bt[3] = {c.beta.x, c.beta.y, c.beta.z};
                float* dst = reinterpret_cast<float*>(fb + pixel);
                for (int e = 0; e < 2; ++e) {
                    const int ch = 2 * t + e;
                    if (ch < kOut) {
                        const float v = bt[ch] * fmaxf(y[2 * h + e], 0.0f);
                        if (v > 0.0f) atomicAdd(dst + ch, v);
                    }
                }
            }
        }
        __syncwarp();
    }
}

// Encoding hook: the 96 features of n cache points (tests).
__global__ void encode_kernel(const Net net, const CachePoint* pts, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint16_t row[kIn];
    encode_half(pts[i], net.lo, net.hi, 0, row);
    encode_half(pts[i], net.lo, net.hi, 1, row);
    for (int k = 0; k < kIn; ++k) {
        const uint32_t u = (uint32_t)row[k] << 16;
        out[(size_t)i * kIn + k] = __uint_as_float(u);
    }
}

__device__ __forceinline__ void write_images(const Net& net, int i, float w) {
    int l = 0;
    while (l + 1 < kLayers && i >= ParamOffset(l + 1)) ++l;
    const int N = LayerN(l), K = LayerK(l);
    const int k = (i - ParamOffset(l)) / N, nn = (i - ParamOffset(l)) % N;
    const uint16_t b = bf16_bits(w);
    net.fwd[FwdOffset(l) + nn * (K + kPad) + k] = b;
    net.bwd[BwdOffset(l) + k * (LayerNb(l) + kPad) + nn] = b;
}

// The forward image only (the averaged weights are never trained).
__device__ __forceinline__ void write_fwd_image(uint16_t* fwd, int i, float w) {
    int l = 0;
    while (l + 1 < kLayers && i >= ParamOffset(l + 1)) ++l;
    const int N = LayerN(l), K = LayerK(l);
    const int k = (i - ParamOffset(l)) / N, nn = (i - ParamOffset(l)) % N;
    fwd[FwdOffset(l) + nn * (K + kPad) + k] = bf16_bits(w);
}

// Weight averaging restarts from the current weights: the average is empty
// and the query image holds the weights themselves.
__device__ __forceinline__ void restart_average(const Net& net, int i, float w) {
    if (!net.avg) return;
    net.avg[i] = 0.0f;
    write_fwd_image(net.fwd_avg, i, w);
}

// c3 = 1 - avg_decay^avg_steps (the bias correction of the average)
__global__ void adam_kernel(const Net net, float lr, float c1, float c2, float c3) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x) {
        const float gr = net.grad[i];
        const float m = b1 * net.adam_m[i] + (1.0f - b1) * gr;
        const float v = b2 * net.adam_v[i] + (1.0f - b2) * gr * gr;
        net.adam_m[i] = m;
        net.adam_v[i] = v;
        const float w = net.master[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
        net.master[i] = w;
        net.grad[i] = 0.0f;
        write_images(net, i, w);
        if (net.avg) {
            const float a = net.avg_decay * net.avg[i] + (1.0f - net.avg_decay) * w;
            net.avg[i] = a;
            write_fwd_image(net.fwd_avg, i, a / c3);
        }
    }
}

__global__ void init_kernel(const Net net, uint64_t seed) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x) {
        int l = 0;
        while (l + 1 < kLayers && i >= ParamOffset(l + 1)) ++l;
        const float bound = sqrtf(6.0f / (float)LayerK(l));
        const uint32_t h = pcg_hash((uint32_t)i ^ pcg_hash((uint32_t)seed ^ pcg_hash((uint32_t)(seed >> 32))));
        const float u = (float)(h >> 8) * (1.0f / 16777216.0f);
        const float w = (2.0f * u - 1.0f) * bound;
        net.master[i] = w;
        net.adam_m[i] = 0.0f;
        net.adam_v[i] = 0.0f;
        net.grad[i] = 0.0f;
        write_images(net, i, w);
        restart_average(net, i, w);
    }
}

__global__ void images_kernel(const Net net) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x) {
        write_images(net, i, net.master[i]);
        restart_average(net, i, net.master[i]);
    }
}

size_t train_smem() {
    return sizeof(uint16_t) * ((size_t)kFwdElems + kBwdElems + (size_t)kTileRows * kStrideX +
                               6 * (size_t)kTileRows * kStrideH) +
           sizeof(float) * 4 * kTileRows;
}
size_t infer_smem() { return sizeof(uint16_t) * ((size_t)kFwdElems + (size_t)kInferWarps * 16 * kStrideX); }

template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

size_t TrainSmemBytes() { return train_smem(); }
size_t InferSmemBytes() { return infer_smem(); }

cudaError_t InitNet(const Net& net, uint64_t seed, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(net.fwd, 0, sizeof(uint16_t) * kFwdElems, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net.bwd, 0, sizeof(uint16_t) * kBwdElems, s);
    if (e == cudaSuccess && net.fwd_avg) e = cudaMemsetAsync(net.fwd_avg, 0, sizeof(uint16_t) * kFwdElems, s);
    if (e != cudaSuccess) return e;
    init_kernel<<<(kNumParams + 255) / 256, 256, 0, s>>>(net, seed);
    return cudaGetLastError();
}

cudaError_t RewriteImages(const Net& net, cudaStream_t s) {
    images_kernel<<<(kNumParams + 255) / 256, 256, 0, s>>>(net);
    return cudaGetLastError();
}

cudaError_t Infer(const Net& net, const CachePoint* pts, const uint32_t* count, uint32_t capacity, float4* fb,
                  int grid, cudaStream_t s) {
    cudaError_t e = allow_smem(infer_kernel<false>, infer_smem());
    if (e != cudaSuccess) return e;
    infer_kernel<false><<<grid, 32 * kInferWarps, infer_smem(), s>>>(net, pts, count, capacity, fb, nullptr, 0,
                                                                      nullptr);
    return cudaGetLastError();
}

cudaError_t InferRaw(const Net& net, const float* feats, uint32_t n, float* out, cudaStream_t s) {
    cudaError_t e = allow_smem(infer_kernel<true>, infer_smem());
    if (e != cudaSuccess) return e;
    const uint32_t tiles = (n + 15) / 16;
    const int grid = (int)((tiles + kInferWarps - 1) / kInferWarps);
    infer_kernel<true><<<grid > 0 ? grid : 1, 32 * kInferWarps, infer_smem(), s>>>(net, nullptr, nullptr, 0, nullptr,
                                                                                   feats, n, out);
    return cudaGetLastError();
}

static cudaError_t launch_adam(Net& net, float lr, cudaStream_t s) {
    net.step += 1;
    const double c1 = 1.0 - std::pow(0.9, (double)net.step), c2 = 1.0 - std::pow(0.99, (double)net.step);
    double c3 = 1.0;
    if (net.avg) {
        net.avg_steps += 1;
        c3 = 1.0 - std::pow((double)net.avg_decay, (double)net.avg_steps);
    }
    adam_kernel<<<(kNumParams + 255) / 256, 256, 0, s>>>(net, lr, (float)c1, (float)c2, (float)c3);
    return cudaGetLastError();
}

cudaError_t TrainStep(Net& net, const TrainSample* smp, const float4* targets, const uint32_t* count, uint32_t batch,
                      uint64_t seed, float lr, int grid, cudaStream_t s) {
    cudaError_t e = allow_smem(train_kernel<false>, train_smem());
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(net.loss, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    TrainArgs A{};
    A.net = net;
    A.samples = smp;
    A.targets = targets;
    A.count = count;
    A.rows = batch;
    A.seed = (uint32_t)(seed ^ (seed >> 32));
    A.inv_norm = 1.0f / (3.0f * (float)batch);
    train_kernel<false><<<grid, kThreads, train_smem(), s>>>(A);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_adam(net, lr, s);
}

cudaError_t GradRaw(const Net& net, const float* feats, const float* targets, uint32_t n, cudaStream_t s) {
    cudaError_t e = allow_smem(train_kernel<true>, train_smem());
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(net.grad, 0, sizeof(float) * kNumParams, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net.loss, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    TrainArgs A{};
    A.net = net;
    A.raw_feats = feats;
    A.raw_targets = targets;
    A.rows = n;
    A.inv_norm = 1.0f / (3.0f * (float)n);
    const int tiles = (int)((n + kTileRows - 1) / kTileRows);
    train_kernel<true><<<tiles > 0 ? tiles : 1, kThreads, train_smem(), s>>>(A);
    return cudaGetLastError();
}

cudaError_t AdamRaw(Net& net, float lr, cudaStream_t s) { return launch_adam(net, lr, s); }

cudaError_t EncodeRaw(const Net& net, const CachePoint* pts, uint32_t n, float* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    encode_kernel<<<(n + 127) / 128, 128, 0, s>>>(net, pts, n, out);
    return cudaGetLastError();
}

}  // namespace NRC
}  // namespace Foundation
