// mlp.cu — the radiance cache's BF16 MLP outside training (sm_103a):
// inference, the encoding hook, Adam, initialisation and the weight images.
//
// Inference runs on warp-level mma.sync.m16n8k16 BF16 x BF16 -> FP32 with
// operands fetched by ldmatrix: a warp owns 16 query rows and keeps the
// activations in registers (the accumulator fragment of one layer, after
// ReLU and BF16 rounding, is the A fragment of the next), which suits the
// scattered, variable-length query batches of a frame. Training runs on the
// fifth-generation tensor cores in 128-row tiles (train_umma.cu).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "mlp_common.cuh"
#include "nrc.hpp"
#include "umma.cuh"

namespace Foundation {
namespace NRC {
namespace {

constexpr int kStrideX = kIn + kPad;    // 104
constexpr int kStrideH = kWidth + kPad; // 72

__device__ __forceinline__ uint32_t sptr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm4(uint32_t* r, uint32_t a) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm2(uint32_t* r, uint32_t a) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
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

// Inference forward of one warp's 16 rows with the activations kept in
// registers: the FP32 accumulator fragment of one layer, after ReLU and
// BF16 rounding, is exactly the A fragment of the next (same values as the
// shared-memory round trip of the tile-wide forward). x: input rows (stride
// 104).
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
    // tcgen05 training images: W^T[n][k] and, past layer 0, W[k][n] (umma.cuh layout)
    net.ufwd[UFwdOffset(l) + Umma::canon_offset(nn, k, K) / 2] = b;
    if (l > 0) net.ubwd[UBwdOffset(l) + Umma::canon_offset(k, nn, UmmaN(l)) / 2] = b;
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

size_t infer_smem() { return sizeof(uint16_t) * ((size_t)kFwdElems + (size_t)kInferWarps * 16 * kStrideX); }

template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

size_t InferSmemBytes() { return infer_smem(); }

cudaError_t InitNet(const Net& net, uint64_t seed, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(net.fwd, 0, sizeof(uint16_t) * kFwdElems, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net.ufwd, 0, sizeof(uint16_t) * kUFwdElems, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net.ubwd, 0, sizeof(uint16_t) * kUBwdElems, s);
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
                      uint64_t seed, float lr, uint32_t* status, cudaStream_t s) {
    cudaError_t e = LaunchTrainUmma(net, smp, targets, count, batch, seed, status, s);
    if (e != cudaSuccess) return e;
    return launch_adam(net, lr, s);
}

cudaError_t AdamRaw(Net& net, float lr, cudaStream_t s) { return launch_adam(net, lr, s); }

cudaError_t EncodeRaw(const Net& net, const CachePoint* pts, uint32_t n, float* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    encode_kernel<<<(n + 127) / 128, 128, 0, s>>>(net, pts, n, out);
    return cudaGetLastError();
}

}  // namespace NRC
}  // namespace Foundation
