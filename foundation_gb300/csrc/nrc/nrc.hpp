// nrc.hpp — host-visible interface of the neural radiance cache (BF16 MLP).
//
// Network 96 -> 64 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU hidden layers, linear
// output, no biases (the fully fused MLP of Müller, Rousselle, Novák &
// Keller, "Real-time Neural Radiance Caching for Path Tracing", SIGGRAPH
// 2021). BF16 weights and activations, FP32 accumulation on the tensor cores,
// FP32 master weights and Adam state, relative-L2 loss. Training runs on the
// fifth-generation tensor cores (tcgen05, accumulators in tensor memory,
// train_umma.cu); inference on warp-level mma.sync m16n8k16 (mlp.cu), whose
// 16-row register-resident tiles suit the scattered queries of a frame.
//
// Weight layouts in global memory are the shared-memory images the kernels
// copy verbatim:
//  * inference: per layer a "forward" image WT[Npad][K + 8] (B operand of
//    x * W), bf16 with 8 elements of row padding against bank conflicts
//    (ldmatrix);
//  * training (tcgen05): per layer the forward B operand W^T[Npad][K]
//    (Npad = 16 for the 3-wide output) and, for layers 1..5, the backward B
//    operand W[K][Nb] (Nb = 16 for the output layer), in the row-group-major
//    core-matrix layout of umma.cuh; padding entries are zero.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace Foundation {
namespace NRC {

constexpr int kLayers = 6;
constexpr int kIn = 96;
constexpr int kWidth = 64;
constexpr int kOut = 3;
constexpr int kPad = 8;

__host__ __device__ constexpr int LayerK(int l) { return l == 0 ? kIn : kWidth; }
__host__ __device__ constexpr int LayerN(int l) { return l == kLayers - 1 ? kOut : kWidth; }
__host__ __device__ constexpr int LayerNpad(int l) { return l == kLayers - 1 ? 8 : kWidth; }   // forward N tiles
__host__ __device__ constexpr int FwdElems(int l) { return LayerNpad(l) * (LayerK(l) + kPad); }
__host__ __device__ constexpr int ParamOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += LayerK(i) * LayerN(i);
    return o;
}
constexpr int kNumParams = ParamOffset(kLayers);  // 22,720
__host__ __device__ constexpr int FwdOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += FwdElems(i);
    return o;
}
constexpr int kFwdElems = FwdOffset(kLayers);

// tcgen05 training images (elements): forward W^T[UmmaN(l)][K], backward
// W[K][UmmaN(l)] for l >= 1
__host__ __device__ constexpr int UmmaN(int l) { return l == kLayers - 1 ? 16 : kWidth; }
__host__ __device__ constexpr int UFwdOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += UmmaN(i) * LayerK(i);
    return o;
}
__host__ __device__ constexpr int UBwdOffset(int l) {  // l >= 1
    int o = 0;
    for (int i = 1; i < l; ++i) o += LayerK(i) * UmmaN(i);
    return o;
}
constexpr int kUFwdElems = UFwdOffset(kLayers);  // 23,552
constexpr int kUBwdElems = UBwdOffset(kLayers);  // 17,408

// Raw record of one cache point (features are derived on the fly).
struct CachePoint {
    float4 p_rough;   // world position, roughness (GGX alpha; 1 for Lambert)
    float4 wo_aux;    // unit outgoing direction, w = pixel / slot bits
    float4 n_pad;     // unit shading normal
    float4 albedo;    // rgb albedo / specular colour
    float4 beta;      // rgb path throughput at the point
};

struct TrainSample {
    CachePoint pt;    // pt.wo_aux.w = training-path slot
    float4 before;    // rgb radiance the path had collected before this vertex
};

struct Net {
    uint16_t* fwd;    // bf16 forward images (kFwdElems)
    uint16_t* ufwd;   // bf16 tcgen05 forward images (kUFwdElems)
    uint16_t* ubwd;   // bf16 tcgen05 backward images (kUBwdElems)
    float* master;    // fp32 weights, row-major W[K][N] per layer (kNumParams)
    float* adam_m;
    float* adam_v;
    float* grad;      // fp32 gradient accumulator (kNumParams)
    double* loss;     // [0] running sum of the loss of the current step
    uint32_t step;    // Adam steps taken
    // weight averaging (queries only): fp32 moving average of the iterates
    // and the bf16 forward image of avg / (1 - decay^avg_steps); null: off
    float* avg;
    uint16_t* fwd_avg;
    float avg_decay;
    uint32_t avg_steps;
    float lo[3], hi[3];  // scene box for the position encoding
};

// Host API (launches on `s`).
cudaError_t InitNet(const Net& net, uint64_t seed, cudaStream_t s);        // He-uniform init + images
// Queries evaluate the averaged weights when averaging is on, else the latest.
cudaError_t Infer(const Net& net, const CachePoint* pts, const uint32_t* count, uint32_t capacity,
                  float4* fb, int grid, cudaStream_t s);                     // fb[pixel] += beta * max(0, f(x))
cudaError_t InferRaw(const Net& net, const float* feats, uint32_t n, float* out, cudaStream_t s);  // test hook
// One training step on `batch` samples drawn (with replacement, by hash)
// from the first *count samples; accumulates the gradient, then Adam. A
// tensor-core completion wait that runs out latches the timeout bit in
// *status and ends the step early.
cudaError_t TrainStep(Net& net, const TrainSample* smp, const float4* targets, const uint32_t* count,
                      uint32_t batch, uint64_t seed, float lr, uint32_t* status, cudaStream_t s);
// Test hook: gradient of the loss on explicit features / targets (no Adam).
cudaError_t GradRaw(const Net& net, const float* feats, const float* targets, uint32_t n, uint32_t* status,
                    cudaStream_t s);
cudaError_t AdamRaw(Net& net, float lr, cudaStream_t s);
// The step's gradient alone (train_umma.cu): accumulates into net.grad.
cudaError_t LaunchTrainUmma(const Net& net, const TrainSample* smp, const float4* targets, const uint32_t* count,
                            uint32_t batch, uint64_t seed, uint32_t* status, cudaStream_t s);
// bf16 images from the fp32 master weights; restarts the weight average
// (the caller zeroes net.avg_steps)
cudaError_t RewriteImages(const Net& net, cudaStream_t s);
// Test hook: the bf16 input features (widened to float) of n cache points.
cudaError_t EncodeRaw(const Net& net, const CachePoint* pts, uint32_t n, float* out, cudaStream_t s);
size_t TrainSmemBytes();
size_t InferSmemBytes();

}  // namespace NRC
}  // namespace Foundation
