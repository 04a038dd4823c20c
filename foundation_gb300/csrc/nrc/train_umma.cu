// train_umma.cu — one optimiser step of the radiance cache's MLP on the
// fifth-generation tensor cores (tcgen05, sm_103a): input encoding, forward,
// relative-L2 loss, backward and weight gradients of 128-row tiles, fused in
// one kernel.
//
// A CTA takes tiles of kRows = 128 samples, the M of one tcgen05 MMA:
//  * the tcgen05 weight images (nrc.hpp) arrive once in shared memory by two
//    bulk copies (TMA) that run under the first tile's input encoding;
//    each tile's encoded inputs X, the five hidden activations H1..H5 and one
//    gradient buffer dZ stay there in the core-matrix layout of umma.cuh, so
//    every GEMM of the step reads its operands from shared memory;
//  * forward: Z_l = H_l W_l (H_0 = X) accumulates in tensor memory; the
//    epilogue (8 warps, each a quarter of the lanes and half the columns)
//    applies ReLU, rounds to BF16 and writes H_{l+1};
//  * loss: the 3 outputs of each row, relative L2 (y - t)^2 / (y^2 + eps)
//    with the denominator held constant (Müller et al. 2021), give dZ_5;
//  * backward, per layer l = 5 .. 0, one commit covers two GEMMs:
//      dW_l += H_l^T dZ_l   (M = features padded to 128, K = the 128 rows:
//                            both operands MN-major, the transposed reads of
//                            the same shared arrays),
//      dH_l  = dZ_l W_l^T   (M = 128 rows), and the epilogue masks dH_l by
//                            H_l > 0 into dZ_{l-1} (BF16);
//  * the weight gradients stay in tensor memory for all of a CTA's tiles and
//    are added to the global FP32 gradient once, with vector atomics.
// One elected thread issues every MMA and commits it to one mbarrier; each
// wait for it is bounded and, when it runs out, the step latches the
// timeout bit of the status word, stops, and still releases its tensor
// memory. Adam (mlp.cu) then applies the gradient.
//
// Tensor memory (512 columns): Z at column 0 (64), dH at 64 (64), dW_l at
// 128 + 64 l (layer 5: 16 columns).
#include <cuda_bf16.h>

#include "../rt/device_scene.hpp"
#include "mlp_common.cuh"
#include "nrc.hpp"
#include "umma.cuh"

namespace Foundation {
namespace NRC {
namespace {

using namespace Umma;

constexpr uint32_t kRows = 128;
constexpr uint32_t kThreads = 256;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kColZ = 0, kColDH = 64, kColDW = 128;
constexpr uint32_t kWaitLimit = 1u << 22;

// shared-memory map (bytes, each region 1024-aligned)
constexpr uint32_t kSmWf = 0;                                 // forward images, layers 0..5
constexpr uint32_t kSmWb = kSmWf + 2 * kUFwdElems;            // backward images, layers 1..5
constexpr uint32_t kSmX = kSmWb + 2 * kUBwdElems;             // X [128][96]
constexpr uint32_t kSmH = kSmX + 2 * kRows * kIn;             // H1..H5 [128][64]
constexpr uint32_t kHBytes = 2 * kRows * kWidth;
constexpr uint32_t kSmDz = kSmH + 5 * kHBytes;                // dZ [128][64] (layer 5: [128][16])
constexpr uint32_t kSmTgt = kSmDz + kHBytes;                  // float4 per row
constexpr uint32_t kSmBytes = kSmTgt + 16 * kRows;
static_assert(kSmWb % 1024 == 0 && kSmX % 1024 == 0 && kSmH % 1024 == 0 && kSmDz % 1024 == 0, "alignment");
// the padded M = 128 reads of the weight-gradient GEMMs run past X by 512
// bytes (into H1) and past H5 by 1024 bytes (into dZ): both stay inside
static_assert(kSmBytes <= 227 * 1024, "shared memory");

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
    uint32_t* status;            // timeout bit on a wait that ran out
};

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xFFFF0000u); }

// K-major operand of a row-group-major [rows][cols] array: K steps of 16
// are 256 bytes apart.
__device__ __forceinline__ uint64_t kmajor(uint32_t saddr, uint32_t cols) {
    return smem_desc(saddr, 128u, cols / 8u * 128u);
}
// MN-major operand (the transposed read): the K (row) steps of 16 are
// 2 * cols / 8 * 128 bytes apart.
__device__ __forceinline__ uint64_t mnmajor(uint32_t saddr, uint32_t cols) {
    return smem_desc(saddr, cols / 8u * 128u, 128u);
}

// Row r's 48 features of one half (tid & 1) into the X array.
template <bool kRaw>
__device__ __forceinline__ void stage_inputs(const TrainArgs& A, unsigned char* smem, uint32_t tile, uint32_t count,
                                             uint32_t tid) {
    const uint32_t r = tid >> 1, half = tid & 1;
    const uint32_t b = tile * kRows + r;
    uint16_t f[96];
    float4 tg = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool valid = b < A.rows && count > 0;
    if (valid && kRaw) {
        const float* src = A.raw_feats + (size_t)b * kIn;
        if (half == 0) {
#pragma unroll
            for (int i = 0; i < 48; ++i) f[i] = bf16_bits(src[i]);
            tg = make_float4(A.raw_targets[3 * (size_t)b], A.raw_targets[3 * (size_t)b + 1],
                             A.raw_targets[3 * (size_t)b + 2], 1.0f);
        } else {
#pragma unroll
            for (int i = 48; i < 96; ++i) f[i] = bf16_bits(src[i]);
        }
    } else if (valid) {
        const uint32_t si = pcg_hash(A.seed ^ pcg_hash(b)) % count;
        const CachePoint pt = A.samples[si].pt;
        encode_half(pt, A.net.lo, A.net.hi, (int)half, f);
        if (half == 0) tg = A.targets[si];
    } else {
#pragma unroll
        for (int i = 0; i < 96; ++i) f[i] = 0;
    }
    unsigned char* x = smem + kSmX;
    if (half == 0) {
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            uint4 v;
            v.x = (uint32_t)f[8 * j] | ((uint32_t)f[8 * j + 1] << 16);
            v.y = (uint32_t)f[8 * j + 2] | ((uint32_t)f[8 * j + 3] << 16);
            v.z = (uint32_t)f[8 * j + 4] | ((uint32_t)f[8 * j + 5] << 16);
            v.w = (uint32_t)f[8 * j + 6] | ((uint32_t)f[8 * j + 7] << 16);
            *reinterpret_cast<uint4*>(x + canon_offset(r, 8 * j, kIn)) = v;
        }
        reinterpret_cast<float4*>(smem + kSmTgt)[r] = tg;
    } else {
#pragma unroll
        for (int j = 6; j < 12; ++j) {
            uint4 v;
            v.x = (uint32_t)f[8 * j] | ((uint32_t)f[8 * j + 1] << 16);
            v.y = (uint32_t)f[8 * j + 2] | ((uint32_t)f[8 * j + 3] << 16);
            v.z = (uint32_t)f[8 * j + 4] | ((uint32_t)f[8 * j + 5] << 16);
            v.w = (uint32_t)f[8 * j + 6] | ((uint32_t)f[8 * j + 7] << 16);
            *reinterpret_cast<uint4*>(x + canon_offset(r, 8 * j, kIn)) = v;
        }
    }
}

// Shared-memory writes of the epilogue -> visible to the next MMAs.
__device__ __forceinline__ void publish_smem() {
    fence_smem_to_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
}

template <bool kRaw>
__global__ void __launch_bounds__(kThreads, 1) train_umma_kernel(const TrainArgs A) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t s_mbar;    // MMA completion
    __shared__ uint64_t s_mbar_w;  // weight images in shared memory
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t quarter = warp & 3, chalf = warp >> 2;
    const uint32_t row = 32 * quarter + lane;  // the tile row (tensor-memory lane) of this thread's epilogue
    const uint32_t sbase = smem_u32(smem);

    if (tid == 0) {
        mbar_init(&s_mbar, 1);
        mbar_init(&s_mbar_w, 1);
        s_abort = 0;
        // weight images -> shared memory by two bulk copies, under the first
        // tile's input encoding
        mbar_expect_tx(&s_mbar_w, 2 * (kUFwdElems + kUBwdElems));
        bulk_g2s(smem + kSmWf, A.net.ufwd, 2 * kUFwdElems, &s_mbar_w);
        bulk_g2s(smem + kSmWb, A.net.ubwd, 2 * kUBwdElems, &s_mbar_w);
    }
    if (warp == 0) tmem_alloc(&s_tmem, kTmemCols);
    bool weights_ready = false;  // thread 0: the bulk copies have landed
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = s_tmem;
    const uint32_t count = kRaw ? A.rows : (A.count ? *A.count : 0u);
    const uint32_t ntiles = (A.rows + kRows - 1) / kRows;
    uint32_t phase = 0;
    bool alive = true, first = true;
    double loss = 0.0;

    // All threads: waits for the last commit; false (for every thread) when
    // the wait ran out anywhere in the CTA.
    auto wait_mma = [&]() -> bool {
        const bool ok = mbar_wait(&s_mbar, phase & 1u, kWaitLimit);
        phase++;
        if (!ok) s_abort = 1;
        __syncthreads();
        fence_after_sync();
        return s_abort == 0;
    };

    for (uint32_t tile = blockIdx.x; tile < ntiles && alive; tile += gridDim.x) {
        stage_inputs<kRaw>(A, smem, tile, count, tid);
        publish_smem();
        // ---- forward ----------------------------------------------------
        for (int l = 0; l < kLayers && alive; ++l) {
            const uint32_t K = LayerK(l), N = UmmaN(l);
            if (tid == 0) {
                if (!weights_ready) weights_ready = mbar_wait(&s_mbar_w, 0, kWaitLimit);
                if (weights_ready) {
                    const uint32_t a0 = sbase + (l == 0 ? kSmX : kSmH + (l - 1) * kHBytes);
                    const uint32_t b0 = sbase + kSmWf + 2 * UFwdOffset(l);
                    const uint32_t idesc = instr_desc_bf16(128, N, false, false);
                    for (uint32_t k = 0; k < K / 16; ++k)
                        mma_bf16(tmem + kColZ, kmajor(a0 + 256 * k, K), kmajor(b0 + 256 * k, K), idesc, k > 0);
                    mma_commit(&s_mbar);
                } else {
                    s_abort = 1;          // the copies never landed: complete the phase
                    mbar_arrive(&s_mbar);  // without an MMA and stop
                }
            }
            alive = wait_mma();
            if (!alive) break;
            if (l + 1 < kLayers) {
                uint32_t v[32];
                tmem_ld16(tmem_addr(tmem, 32 * quarter, kColZ + 32 * chalf), v);
                tmem_ld16(tmem_addr(tmem, 32 * quarter, kColZ + 32 * chalf + 16), v + 16);
                tmem_ld_wait();
                unsigned char* h = smem + kSmH + l * kHBytes;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    uint4 o;
                    o.x = bf16x2(fmaxf(__uint_as_float(v[8 * j]), 0.f), fmaxf(__uint_as_float(v[8 * j + 1]), 0.f));
                    o.y = bf16x2(fmaxf(__uint_as_float(v[8 * j + 2]), 0.f), fmaxf(__uint_as_float(v[8 * j + 3]), 0.f));
                    o.z = bf16x2(fmaxf(__uint_as_float(v[8 * j + 4]), 0.f), fmaxf(__uint_as_float(v[8 * j + 5]), 0.f));
                    o.w = bf16x2(fmaxf(__uint_as_float(v[8 * j + 6]), 0.f), fmaxf(__uint_as_float(v[8 * j + 7]), 0.f));
                    *reinterpret_cast<uint4*>(h + canon_offset(row, 32 * chalf + 8 * j, kWidth)) = o;
                }
            } else if (chalf == 0) {
                // outputs -> loss and its gradient dZ_5 ([128][16], columns 3.. zero)
                uint32_t v[16];
                tmem_ld16(tmem_addr(tmem, 32 * quarter, kColZ), v);
                tmem_ld_wait();
                const float4 tg = reinterpret_cast<const float4*>(smem + kSmTgt)[row];
                float g[3] = {0.f, 0.f, 0.f};
                if (tg.w > 0.0f) {
                    const float t3[3] = {tg.x, tg.y, tg.z};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float y = __uint_as_float(v[c]);
                        const float den = y * y + kLossEps;
                        const float d = y - t3[c];
                        loss += (double)(d * d / den);
                        g[c] = 2.0f * d / den * A.inv_norm;
                    }
                }
                unsigned char* dz = smem + kSmDz;
                *reinterpret_cast<uint4*>(dz + canon_offset(row, 0, 16)) =
                    make_uint4(bf16x2(g[0], g[1]), bf16x2(g[2], 0.f), 0u, 0u);
                *reinterpret_cast<uint4*>(dz + canon_offset(row, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
            }
            publish_smem();
        }
        // ---- backward ---------------------------------------------------
        for (int l = kLayers - 1; l >= 0 && alive; --l) {
            const uint32_t F = LayerK(l), Nb = UmmaN(l);
            if (tid == 0) {
                const uint32_t h0 = sbase + (l == 0 ? kSmX : kSmH + (l - 1) * kHBytes);
                const uint32_t dz0 = sbase + kSmDz;
                // dW_l (+)= H_l^T dZ_l over this tile's rows
                const uint32_t idesc_w = instr_desc_bf16(128, Nb, true, true);
                for (uint32_t k = 0; k < kRows / 16; ++k)
                    mma_bf16(tmem + kColDW + 64 * l, mnmajor(h0 + 2 * (F / 8 * 128) * k, F),
                             mnmajor(dz0 + 2 * (Nb / 8 * 128) * k, Nb), idesc_w, !first || k > 0);
                if (l > 0) {
                    // dH_l = dZ_l W_l^T
                    const uint32_t b0 = sbase + kSmWb + 2 * UBwdOffset(l);
                    const uint32_t idesc_a = instr_desc_bf16(128, kWidth, false, false);
                    for (uint32_t k = 0; k < Nb / 16; ++k)
                        mma_bf16(tmem + kColDH, kmajor(dz0 + 256 * k, Nb), kmajor(b0 + 256 * k, Nb), idesc_a, k > 0);
                }
                mma_commit(&s_mbar);
            }
            alive = wait_mma();
            if (!alive || l == 0) break;
            // dZ_{l-1} = dH_l masked by H_l > 0 (BF16), over dZ_l
            uint32_t v[32];
            tmem_ld16(tmem_addr(tmem, 32 * quarter, kColDH + 32 * chalf), v);
            tmem_ld16(tmem_addr(tmem, 32 * quarter, kColDH + 32 * chalf + 16), v + 16);
            tmem_ld_wait();
            const unsigned char* h = smem + kSmH + (l - 1) * kHBytes;
            unsigned char* dz = smem + kSmDz;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t off = canon_offset(row, 32 * chalf + 8 * j, kWidth);
                const uint4 a = *reinterpret_cast<const uint4*>(h + off);
                const uint32_t aw[4] = {a.x, a.y, a.z, a.w};
                uint32_t o[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float d0 = bf16_lo(aw[e]) > 0.f ? __uint_as_float(v[8 * j + 2 * e]) : 0.f;
                    const float d1 = bf16_hi(aw[e]) > 0.f ? __uint_as_float(v[8 * j + 2 * e + 1]) : 0.f;
                    o[e] = bf16x2(d0, d1);
                }
                *reinterpret_cast<uint4*>(dz + off) = make_uint4(o[0], o[1], o[2], o[3]);
            }
            publish_smem();
        }
        first = false;
    }
    // ---- the CTA's weight gradients -> global (FP32 vector atomics) --------
    if (alive && !first) {
#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            const uint32_t F = LayerK(l), N = LayerN(l);
            if (32 * quarter >= F) continue;  // whole warp: rows past the layer's inputs are padding
            float* G = A.net.grad + ParamOffset(l) + (size_t)row * N;
            if (l + 1 < kLayers) {
                uint32_t v[32];
                tmem_ld16(tmem_addr(tmem, 32 * quarter, kColDW + 64 * l + 32 * chalf), v);
                tmem_ld16(tmem_addr(tmem, 32 * quarter, kColDW + 64 * l + 32 * chalf + 16), v + 16);
                tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    atomicAdd(reinterpret_cast<float4*>(G + 32 * chalf + 4 * j),
                              make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                                          __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3])));
            } else if (chalf == 0) {
                uint32_t v[16];
                tmem_ld16(tmem_addr(tmem, 32 * quarter, kColDW + 64 * l), v);
                tmem_ld_wait();
                for (int c = 0; c < 3; ++c) atomicAdd(G + c, __uint_as_float(v[c]));
            }
        }
    }
    if (!alive) {
        if (lane == 0 && A.status) atomicOr(A.status, Foundation::RT::kStatusTimeout);
        // let the MMAs of the unfinished phase and the weight copies drain
        // (bounded) before the tensor memory is released
        if (tid == 0) {
            (void)mbar_wait(&s_mbar, (phase - 1) & 1u, kWaitLimit);
            if (!weights_ready) (void)mbar_wait(&s_mbar_w, 0, kWaitLimit);
        }
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xFFFFFFFFu, loss, o);
    if (lane == 0 && A.net.loss && loss != 0.0) atomicAdd(A.net.loss, loss);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

template <typename K>
cudaError_t allow_smem(K kernel) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmBytes);
}

}  // namespace

size_t TrainSmemBytes() { return kSmBytes; }

// One CTA per 128-row tile (a single wave for the 16,384-sample batches).
static int train_grid(uint32_t rows) { return (int)((rows + kRows - 1) / kRows); }

cudaError_t LaunchTrainUmma(const Net& net, const TrainSample* smp, const float4* targets, const uint32_t* count,
                            uint32_t batch, uint64_t seed, uint32_t* status, cudaStream_t s) {
    cudaError_t e = allow_smem(train_umma_kernel<false>);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(net.loss, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    if (batch == 0) return cudaSuccess;
    TrainArgs A{};
    A.net = net;
    A.samples = smp;
    A.targets = targets;
    A.count = count;
    A.rows = batch;
    A.seed = (uint32_t)(seed ^ (seed >> 32));
    A.inv_norm = 1.0f / (3.0f * (float)batch);
    A.status = status;
    train_umma_kernel<false><<<train_grid(batch), kThreads, kSmBytes, s>>>(A);
    return cudaGetLastError();
}

cudaError_t GradRaw(const Net& net, const float* feats, const float* targets, uint32_t n, uint32_t* status,
                    cudaStream_t s) {
    cudaError_t e = allow_smem(train_umma_kernel<true>);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(net.grad, 0, sizeof(float) * kNumParams, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net.loss, 0, sizeof(double), s);
    if (e != cudaSuccess || n == 0) return e;
    TrainArgs A{};
    A.net = net;
    A.raw_feats = feats;
    A.raw_targets = targets;
    A.rows = n;
    A.inv_norm = 1.0f / (3.0f * (float)n);
    A.status = status;
    train_umma_kernel<true><<<train_grid(n), kThreads, kSmBytes, s>>>(A);
    return cudaGetLastError();
}

}  // namespace NRC
}  // namespace Foundation
