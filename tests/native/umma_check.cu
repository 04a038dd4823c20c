// umma_check.cu — TEST HARNESS: one CTA runs the tensor-core primitives of
// foundation_gb300/csrc/nrc/umma.cuh (tensor-memory allocation, shared-memory
// descriptors, tcgen05.mma kind::f16, commit, tensor-memory loads) on small
// BF16 matrices so a test can compare the products with the host's:
//   mode 0 (both operands K-major): D[128][N] = A[128][K] x B[N][K]^T
//   mode 1 (both operands MN-major, the weight-gradient use):
//          D[128][N] = H[128][F]^T x G[128][N], rows f < F of D valid
//          (the M = 128 tile reads past F into the next row group, which the
//          shared-memory slack keeps in bounds)
// Inputs are row-major BF16 bit patterns on the host; D comes back as FP32.
// status: 0 ok, 1 the completion wait ran out, 2 bad sizes, 3 CUDA error.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../foundation_gb300/csrc/nrc/umma.cuh"

using namespace Foundation::NRC::Umma;

namespace {

constexpr uint32_t kWaitLimit = 1u << 20;
// bytes after each operand: the padded M = 128 reads of mode 1 stay inside
// the allocation, and so would every read under the other assignment of the
// two descriptor strides
constexpr uint32_t kSlack = 16384;

__global__ void __launch_bounds__(128) umma_kernel(int mode, const uint16_t* a, const uint16_t* b, uint32_t k_or_f,
                                                   uint32_t n, float* d, uint32_t* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // operand sizes: mode 0: A 128 x K, B N x K; mode 1: A (=H) 128 x F, B (=G) 128 x N
    const uint32_t a_cols = k_or_f, b_rows = mode == 0 ? n : 128u, b_cols = mode == 0 ? k_or_f : n;
    unsigned char* sa = smem;
    unsigned char* sb = smem + 128u * a_cols * 2u + kSlack;
    for (uint32_t i = tid; i < 128u * a_cols; i += 128) {
        const uint32_t r = i / a_cols, c = i % a_cols;
        *reinterpret_cast<uint16_t*>(sa + canon_offset(r, c, a_cols)) = a[i];
    }
    for (uint32_t i = tid; i < kSlack / 4; i += 128) reinterpret_cast<uint32_t*>(sa + 128u * a_cols * 2u)[i] = 0u;
    for (uint32_t i = tid; i < b_rows * b_cols; i += 128) {
        const uint32_t r = i / b_cols, c = i % b_cols;
        *reinterpret_cast<uint16_t*>(sb + canon_offset(r, c, b_cols)) = b[i];
    }
    for (uint32_t i = tid; i < kSlack / 4; i += 128) reinterpret_cast<uint32_t*>(sb + b_rows * b_cols * 2u)[i] = 0u;
    if (tid == 0) mbar_init(&mbar, 1);
    if (warp == 0) tmem_alloc(&tmem_slot, 64);
    fence_smem_to_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_slot;
    if (tid == 0) {
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
        if (mode == 0) {
            const uint32_t idesc = instr_desc_bf16(128, n, false, false);
            for (uint32_t k = 0; k < k_or_f / 16; ++k)
                mma_bf16(tmem, smem_desc(a0 + 256u * k, 128u, a_cols / 8u * 128u),
                         smem_desc(b0 + 256u * k, 128u, b_cols / 8u * 128u), idesc, k > 0);
        } else {
            const uint32_t idesc = instr_desc_bf16(128, n, true, true);
            const uint32_t a_lbo = a_cols / 8u * 128u, b_lbo = b_cols / 8u * 128u;
            for (uint32_t k = 0; k < 128u / 16u; ++k)
                mma_bf16(tmem, smem_desc(a0 + 2u * a_lbo * k, a_lbo, 128u), smem_desc(b0 + 2u * b_lbo * k, b_lbo, 128u),
                         idesc, k > 0);
        }
        mma_commit(&mbar);
    }
    const bool ok = mbar_wait(&mbar, 0, kWaitLimit);
    fence_after_sync();
    if (ok) {
        const uint32_t row = 32u * warp + lane;
        for (uint32_t c = 0; c < n; c += 16) {
            uint32_t r[16];
            tmem_ld16(tmem_addr(tmem, 32u * warp, c), r);
            tmem_ld_wait();
            for (int j = 0; j < 16; ++j) d[(size_t)row * n + c + j] = __uint_as_float(r[j]);
        }
    } else if (lane == 0) {
        atomicOr(status, 1u);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

}  // namespace

extern "C" int umma_check(int mode, const uint16_t* a, const uint16_t* b, uint32_t k_or_f, uint32_t n, float* d) {
    // sizes the kernel supports: K (mode 0) or F (mode 1) a multiple of 16 up
    // to 128, N a multiple of 16 from 16 to 64
    if ((mode != 0 && mode != 1) || k_or_f == 0 || k_or_f % 16 || k_or_f > 128 || n < 16 || n > 64 || n % 16)
        return 2;
    const uint32_t a_elems = 128u * k_or_f, b_elems = mode == 0 ? n * k_or_f : 128u * n;
    const size_t smem = 2u * (a_elems + b_elems) + 2u * kSlack;
    uint16_t *da = nullptr, *db = nullptr;
    float* dd = nullptr;
    uint32_t* dst = nullptr;
    int rc = 3;
    if (cudaMalloc(&da, 2u * a_elems) == cudaSuccess && cudaMalloc(&db, 2u * b_elems) == cudaSuccess &&
        cudaMalloc(&dd, 4u * 128u * n) == cudaSuccess && cudaMalloc(&dst, 4) == cudaSuccess &&
        cudaMemcpy(da, a, 2u * a_elems, cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(db, b, 2u * b_elems, cudaMemcpyHostToDevice) == cudaSuccess && cudaMemset(dst, 0, 4) == cudaSuccess &&
        cudaMemset(dd, 0, 4u * 128u * n) == cudaSuccess &&
        cudaFuncSetAttribute(umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess) {
        umma_kernel<<<1, 128, smem>>>(mode, da, db, k_or_f, n, dd, dst);
        uint32_t st = 0;
        if (cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
            cudaMemcpy(d, dd, 4u * 128u * n, cudaMemcpyDeviceToHost) == cudaSuccess &&
            cudaMemcpy(&st, dst, 4, cudaMemcpyDeviceToHost) == cudaSuccess)
            rc = st ? 1 : 0;
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(dst);
    return rc;
}
