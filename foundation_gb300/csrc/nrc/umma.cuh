// umma.cuh — fifth-generation tensor-core primitives (tcgen05, sm_100 family)
// as inline PTX: tensor-memory allocation, shared-memory matrix descriptors,
// the BF16 x BF16 -> FP32 MMA with its completion barrier, and tensor-memory
// loads. Shared by the radiance cache's training kernel and the GPU check
// of the primitives (tests/native/umma_check.cu).
//
// Shared-memory operand layout (no swizzle). An operand is a grid of "core
// matrices" of 8 rows x 16 bytes (8 BF16), each stored as 128 contiguous
// bytes (row r at +16 r). Matrices here are stored row-group major: the core
// matrix of row group g and column group j of a [rows][cols] BF16 array sits
// at (g * cols / 8 + j) * 128 bytes, so one row group (8 rows x cols) is a
// contiguous block (canon_offset below). The same array serves two ways:
//  * K-major (rows = M or N, cols = K): the K-direction stride between core
//    matrices (leading byte offset) is 128, the M/N-direction stride
//    (stride byte offset) is cols / 8 * 128;
//  * MN-major (cols = M or N, rows = K; the transposed use, for the weight
//    gradients whose reduction runs over the batch rows): the M/N-direction
//    stride (stride byte offset) is 128, the K-direction stride (leading byte
//    offset) is cols / 8 * 128.
// One MMA consumes K = 16 (two core matrices along K); the next K step
// starts 2 x the K-direction stride further on.
//
// Tensor memory: 128 lanes x 512 columns of 32 bits per SM. An M = 128 MMA
// writes row i of D to lane i, column j to column base + j. A warp may read
// only its lane quarter (lanes 32 (warp % 4) .. + 31).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace Foundation {
namespace NRC {
namespace Umma {

// Byte offset of element (r, c) in a row-group-major BF16 array of `cols`
// columns (cols a multiple of 8).
__host__ __device__ constexpr uint32_t canon_offset(uint32_t r, uint32_t c, uint32_t cols) {
    return ((r >> 3) * (cols >> 3) + (c >> 3)) * 128u + (r & 7u) * 16u + (c & 7u) * 2u;
}

// Shared-memory matrix descriptor (64 bits): start address >> 4 in bits
// 0-13, leading byte offset >> 4 in 16-29, stride byte offset >> 4 in 32-45,
// the fixed value 0b001 in 46-48, base offset 0, relative leading offset,
// no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 D (bits 4-5 = 1), BF16 A and B
// (bits 7-9 = 1, 10-12 = 1), A / B MN-major when a_mn / b_mn (bits 15, 16),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28, dense, no negation.
__host__ __device__ constexpr uint32_t instr_desc_bf16(uint32_t m, uint32_t n, bool a_mn, bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- tensor memory --------------------------------------------------------
// Allocation and release are warp-wide (all 32 lanes of one warp).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot_smem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes become visible to the tensor core
// (async proxy) reads issued after the next barrier.
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA --------------------------------------------------------------------
// D[tmem] (+)= A[smem] x B[smem]; accumulate = false overwrites D.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}
// The barrier at `mbar` gets one arrival once every MMA this thread issued
// before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

// ---- mbarrier ---------------------------------------------------------------
// Initialises the barrier and makes the initialisation visible to the
// tensor core's (async proxy) arrivals; the caller then syncs the CTA.
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits for the phase with the given parity to complete, at most `limit`
// polls (each try_wait itself blocks for a bounded, hardware-defined time).
// Returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}

// One plain arrival (completes a phase of a count-1 barrier without an MMA).
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}
// Arrives on the barrier and expects `bytes` of asynchronous copies to
// complete the phase.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// ---- bulk copy (TMA, untiled) ----------------------------------------------
// global -> shared, both 16-byte aligned, `bytes` a multiple of 16; the bytes
// count towards the barrier's expected transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_u32(mbar))
                 : "memory");
}

// ---- tensor memory -> registers -------------------------------------------
// 16 consecutive 32-bit columns of this thread's lane (32x32b shape: thread t
// of the warp reads lane (taddr lane) + t).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Tensor-memory address of lane `lane`, column `col` relative to `base`.
__device__ __forceinline__ uint32_t tmem_addr(uint32_t base, uint32_t lane, uint32_t col) {
    return base + (lane << 16) + col;
}

}  // namespace Umma
}  // namespace NRC
}  // namespace Foundation
