// pcg_check.cu — TEST HARNESS: runs the path tracer's device PCG32
// (foundation_gb300/csrc/pt/pt_math.cuh) on the GPU so a test can compare
// its output word for word with the oracle's generator:
//   mode 0: Pcg32::seed(a[j], b[j]), then n outputs;
//   mode 1: camera_path_rng(a[j], pixel c[j], sample d[j]), with the stream
//           packed into its 16-byte path record and unpacked again after
//           every output (the wavefront's save / restore between stages);
//   mode 2: training_path_rng(a[j], pixel c[j], path index d[j], round b[j]).
// One thread per stream j < m writes words[j * n + k] = k-th output and
// uniforms[j * n + k] = the k-th uniform() of an identically seeded stream.
// The caller owns the host buffers; the harness allocates and frees its own
// device copies.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../foundation_gb300/csrc/pt/pt_math.cuh"

using Foundation::PT::Pcg32;

namespace {

__device__ Pcg32 make_stream(int mode, const uint64_t* a, const uint64_t* b, const uint32_t* c, const uint32_t* d,
                             uint32_t j) {
    if (mode == 1) return Foundation::PT::camera_path_rng(a[j], c[j], d[j]);
    if (mode == 2) return Foundation::PT::training_path_rng(a[j], c[j], d[j], (uint32_t)b[j]);
    Pcg32 g;
    g.seed(a[j], b[j]);
    return g;
}

__global__ void pcg_kernel(int mode, const uint64_t* a, const uint64_t* b, const uint32_t* c, const uint32_t* d,
                           uint32_t m, uint32_t n, uint32_t* words, float* uniforms) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    Pcg32 g = make_stream(mode, a, b, c, d, j);
    Pcg32 u = make_stream(mode, a, b, c, d, j);
    for (uint32_t k = 0; k < n; ++k) {
        words[(size_t)j * n + k] = g.next();
        uniforms[(size_t)j * n + k] = u.uniform();
        if (mode == 1) {
            g = Foundation::PT::unpack_rng(Foundation::PT::pack_rng(g, d[j], 0u));
            u = Foundation::PT::unpack_rng(Foundation::PT::pack_rng(u, d[j], 0u));
        }
    }
}

}  // namespace

// Returns 0 on success, 1 on a CUDA error.
extern "C" int pcg_check(int mode, const uint64_t* a, const uint64_t* b, const uint32_t* c, const uint32_t* d,
                         uint32_t m, uint32_t n, uint32_t* words, float* uniforms) {
    if (m == 0 || n == 0) return 0;
    const size_t in_bytes = (2 * sizeof(uint64_t) + 2 * sizeof(uint32_t)) * m;
    const size_t out_words = (size_t)m * n;
    unsigned char* dbuf = nullptr;
    if (cudaMalloc(&dbuf, in_bytes + out_words * (sizeof(uint32_t) + sizeof(float))) != cudaSuccess) return 1;
    uint64_t* da = reinterpret_cast<uint64_t*>(dbuf);
    uint64_t* db = da + m;
    uint32_t* dc = reinterpret_cast<uint32_t*>(db + m);
    uint32_t* dd = dc + m;
    uint32_t* dw = dd + m;
    float* du = reinterpret_cast<float*>(dw + out_words);
    int rc = 0;
    if (cudaMemcpy(da, a, sizeof(uint64_t) * m, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(db, b, sizeof(uint64_t) * m, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dc, c, sizeof(uint32_t) * m, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dd, d, sizeof(uint32_t) * m, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = 1;
    } else {
        pcg_kernel<<<(m + 127) / 128, 128>>>(mode, da, db, dc, dd, m, n, dw, du);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(words, dw, sizeof(uint32_t) * out_words, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(uniforms, du, sizeof(float) * out_words, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = 1;
    }
    cudaFree(dbuf);
    return rc;
}
