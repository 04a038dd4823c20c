// minmax_check.cu — TEST HARNESS: evaluates, on the GPU, the operations the
// traversal's child-box test relies on, over a table of special and ordinary
// inputs, so a test can compare them with their host definitions:
//   op 0: three-input max.f32 (PTX, sm_100 family) vs fmaxf(fmaxf(a, b), c)
//   op 1: three-input min.f32 vs fminf(fminf(a, b), c)
//   op 2: __fmaf_rd(a, b, c)     op 3: __fmaf_ru(a, b, c)
// and (fma2_check) the packed fma.rm / fma.rp .f32x2 on the lane pair
// (a, b) * (b, c) + (c, a) beside the scalar __fmaf_rd / __fmaf_ru of each
// lane's operands.
// One thread per input triple; the caller owns the host buffers.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__global__ void check_kernel(const float* a, const float* b, const float* c, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float mx, mn;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(mx) : "f"(a[i]), "f"(b[i]), "f"(c[i]));
    asm("min.f32 %0, %1, %2, %3;" : "=f"(mn) : "f"(a[i]), "f"(b[i]), "f"(c[i]));
    out[4 * (size_t)i + 0] = mx;
    out[4 * (size_t)i + 1] = mn;
    out[4 * (size_t)i + 2] = __fmaf_rd(a[i], b[i], c[i]);
    out[4 * (size_t)i + 3] = __fmaf_ru(a[i], b[i], c[i]);
}

__global__ void fma2_kernel(const float* a, const float* b, const float* c, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long x, y, z, rd, ru;
    asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(a[i]), "f"(b[i]));
    asm("mov.b64 %0, {%1, %2};" : "=l"(y) : "f"(b[i]), "f"(c[i]));
    asm("mov.b64 %0, {%1, %2};" : "=l"(z) : "f"(c[i]), "f"(a[i]));
    asm("fma.rm.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(x), "l"(y), "l"(z));
    asm("fma.rp.f32x2 %0, %1, %2, %3;" : "=l"(ru) : "l"(x), "l"(y), "l"(z));
    float* o = out + 8 * (size_t)i;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(o[0]), "=f"(o[1]) : "l"(rd));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(o[2]), "=f"(o[3]) : "l"(ru));
    o[4] = __fmaf_rd(a[i], b[i], c[i]);
    o[5] = __fmaf_rd(b[i], c[i], a[i]);
    o[6] = __fmaf_ru(a[i], b[i], c[i]);
    o[7] = __fmaf_ru(b[i], c[i], a[i]);
}

}  // namespace

extern "C" int fma2_check(const float* a, const float* b, const float* c, uint32_t n, float* out) {
    if (n == 0) return 0;
    float *da = nullptr, *dout = nullptr;
    const size_t in = sizeof(float) * (size_t)n;
    if (cudaMalloc(&da, 3 * in) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, 8 * in) != cudaSuccess) {
        cudaFree(da);
        return 1;
    }
    int rc = 0;
    if (cudaMemcpy(da, a, in, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(da + n, b, in, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(da + 2 * (size_t)n, c, in, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = 2;
    if (!rc) {
        fma2_kernel<<<(n + 127) / 128, 128>>>(da, da + n, da + 2 * (size_t)n, n, dout);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = 3;
    }
    if (!rc && cudaMemcpy(out, dout, 8 * in, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 4;
    cudaFree(da);
    cudaFree(dout);
    return rc;
}

extern "C" int minmax_check(const float* a, const float* b, const float* c, uint32_t n, float* out) {
    if (n == 0) return 0;
    float *da = nullptr, *dout = nullptr;
    const size_t in = sizeof(float) * (size_t)n;
    if (cudaMalloc(&da, 3 * in) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, 4 * in) != cudaSuccess) {
        cudaFree(da);
        return 1;
    }
    int rc = 0;
    if (cudaMemcpy(da, a, in, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(da + n, b, in, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(da + 2 * (size_t)n, c, in, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = 2;
    if (!rc) {
        check_kernel<<<(n + 127) / 128, 128>>>(da, da + n, da + 2 * (size_t)n, n, dout);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = 3;
    }
    if (!rc && cudaMemcpy(out, dout, 4 * in, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 4;
    cudaFree(da);
    cudaFree(dout);
    return rc;
}
