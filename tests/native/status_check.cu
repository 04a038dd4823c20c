// status_check.cu — TEST HARNESS: runs the product's traversal code on the
// GPU over hand-made node and triangle arrays (built by the test), so the
// device status word can be driven without a fault: a child index past the
// node array, a leaf's triangle range past the triangle arrays and a chain
// deeper than the traversal stack are each caught by the kernels' own
// checks, which latch a status bit and end the ray before any out-of-range
// access.
//   mode 0: RT::trace_single (the per-thread traversal of the path-tracing
//           megakernels), closest hit, one thread per ray;
//   mode 1: the persistent closest-hit kernel, launched through the
//           library's RT::LaunchTrace (links libfnd_rt.so);
//   mode 2: the persistent any-hit kernel.
// hits[2 i] = prim id, hits[2 i + 1] = t bits (mode 2: occlusion flag);
// *status_out = the latched status word. The caller owns the host buffers.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../foundation_gb300/csrc/rt/traverse.cuh"
#include "../../foundation_gb300/csrc/rt/traverse_launch.hpp"

using namespace Foundation::RT;

namespace {

__global__ void single_kernel(DeviceScene sc, const float4* rays, uint32_t n, uint32_t* hits, uint32_t* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const RayState r = setup_ray(rays[2 * i], rays[2 * i + 1]);
    float t = r.tmax;
    uint32_t p = FND_INVALID_ID;
    const bool h = trace_single<false>(sc, r, t, p, status);
    hits[2 * i] = h ? p : FND_INVALID_ID;
    hits[2 * i + 1] = h ? __float_as_uint(t) : 0x7F800000u;
}

}  // namespace

// Returns 0 on success, 1 on a CUDA error.
extern "C" int status_trace(int mode, const void* nodes, uint32_t num_nodes, const float* planes, uint32_t num_tris,
                            const float* rays, uint32_t n, uint32_t* hits, uint32_t* status_out) {
    const size_t node_bytes = 80 * (size_t)num_nodes;
    const size_t plane_bytes = 3 * 16 * (size_t)num_tris;
    const size_t ray_bytes = 32 * (size_t)n;
    const size_t hit_bytes = 8 * (size_t)n;
    const size_t total = 256 + node_bytes + plane_bytes + ray_bytes + hit_bytes + 64;
    unsigned char* d = nullptr;
    if (cudaMalloc(&d, total) != cudaSuccess) return 1;
    uint32_t* counter = reinterpret_cast<uint32_t*>(d);
    uint32_t* status = counter + 1;
    unsigned char* p = d + 256;
    const uint4* d_nodes = reinterpret_cast<const uint4*>(p);
    const float4* d_planes = reinterpret_cast<const float4*>(p + node_bytes);
    const float4* d_rays = reinterpret_cast<const float4*>(p + node_bytes + plane_bytes);
    unsigned char* d_hits = p + node_bytes + plane_bytes + ray_bytes;
    int rc = 0;
    if (cudaMemset(d, 0, 256) != cudaSuccess ||
        (node_bytes && cudaMemcpy(p, nodes, node_bytes, cudaMemcpyHostToDevice) != cudaSuccess) ||
        (plane_bytes && cudaMemcpy(p + node_bytes, planes, plane_bytes, cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemcpy(p + node_bytes + plane_bytes, rays, ray_bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(d_hits, 0, hit_bytes) != cudaSuccess) {
        rc = 1;
    } else {
        DeviceScene sc{};
        sc.nodes = d_nodes;
        sc.v0 = d_planes;
        sc.v1 = d_planes + num_tris;
        sc.v2 = d_planes + 2 * (size_t)num_tris;
        sc.num_nodes = num_nodes;
        sc.num_tris = num_tris;
        cudaError_t e = cudaSuccess;
        if (mode == 0) {
            single_kernel<<<(n + 63) / 64, 64>>>(sc, d_rays, n, reinterpret_cast<uint32_t*>(d_hits), status);
            e = cudaGetLastError();
        } else {
            TraceLaunch L{};
            L.scene = sc;
            L.rays = d_rays;
            L.n = n;
            L.hits = d_hits;
            L.occluded = d_hits;
            L.counter = counter;
            L.status = status;
            L.refill_min = 8;
            int sms = 0, blocks = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
            if (e == cudaSuccess) e = TraceOccupancy(mode == 2 ? 1 : 0, &blocks);
            if (e == cudaSuccess) e = LaunchTrace(L, mode == 2, false, sms * (blocks > 0 ? blocks : 1), nullptr);
        }
        if (e != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
            rc = 1;
        } else if (mode == 2) {
            // occlusion bytes -> (flag, 0) pairs
            uint8_t* occ = new uint8_t[n ? n : 1];
            if (cudaMemcpy(occ, d_hits, n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 1;
            for (uint32_t i = 0; i < n && rc == 0; ++i) {
                hits[2 * i] = occ[i];
                hits[2 * i + 1] = 0;
            }
            delete[] occ;
        } else if (cudaMemcpy(hits, d_hits, hit_bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = 1;
        }
        if (rc == 0 && cudaMemcpy(status_out, status, sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess) rc = 1;
    }
    cudaFree(d);
    return rc;
}
