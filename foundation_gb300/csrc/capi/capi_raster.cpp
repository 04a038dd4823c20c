// capi_raster.cpp — C ABI of the raster-pass restatement (raster/raster.cu):
// the reference's per-frame uniforms (src/Renderer/Renderer.cpp:370-380,
// computed on the host as there) and the draw of an indexed triangle list
// into an R8G8B8A8_UNORM target (Renderer.cpp:312-366).
#include <cmath>
#include <cstring>

#include "../raster/raster.hpp"
#include "context.hpp"

using namespace Foundation;
using Foundation::CApi::Guard;

namespace {

struct V3 {
    float x, y, z;
};
V3 Sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 Cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 Normalize(V3 v) {
    const float k = 1.0f / std::sqrt(Dot(v, v));
    return {v.x * k, v.y * k, v.z * k};
}

// glm conventions (column-major, right-handed, clip depth -1..1), restated:
// rotate about +z, lookAt, infinitePerspective, then the Vulkan y flip.
void ReferenceUniforms(float time, float aspect, float M[16], float V[16], float P[16]) {
    std::memset(M, 0, 64);
    std::memset(V, 0, 64);
    std::memset(P, 0, 64);
    const float deg = 0.01745329251994329576923690768489f;  // radians per degree
    const float angle = time * (90.0f * deg);
    const float c = std::cos(angle), s = std::sin(angle);
    M[0] = c;
    M[1] = s;
    M[4] = -s;
    M[5] = c;
    M[10] = c + (1.0f - c);
    M[15] = 1.0f;
    const V3 eye{2.0f, 2.0f, 2.0f}, center{0.0f, 0.0f, 0.0f}, up{0.0f, 0.0f, 1.0f};
    const V3 f = Normalize(Sub(center, eye));
    const V3 sv = Normalize(Cross(f, up));
    const V3 u = Cross(sv, f);
    V[0] = sv.x;
    V[4] = sv.y;
    V[8] = sv.z;
    V[1] = u.x;
    V[5] = u.y;
    V[9] = u.z;
    V[2] = -f.x;
    V[6] = -f.y;
    V[10] = -f.z;
    V[12] = -Dot(sv, eye);
    V[13] = -Dot(u, eye);
    V[14] = Dot(f, eye);
    V[15] = 1.0f;
    const float fovy = 45.0f * deg, znear = 0.1f;
    const float range = std::tan(fovy / 2.0f) * znear;
    const float left = -range * aspect, right = range * aspect, bottom = -range, top = range;
    P[0] = (2.0f * znear) / (right - left);
    P[5] = (2.0f * znear) / (top - bottom);
    P[10] = -1.0f;
    P[11] = -1.0f;
    P[14] = -2.0f * znear;
    P[5] *= -1.0f;
}

}  // namespace

extern "C" {

int fnd_rt_raster_uniforms(float time_s, float aspect, float* model, float* view, float* proj) {
    if (!model || !view || !proj || !std::isfinite(time_s) || !(aspect > 0.0f) || !std::isfinite(aspect))
        return FND_ERR_INVALID_ARG;
    ReferenceUniforms(time_s, aspect, model, view, proj);
    return FND_OK;
}

int fnd_rt_raster_draw(fnd_rt_ctx* ctx, const fnd_raster_desc* desc, const fnd_raster_vertex* verts, uint32_t nv,
                       const uint16_t* idx, uint32_t ni, const uint8_t* texture, uint32_t tex_w, uint32_t tex_h,
                       uint8_t* rgba, int mem) {
    if (!ctx) return FND_ERR_INVALID_ARG;
    return Guard(ctx, [&] {
        CHECK(desc != nullptr && rgba != nullptr && (nv == 0 || verts != nullptr) && (ni == 0 || idx != nullptr));
        CHECK(mem == FND_MEM_HOST || mem == FND_MEM_DEVICE);
        CHECK_CODE(ni % 3 == 0, FND_ERR_INVALID_ARG, "%u indices is not a triangle list", ni);
        CHECK_CODE(desc->width >= 1 && desc->height >= 1 && desc->width <= 16384 && desc->height <= 16384,
                   FND_ERR_INVALID_ARG, "target %ux%u", desc->width, desc->height);
        CHECK_CODE(texture != nullptr && tex_w >= 1 && tex_h >= 1 && (uint64_t)tex_w * tex_h <= (1ull << 28),
                   FND_ERR_INVALID_ARG, "texture %ux%u", tex_w, tex_h);
        for (uint32_t i = 0; i < ni; ++i)
            CHECK_CODE(idx[i] < nv, FND_ERR_INVALID_ARG, "index %u = %u, %u vertices", i, idx[i], nv);
        CHECK_CODE(mem == FND_MEM_HOST || ((uintptr_t)rgba & 3u) == 0, FND_ERR_INVALID_ARG,
                   "device target must be 4-byte aligned");
        CUDA_CHECK(cudaSetDevice(ctx->device));
        const size_t vb = sizeof(fnd_raster_vertex) * nv, ib = 2ull * ni, tb = 4ull * tex_w * tex_h;
        const size_t npix = (size_t)desc->width * desc->height;
        const size_t off_i = (vb + 255) & ~size_t(255), off_t = (off_i + ib + 255) & ~size_t(255);
        const size_t off_c = (off_t + tb + 255) & ~size_t(255), off_s = off_c + 32ull * nv;
        const size_t off_o = (off_s + 256 + 255) & ~size_t(255);
        const size_t total = off_o + (mem == FND_MEM_HOST ? 4 * npix : 0);
        CApi::EnsureDevice(ctx->d_in, ctx->d_in_cap, total);
        char* base = static_cast<char*>(ctx->d_in);
        if (vb) CUDA_CHECK(cudaMemcpyAsync(base, verts, vb, cudaMemcpyHostToDevice, ctx->stream));
        if (ib) CUDA_CHECK(cudaMemcpyAsync(base + off_i, idx, ib, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemcpyAsync(base + off_t, texture, tb, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_CHECK(cudaMemsetAsync(base + off_s, 0, 4, ctx->stream));
        Raster::DrawArgs A{};
        A.width = desc->width;
        A.height = desc->height;
        std::memcpy(A.u.model, desc->model, 64);
        std::memcpy(A.u.view, desc->view, 64);
        std::memcpy(A.u.proj, desc->proj, 64);
        std::memcpy(A.clear, desc->clear, 16);
        A.cull_back = desc->cull_back;
        A.verts = reinterpret_cast<const Raster::Vertex*>(base);
        A.nv = nv;
        A.idx = reinterpret_cast<const uint16_t*>(base + off_i);
        A.ntri = ni / 3;
        A.texture = reinterpret_cast<const uint32_t*>(base + off_t);
        A.tex_w = tex_w;
        A.tex_h = tex_h;
        A.clip = reinterpret_cast<double4*>(base + off_c);
        A.status = reinterpret_cast<uint32_t*>(base + off_s);
        A.target = mem == FND_MEM_HOST ? reinterpret_cast<uint32_t*>(base + off_o) : reinterpret_cast<uint32_t*>(rgba);
        CUDA_CHECK(Raster::LaunchDraw(A, ctx->stream));
        if (mem == FND_MEM_HOST) {
            CUDA_CHECK(cudaMemcpyAsync(rgba, A.target, 4 * npix, cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        }
    });
}

}  // extern "C"
