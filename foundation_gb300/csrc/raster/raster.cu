// raster.cu — the reference renderer's raster pass as CUDA kernels (see
// raster.hpp for the rules).
//
//  vertex_kernel  per vertex: clip = proj (view (model (x, y, 0, 1))), the
//                 matrix products in FP32 with sums taken left to right
//                 (Triangle.slang:23-31 computes mul(proj, mul(view, model)))
//  setup_kernel   per triangle: perspective divide, viewport transform
//                 (Vulkan: y grows downwards), vertex snap to 1/256 pixel,
//                 signed area (front face counter-clockwise: Vulkan's
//                 a = -1/2 sum(x_i y_{i+1} - x_{i+1} y_i) > 0), culling,
//                 edge orientation and top-left flags, pixel bounding box
//  pixel_kernel   per pixel: coverage of every triangle in index order (no
//                 depth test: the last covering triangle wins), perspective-
//                 correct barycentrics, bilinear texel fetch with repeat
//                 addressing, colour = texel * (vertex colour, 1), UNORM
//                 encoding round(clamp(c, 0, 1) * 255)
// Triangles with a vertex at w <= 0 (behind the eye) or outside a +-2^20
// pixel guard band are skipped rather than clipped.
#include "raster.hpp"

#include <cstdint>

namespace Foundation {
namespace Raster {
namespace {

constexpr int kSub = 256;  // sub-pixel steps per pixel

struct Tri {
    long long X[3], Y[3];  // snapped framebuffer positions (1/256 pixel), oriented so the inside is E >= 0
    long long A;           // twice the area (> 0)
    double w[3];           // clip w per vertex (after orientation)
    uint32_t vid[3];       // vertex ids (after orientation)
    uint32_t topleft;      // bit i: edge opposite vertex i is a top or left edge
    int x0, y0, x1, y1;    // inclusive pixel bounds; x0 > x1 when the triangle is skipped
};

__device__ __forceinline__ float madd4(const float* a, const float* b, int r, int c) {
    // (A B)[r][c] with column-major storage m[col * 4 + row]
    float s = __fmul_rn(a[0 * 4 + r], b[c * 4 + 0]);
    s = __fadd_rn(s, __fmul_rn(a[1 * 4 + r], b[c * 4 + 1]));
    s = __fadd_rn(s, __fmul_rn(a[2 * 4 + r], b[c * 4 + 2]));
    return __fadd_rn(s, __fmul_rn(a[3 * 4 + r], b[c * 4 + 3]));
}

__global__ void vertex_kernel(const DrawArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.nv) return;
    float vm[16], pvm[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) vm[c * 4 + r] = madd4(A.u.view, A.u.model, r, c);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) pvm[c * 4 + r] = madd4(A.u.proj, vm, r, c);
    const float p[4] = {A.verts[i].pos[0], A.verts[i].pos[1], 0.0f, 1.0f};
    float o[4];
    for (int r = 0; r < 4; ++r) {
        float s = __fmul_rn(pvm[0 * 4 + r], p[0]);
        s = __fadd_rn(s, __fmul_rn(pvm[1 * 4 + r], p[1]));
        s = __fadd_rn(s, __fmul_rn(pvm[2 * 4 + r], p[2]));
        o[r] = __fadd_rn(s, __fmul_rn(pvm[3 * 4 + r], p[3]));
    }
    A.clip[i] = make_double4(o[0], o[1], o[2], o[3]);
}

__device__ __forceinline__ long long edge(long long ax, long long ay, long long bx, long long by, long long px,
                                          long long py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

__global__ void setup_kernel(const DrawArgs A, Tri* tris) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.ntri) return;
    Tri T;
    T.x0 = 1;
    T.x1 = 0;
    T.y0 = T.y1 = 0;
    bool ok = true;
    long long X[3], Y[3];
    double w[3];
    uint32_t vid[3];
    for (int k = 0; k < 3; ++k) {
        vid[k] = A.idx[3 * (size_t)t + k];
        if (vid[k] >= A.nv) {
            atomicOr(A.status, 1u);
            ok = false;
            break;
        }
        const double4 c = A.clip[vid[k]];
        w[k] = c.w;
        if (!(c.w > 0.0)) {
            ok = false;
            break;
        }
        const double xd = __ddiv_rn(c.x, c.w), yd = __ddiv_rn(c.y, c.w);
        const double xf = __dadd_rn(__dmul_rn(0.5 * (double)A.width, xd), 0.5 * (double)A.width);
        const double yf = __dadd_rn(__dmul_rn(0.5 * (double)A.height, yd), 0.5 * (double)A.height);
        if (!(fabs(xf) < 1048576.0 && fabs(yf) < 1048576.0)) {
            ok = false;
            break;
        }
        X[k] = __double2ll_rn(__dmul_rn(xf, (double)kSub));
        Y[k] = __double2ll_rn(__dmul_rn(yf, (double)kSub));
    }
    if (ok) {
        // 2x the shoelace area; Vulkan's a = -area, front-facing when a > 0
        const long long s2 = edge(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
        const bool front = s2 < 0;
        if (s2 == 0 || (A.cull_back && !front)) ok = false;
        if (ok) {
            if (s2 < 0) {  // orient so the inside has positive edge functions
                long long tx = X[1], ty = Y[1];
                X[1] = X[2];
                Y[1] = Y[2];
                X[2] = tx;
                Y[2] = ty;
                const double tw = w[1];
                w[1] = w[2];
                w[2] = tw;
                const uint32_t tv = vid[1];
                vid[1] = vid[2];
                vid[2] = tv;
            }
            T.A = s2 < 0 ? -s2 : s2;
            T.topleft = 0;
            for (int k = 0; k < 3; ++k) {
                // edge opposite vertex k runs from vertex k+1 to vertex k+2
                const int a = (k + 1) % 3, b = (k + 2) % 3;
                const long long dx = X[b] - X[a], dy = Y[b] - Y[a];
                if ((dy == 0 && dx > 0) || dy < 0) T.topleft |= 1u << k;
            }
            long long mnx = X[0], mxx = X[0], mny = Y[0], mxy = Y[0];
            for (int k = 1; k < 3; ++k) {
                mnx = X[k] < mnx ? X[k] : mnx;
                mxx = X[k] > mxx ? X[k] : mxx;
                mny = Y[k] < mny ? Y[k] : mny;
                mxy = Y[k] > mxy ? Y[k] : mxy;
            }
            // pixel p is tested at p * 256 + 128
            long long px0 = (mnx - kSub / 2 + kSub - 1) / kSub, py0 = (mny - kSub / 2 + kSub - 1) / kSub;
            long long px1 = (mxx - kSub / 2) / kSub, py1 = (mxy - kSub / 2) / kSub;
            if (mnx - kSub / 2 < 0) px0 = 0;
            if (mny - kSub / 2 < 0) py0 = 0;
            if (mxx - kSub / 2 < 0) px1 = -1;
            if (mxy - kSub / 2 < 0) py1 = -1;
            px1 = px1 < (long long)A.width - 1 ? px1 : (long long)A.width - 1;
            py1 = py1 < (long long)A.height - 1 ? py1 : (long long)A.height - 1;
            T.x0 = (int)px0;
            T.y0 = (int)py0;
            T.x1 = (int)px1;
            T.y1 = (int)py1;
            for (int k = 0; k < 3; ++k) {
                T.X[k] = X[k];
                T.Y[k] = Y[k];
                T.w[k] = w[k];
                T.vid[k] = vid[k];
            }
        }
    }
    tris[t] = T;
}

__device__ __forceinline__ double unit_frac(double u) {
    if (!(u == u) || fabs(u) > 4.0e15) return 0.0;  // NaN / beyond exact fractions
    return __dsub_rn(u, floor(u));
}

__device__ __forceinline__ double texel(const DrawArgs& A, long long i, long long j, int ch) {
    const uint32_t v = A.texture[(size_t)j * A.tex_w + (size_t)i];
    return (double)((v >> (8 * ch)) & 0xFFu) / 255.0;
}

__device__ __forceinline__ uint32_t unorm8(double c) {
    c = c < 0.0 ? 0.0 : (c > 1.0 ? 1.0 : c);
    return (uint32_t)floor(__dadd_rn(__dmul_rn(c, 255.0), 0.5));
}

__global__ void pixel_kernel(const DrawArgs A, const Tri* __restrict__ tris) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= A.width || py >= A.height) return;
    const long long cx = (long long)px * kSub + kSub / 2, cy = (long long)py * kSub + kSub / 2;
    int hit = -1;
    long long E[3] = {0, 0, 0};
    for (uint32_t t = 0; t < A.ntri; ++t) {
        const Tri& T = tris[t];
        if ((int)px < T.x0 || (int)px > T.x1 || (int)py < T.y0 || (int)py > T.y1) continue;
        long long e[3];
        bool in = true;
        for (int k = 0; k < 3 && in; ++k) {
            const int a = (k + 1) % 3, b = (k + 2) % 3;
            e[k] = edge(T.X[a], T.Y[a], T.X[b], T.Y[b], cx, cy);
            in = e[k] > 0 || (e[k] == 0 && ((T.topleft >> k) & 1u));
        }
        if (in) {
            hit = (int)t;
            E[0] = e[0];
            E[1] = e[1];
            E[2] = e[2];
        }
    }
    double rgba[4] = {A.clear[0], A.clear[1], A.clear[2], A.clear[3]};
    if (hit >= 0) {
        const Tri& T = tris[hit];
        const double area = (double)T.A;
        double b[3];
        for (int k = 0; k < 3; ++k) b[k] = __ddiv_rn(__ddiv_rn((double)E[k], area), T.w[k]);
        const double s = __dadd_rn(__dadd_rn(b[0], b[1]), b[2]);
        double attr[5];  // u, v, r, g, b
        for (int q = 0; q < 5; ++q) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) {
                const Vertex& V = A.verts[T.vid[k]];
                const double a = q < 2 ? (double)V.uv[q] : (double)V.color[q - 2];
                acc = k == 0 ? __dmul_rn(b[0], a) : __dadd_rn(acc, __dmul_rn(b[k], a));
            }
            attr[q] = __ddiv_rn(acc, s);
        }
        const double ut = __dsub_rn(__dmul_rn(unit_frac(attr[0]), (double)A.tex_w), 0.5);
        const double vt = __dsub_rn(__dmul_rn(unit_frac(attr[1]), (double)A.tex_h), 0.5);
        const double fu = floor(ut), fv = floor(vt);
        const double au = __dsub_rn(ut, fu), av = __dsub_rn(vt, fv);
        const long long W = A.tex_w, H = A.tex_h;
        const long long i0 = (((long long)fu % W) + W) % W, i1 = (i0 + 1) % W;
        const long long j0 = (((long long)fv % H) + H) % H, j1 = (j0 + 1) % H;
        const double w00 = __dmul_rn(__dsub_rn(1.0, au), __dsub_rn(1.0, av)), w10 = __dmul_rn(au, __dsub_rn(1.0, av));
        const double w01 = __dmul_rn(__dsub_rn(1.0, au), av), w11 = __dmul_rn(au, av);
        for (int ch = 0; ch < 4; ++ch) {
            double c = __dmul_rn(w00, texel(A, i0, j0, ch));
            c = __dadd_rn(c, __dmul_rn(w10, texel(A, i1, j0, ch)));
            c = __dadd_rn(c, __dmul_rn(w01, texel(A, i0, j1, ch)));
            c = __dadd_rn(c, __dmul_rn(w11, texel(A, i1, j1, ch)));
            rgba[ch] = ch < 3 ? __dmul_rn(c, attr[2 + ch]) : c;
        }
    }
    A.target[(size_t)py * A.width + px] =
        unorm8(rgba[0]) | (unorm8(rgba[1]) << 8) | (unorm8(rgba[2]) << 16) | (unorm8(rgba[3]) << 24);
}

}  // namespace

cudaError_t LaunchDraw(const DrawArgs& a, cudaStream_t s) {
    Tri* tris = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&tris), sizeof(Tri) * (a.ntri ? a.ntri : 1), s);
    if (e != cudaSuccess) return e;
    if (a.nv) vertex_kernel<<<(a.nv + 127) / 128, 128, 0, s>>>(a);
    if (a.ntri) setup_kernel<<<(a.ntri + 127) / 128, 128, 0, s>>>(a, tris);
    pixel_kernel<<<dim3((a.width + 127) / 128, a.height), 128, 0, s>>>(a, tris);
    e = cudaGetLastError();
    const cudaError_t f = cudaFreeAsync(tris, s);
    return e != cudaSuccess ? e : f;
}

}  // namespace Raster
}  // namespace Foundation
