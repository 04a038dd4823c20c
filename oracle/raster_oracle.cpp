// raster_oracle.cpp — TEST INFRASTRUCTURE ONLY: scalar restatement of the
// raster pass (foundation_gb300/csrc/raster/raster.cu), which restates the
// reference renderer's draw (src/Renderer/Renderer.cpp:312-366,
// src/Renderer/Triangle.slang:23-37). Same rules, same operation order:
// FP32 vertex transform with left-to-right sums, perspective divide and
// viewport in FP64, vertices snapped to 1/256 pixel (round half to even),
// shoelace-sign culling (front faces counter-clockwise in Vulkan's sense),
// top-left fill rule at pixel centres, last covering triangle wins,
// perspective-correct FP64 barycentrics, bilinear repeat texel lookup,
// UNORM rounding. Built with -ffp-contract=off, so every byte should equal
// the device's. Parity against the reference itself is unpinned: its pass
// runs only through Vulkan.
#include <cmath>
#include <cstdint>
#include <utility>
#include <vector>

namespace {

float madd4(const float* a, const float* b, int r, int c) {
    float s = a[0 * 4 + r] * b[c * 4 + 0];
    s = s + a[1 * 4 + r] * b[c * 4 + 1];
    s = s + a[2 * 4 + r] * b[c * 4 + 2];
    return s + a[3 * 4 + r] * b[c * 4 + 3];
}

long long edge(long long ax, long long ay, long long bx, long long by, long long px, long long py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

struct Tri {
    bool ok = false;
    long long X[3], Y[3], A;
    double w[3];
    uint32_t vid[3];
    unsigned topleft = 0;
};

double unit_frac(double u) {
    if (!(u == u) || std::fabs(u) > 4.0e15) return 0.0;
    return u - std::floor(u);
}

uint32_t unorm8(double c) {
    c = c < 0.0 ? 0.0 : (c > 1.0 ? 1.0 : c);
    return (uint32_t)std::floor(c * 255.0 + 0.5);
}

}  // namespace

extern "C" void orc_raster_draw(uint32_t W, uint32_t H, const float* model, const float* view, const float* proj,
                                const float* clear, int cull_back, const float* vtx /* 7 floats per vertex */,
                                uint32_t nv, const uint16_t* idx, uint32_t ni, const uint32_t* tex, uint32_t tw,
                                uint32_t th, uint32_t* out) {
    float vm[16], pvm[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) vm[c * 4 + r] = madd4(view, model, r, c);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) pvm[c * 4 + r] = madd4(proj, vm, r, c);
    std::vector<double> clip(4 * (size_t)nv);
    for (uint32_t i = 0; i < nv; ++i) {
        const float p[4] = {vtx[7 * i + 0], vtx[7 * i + 1], 0.0f, 1.0f};
        for (int r = 0; r < 4; ++r) {
            float s = pvm[0 * 4 + r] * p[0];
            s = s + pvm[1 * 4 + r] * p[1];
            s = s + pvm[2 * 4 + r] * p[2];
            clip[4 * i + r] = (double)(s + pvm[3 * 4 + r] * p[3]);
        }
    }
    const uint32_t nt = ni / 3;
    std::vector<Tri> tris(nt);
    for (uint32_t t = 0; t < nt; ++t) {
        Tri& T = tris[t];
        long long X[3], Y[3];
        double w[3];
        uint32_t vid[3];
        bool ok = true;
        for (int k = 0; k < 3 && ok; ++k) {
            vid[k] = idx[3 * t + k];
            if (vid[k] >= nv) {
                ok = false;
                break;
            }
            const double* c = &clip[4 * vid[k]];
            w[k] = c[3];
            if (!(c[3] > 0.0)) {
                ok = false;
                break;
            }
            const double xd = c[0] / c[3], yd = c[1] / c[3];
            const double xf = 0.5 * (double)W * xd + 0.5 * (double)W;
            const double yf = 0.5 * (double)H * yd + 0.5 * (double)H;
            if (!(std::fabs(xf) < 1048576.0 && std::fabs(yf) < 1048576.0)) {
                ok = false;
                break;
            }
            X[k] = std::llrint(xf * 256.0);
            Y[k] = std::llrint(yf * 256.0);
        }
        if (!ok) continue;
        const long long s2 = edge(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
        if (s2 == 0 || (cull_back && !(s2 < 0))) continue;
        if (s2 < 0) {
            std::swap(X[1], X[2]);
            std::swap(Y[1], Y[2]);
            std::swap(w[1], w[2]);
            std::swap(vid[1], vid[2]);
        }
        T.ok = true;
        T.A = s2 < 0 ? -s2 : s2;
        for (int k = 0; k < 3; ++k) {
            const int a = (k + 1) % 3, b = (k + 2) % 3;
            const long long dx = X[b] - X[a], dy = Y[b] - Y[a];
            if ((dy == 0 && dx > 0) || dy < 0) T.topleft |= 1u << k;
            T.X[k] = X[k];
            T.Y[k] = Y[k];
            T.w[k] = w[k];
            T.vid[k] = vid[k];
        }
    }
    for (uint32_t py = 0; py < H; ++py)
        for (uint32_t px = 0; px < W; ++px) {
            const long long cx = (long long)px * 256 + 128, cy = (long long)py * 256 + 128;
            int hit = -1;
            long long E[3] = {0, 0, 0};
            for (uint32_t t = 0; t < nt; ++t) {
                const Tri& T = tris[t];
                if (!T.ok) continue;
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
            double rgba[4] = {clear[0], clear[1], clear[2], clear[3]};
            if (hit >= 0) {
                const Tri& T = tris[hit];
                const double area = (double)T.A;
                double b[3];
                for (int k = 0; k < 3; ++k) b[k] = ((double)E[k] / area) / T.w[k];
                const double s = (b[0] + b[1]) + b[2];
                double attr[5];
                for (int q = 0; q < 5; ++q) {
                    double acc = 0.0;
                    for (int k = 0; k < 3; ++k) {
                        const float* V = &vtx[7 * T.vid[k]];
                        const double a = q < 2 ? (double)V[5 + q] : (double)V[2 + (q - 2)];
                        acc = k == 0 ? b[0] * a : acc + b[k] * a;
                    }
                    attr[q] = acc / s;
                }
                const double ut = unit_frac(attr[0]) * (double)tw - 0.5;
                const double vt = unit_frac(attr[1]) * (double)th - 0.5;
                const double fu = std::floor(ut), fv = std::floor(vt);
                const double au = ut - fu, av = vt - fv;
                const long long TW = tw, TH = th;
                const long long i0 = (((long long)fu % TW) + TW) % TW, i1 = (i0 + 1) % TW;
                const long long j0 = (((long long)fv % TH) + TH) % TH, j1 = (j0 + 1) % TH;
                const double w00 = (1.0 - au) * (1.0 - av), w10 = au * (1.0 - av);
                const double w01 = (1.0 - au) * av, w11 = au * av;
                auto texel = [&](long long i, long long j, int ch) {
                    return (double)((tex[(size_t)j * tw + (size_t)i] >> (8 * ch)) & 0xFFu) / 255.0;
                };
                for (int ch = 0; ch < 4; ++ch) {
                    double c = w00 * texel(i0, j0, ch);
                    c = c + w10 * texel(i1, j0, ch);
                    c = c + w01 * texel(i0, j1, ch);
                    c = c + w11 * texel(i1, j1, ch);
                    rgba[ch] = ch < 3 ? c * attr[2 + ch] : c;
                }
            }
            out[(size_t)py * W + px] =
                unorm8(rgba[0]) | (unorm8(rgba[1]) << 8) | (unorm8(rgba[2]) << 16) | (unorm8(rgba[3]) << 24);
        }
}
