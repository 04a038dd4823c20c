// instances.cpp — host side of two-level scenes (see instances.hpp).
#include "instances.hpp"

#include <algorithm>
#include <cmath>

#include "../../../include/fnd_rt.h"
#include "../core/core.hpp"

namespace Foundation {
namespace RT {
namespace {

float Down(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
}
float Up(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}

}  // namespace

bool InstanceInverse(const float* m, float out[12]) {
    for (int k = 0; k < 12; ++k)
        if (!std::isfinite(m[k])) return false;
    const double a00 = m[0], a01 = m[1], a02 = m[2], a10 = m[4], a11 = m[5], a12 = m[6];
    const double a20 = m[8], a21 = m[9], a22 = m[10];
    const double c00 = a11 * a22 - a12 * a21, c01 = a10 * a22 - a12 * a20, c02 = a10 * a21 - a11 * a20;
    const double det = a00 * c00 - a01 * c01 + a02 * c02;
    if (!(std::fabs(det) > 1e-30) || !std::isfinite(det)) return false;
    double inv[12];
    inv[0] = c00 / det;
    inv[1] = (a02 * a21 - a01 * a22) / det;
    inv[2] = (a01 * a12 - a02 * a11) / det;
    inv[4] = (a12 * a20 - a10 * a22) / det;
    inv[5] = (a00 * a22 - a02 * a20) / det;
    inv[6] = (a02 * a10 - a00 * a12) / det;
    inv[8] = c02 / det;
    inv[9] = (a01 * a20 - a00 * a21) / det;
    inv[10] = (a00 * a11 - a01 * a10) / det;
    for (int i = 0; i < 3; ++i)
        inv[4 * i + 3] = -((inv[4 * i] * (double)m[3] + inv[4 * i + 1] * (double)m[7]) + inv[4 * i + 2] * (double)m[11]);
    for (int k = 0; k < 12; ++k) out[k] = (float)inv[k];
    return true;
}

double InstanceReach(const float inv[12], const double lo[3], const double hi[3]) {
    double reach = 0.0;
    for (int c = 0; c < 8; ++c) {
        const double p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
        for (int a = 0; a < 3; ++a) {
            const float* m = inv + 4 * a;
            reach = std::max(reach, std::fabs((((double)m[0] * p[0] + (double)m[1] * p[1]) + (double)m[2] * p[2]) +
                                              (double)m[3]));
        }
    }
    return reach;
}

void BuildInstanceTop(const InstanceInput* in, uint32_t n, InstanceTop& out) {
    out.inv.assign(12 * (size_t)n, 0.0f);
    for (int a = 0; a < 3; ++a) {
        out.lo[a] = INFINITY;
        out.hi[a] = -INFINITY;
    }
    std::vector<float> boxes(9 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        const InstanceInput& I = in[i];
        CHECK_CODE(InstanceInverse(I.transform, &out.inv[12 * (size_t)i]), FND_ERR_INVALID_ARG,
                   "instance %u: singular or non-finite transform", i);
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = 0; c < 8; ++c) {
            const double p[3] = {(c & 1) ? I.hi[0] : I.lo[0], (c & 2) ? I.hi[1] : I.lo[1], (c & 4) ? I.hi[2] : I.lo[2]};
            for (int a = 0; a < 3; ++a) {
                const float* m = I.transform + 4 * a;
                const double w = ((double)m[0] * p[0] + (double)m[1] * p[1]) + (double)m[2] * p[2] + (double)m[3];
                lo[a] = std::min(lo[a], w);
                hi[a] = std::max(hi[a], w);
            }
        }
        float* t = &boxes[9 * (size_t)i];
        for (int a = 0; a < 3; ++a) {
            t[a] = t[6 + a] = Down(lo[a]);
            t[3 + a] = Up(hi[a]);
            out.lo[a] = std::min(out.lo[a], lo[a]);
            out.hi[a] = std::max(out.hi[a], hi[a]);
        }
    }
    if (n == 0) return;
    BuildParams bp;
    BuildBinaryBvh(boxes.data(), n, bp, out.bin);
    CollapseToWide(out.bin, boxes.data(), n, out.wide);
}

}  // namespace RT
}  // namespace Foundation
