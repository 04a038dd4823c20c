// mlp_oracle.cpp — TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// radiance-cache network (forward, relative-L2 loss, backward, Adam) and of
// its input encoding, the checker of the device kernels in
// foundation_gb300/csrc/nrc/.
//
// Network: 96 -> 64 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU on the five hidden
// layers, linear output, no biases (the fully fused MLP of Müller et al.,
// "Real-time Neural Radiance Caching for Path Tracing", 2021). Weights are
// row-major W[K][N] per layer, layer after layer in one flat array.
// Loss: mean over samples and RGB of (y - t)^2 / (y^2 + 0.01) with y held
// constant in the denominator (relative L2 of the same paper).
// Adam: Kingma & Ba 2015, beta1 0.9, beta2 0.99, eps 1e-8.
//
// With emulate_bf16 != 0 the inputs, hidden activations and backpropagated
// pre-activation gradients are rounded to bfloat16 (round to nearest even)
// at the points where the device kernels round them, and all sums run in
// double; otherwise every value is double.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int kLayers = 6;
constexpr int kDims[kLayers + 1] = {96, 64, 64, 64, 64, 64, 3};

double bf16(double x) {
    float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return f;  // inf / nan unchanged
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7FFFu + lsb;
    u &= 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

size_t offset_of(int l) {
    size_t o = 0;
    for (int i = 0; i < l; ++i) o += (size_t)kDims[i] * kDims[i + 1];
    return o;
}

}  // namespace

extern "C" {

uint64_t orc_mlp_num_params() { return offset_of(kLayers); }

// x: B x 96 inputs, w: parameters (as stored, e.g. bf16 values widened to
// float), t: B x 3 targets (may be NULL: forward only). Outputs: y (B x 3),
// loss (scalar, may be NULL), dw (gradient of the loss, may be NULL).
// fixed_den (B x 3, may be NULL): use these denominators instead of y^2 +
// 0.01, so the loss value is the function whose gradient dw is (used by the
// finite-difference check; the training loss treats the denominator as a
// constant, which is this with fixed_den = y^2 + 0.01 at the current y).
void orc_mlp_forward_backward(const float* w, const float* x, const float* t, uint64_t B, int emulate_bf16,
                              double* y, double* loss, double* dw, const double* fixed_den) {
    const size_t np = offset_of(kLayers);
    std::vector<double> W(np);
    for (size_t i = 0; i < np; ++i) W[i] = w[i];
    if (dw) std::memset(dw, 0, sizeof(double) * np);
    double total = 0.0;
    std::vector<std::vector<double>> act(kLayers + 1);
    for (int l = 0; l <= kLayers; ++l) act[l].assign(kDims[l], 0.0);
    std::vector<double> g(64), gn(96);
    for (uint64_t b = 0; b < B; ++b) {
        for (int k = 0; k < kDims[0]; ++k) act[0][k] = emulate_bf16 ? bf16(x[b * 96 + k]) : x[b * 96 + k];
        for (int l = 0; l < kLayers; ++l) {
            const int K = kDims[l], N = kDims[l + 1];
            const double* Wl = &W[offset_of(l)];
            for (int n = 0; n < N; ++n) {
                double z = 0.0;
                for (int k = 0; k < K; ++k) z += act[l][k] * Wl[(size_t)k * N + n];
                if (l + 1 < kLayers) {
                    z = z > 0.0 ? z : 0.0;
                    if (emulate_bf16) z = bf16(z);
                }
                act[l + 1][n] = z;
            }
        }
        for (int c = 0; c < 3; ++c) y[b * 3 + c] = act[kLayers][c];
        if (!t) continue;
        // loss and its gradient wrt the output
        std::vector<double> dz(3);
        for (int c = 0; c < 3; ++c) {
            const double yy = act[kLayers][c], tt = t[b * 3 + c];
            const double den = fixed_den ? fixed_den[b * 3 + c] : yy * yy + 0.01;
            total += (yy - tt) * (yy - tt) / den;
            dz[c] = 2.0 * (yy - tt) / den / (double)(B * 3);
            if (emulate_bf16) dz[c] = bf16(dz[c]);
        }
        if (!dw) continue;
        std::vector<double> dcur = dz;
        for (int l = kLayers - 1; l >= 0; --l) {
            const int K = kDims[l], N = kDims[l + 1];
            const double* Wl = &W[offset_of(l)];
            double* dWl = &dw[offset_of(l)];
            for (int k = 0; k < K; ++k)
                for (int n = 0; n < N; ++n) dWl[(size_t)k * N + n] += act[l][k] * dcur[n];
            if (l == 0) break;
            std::vector<double> dprev(K);
            for (int k = 0; k < K; ++k) {
                double s = 0.0;
                for (int n = 0; n < N; ++n) s += dcur[n] * Wl[(size_t)k * N + n];
                s = act[l][k] > 0.0 ? s : 0.0;  // ReLU derivative from the stored activation
                dprev[k] = emulate_bf16 ? bf16(s) : s;
            }
            dcur.swap(dprev);
        }
    }
    if (loss) *loss = total / (double)(B * 3);
}

// One Adam step (step counts from 1) on FP64 copies of the state.
void orc_adam_step(double* w, double* m, double* v, const double* g, uint64_t n, uint64_t step, double lr) {
    const double b1 = 0.9, b2 = 0.99, eps = 1e-8;
    const double c1 = 1.0 - std::pow(b1, (double)step), c2 = 1.0 - std::pow(b2, (double)step);
    for (uint64_t i = 0; i < n; ++i) {
        m[i] = b1 * m[i] + (1.0 - b1) * g[i];
        v[i] = b2 * v[i] + (1.0 - b2) * g[i] * g[i];
        w[i] -= lr * (m[i] / c1) / (std::sqrt(v[i] / c2) + eps);
    }
}

// Input encoding of one cache query: position normalised to the scene box,
// 12 sine / cosine bands per axis (sin(2^k pi p), cos(2^k pi p)), outgoing
// direction, normal, roughness, albedo, zero padding to 96.
void orc_nrc_encode(const float* rec /* p3, wo3, n3, rough, albedo3 */, const float* lo, const float* hi,
                    float* out96) {
    const double kPi = 3.14159265358979323846;
    int o = 0;
    for (int a = 0; a < 3; ++a) {
        const double ext = (double)hi[a] - (double)lo[a];
        const double p = ext > 0.0 ? ((double)rec[a] - (double)lo[a]) / ext : 0.0;
        for (int k = 0; k < 12; ++k) {
            const double arg = std::ldexp(p, k) * kPi;
            out96[o++] = (float)std::sin(arg);
            out96[o++] = (float)std::cos(arg);
        }
    }
    for (int i = 3; i < 13; ++i) out96[o++] = rec[i];
    while (o < 96) out96[o++] = 0.0f;
}

}  // extern "C"
