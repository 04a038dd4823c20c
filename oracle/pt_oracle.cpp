// pt_oracle.cpp — TEST INFRASTRUCTURE ONLY: FP64 path-tracing oracle.
//
// Renders a crop of an image with the light-transport definitions of the
// device integrator (foundation_gb300/csrc/pt/shade.cuh), evaluated in
// double precision over the oracle's binary BVH: pinhole camera (glm lookAt
// convention), two-sided surfaces, one-sided black emitters, Lambert and GGX
// (Walter et al. 2007; height-correlated Smith; Schlick Fresnel; alpha =
// roughness; VNDF sampling, Heitz 2018), next-event estimation to one quad
// light per hit (uniform light choice, uniform point) combined with BSDF
// sampling by the power heuristic (Veach 1997), a directional sun, a
// constant sky, Russian roulette from bounce rr_start with survival
// clamp(max(throughput), 0.05, 1) and at most max_depth interactions.
// Random numbers come from PCG32 streams (O'Neill 2014) in 53-bit doubles;
// the oracle and the device agree in expectation, not sample by sample.
// Parity is unpinned against the reference, which has no path tracer.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle_common.hpp"
#include "rt_oracle.h"
#include "rt_oracle_internal.hpp"

using namespace oracle;

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 norm(V3 a) { return a * (1.0 / std::sqrt(dot(a, a))); }
inline double max3(V3 a) { return std::max(a.x, std::max(a.y, a.z)); }
constexpr double kPi = 3.14159265358979323846;

// Layouts of fnd_material / fnd_quad_light (include/fnd_rt.h).
struct Material {
    uint32_t type;
    float albedo[3];
    float roughness;
    float emission[3];
    int32_t light;
    float reserved[3];
};
static_assert(sizeof(Material) == 48, "material layout");
struct QuadLight {
    float corner[3], edge_u[3], edge_v[3], radiance[3];
};
static_assert(sizeof(QuadLight) == 48, "light layout");

struct Scene {
    const orc_bvh* bvh;
    std::vector<V3> normal;
    const uint32_t* tri_mat;
    const Material* mats;
    uint32_t nm;
    const QuadLight* lights;
    uint32_t nl;
    V3 sky, sun_dir, sun_E;
    bool has_sun;
};

// Double-precision watertight test (same structure as the FP32 one).
bool intersect_d(V3 o, V3 d, int kx, int ky, int kz, double Sx, double Sy, double Sz, const float* v0,
                 const float* v1, const float* v2, double tmax, double& t_out) {
    const double A[3] = {v0[0] - o.x, v0[1] - o.y, v0[2] - o.z};
    const double B[3] = {v1[0] - o.x, v1[1] - o.y, v1[2] - o.z};
    const double C[3] = {v2[0] - o.x, v2[1] - o.y, v2[2] - o.z};
    const double Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
    const double Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
    const double Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
    const double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
    const double det = U + V + W;
    if (det == 0.0) return false;
    const double T = U * (Sz * A[kz]) + V * (Sz * B[kz]) + W * (Sz * C[kz]);
    const double t = T / det;
    if (!(t >= 0.0 && t <= tmax)) return false;
    t_out = t;
    return true;
}

// Closest (any_hit=false) or any hit along o + t d, t in [0, tmax].
bool trace_d(const orc_bvh& b, V3 o, V3 d, double tmax, bool any_hit, uint32_t& prim, double& t_hit) {
    const double ad[3] = {std::fabs(d.x), std::fabs(d.y), std::fabs(d.z)};
    const int kz = (ad[0] >= ad[1]) ? (ad[0] >= ad[2] ? 0 : 2) : (ad[1] >= ad[2] ? 1 : 2);
    const int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
    const double dd[3] = {d.x, d.y, d.z};
    const double Sx = dd[kx] / dd[kz], Sy = dd[ky] / dd[kz], Sz = 1.0 / dd[kz];
    double inv[3];
    for (int i = 0; i < 3; ++i) inv[i] = 1.0 / (std::fabs(dd[i]) < 1e-300 ? std::copysign(1e-300, dd[i]) : dd[i]);
    const double oo[3] = {o.x, o.y, o.z};
    auto box = [&](uint32_t n, double tfar, double& tn_out) {
        const BNodeView& nd = node_view(b, n);
        double tn = 0.0, tf = tfar;
        for (int i = 0; i < 3; ++i) {
            const double t0 = (nd.lo[i] - oo[i]) * inv[i], t1 = (nd.hi[i] - oo[i]) * inv[i];
            tn = std::max(tn, std::min(t0, t1));
            tf = std::min(tf, std::max(t0, t1));
        }
        tn_out = tn;
        return tn <= tf * (1.0 + 1e-12) + 1e-12;
    };
    prim = kInvalid;
    t_hit = tmax;
    if (node_count(b) == 0) return false;
    std::vector<std::pair<uint32_t, double>> stack;
    stack.reserve(64);
    double tn;
    if (!box(0, t_hit, tn)) return false;
    stack.push_back({0u, tn});
    while (!stack.empty()) {
        auto [n, tne] = stack.back();
        stack.pop_back();
        if (tne > t_hit) continue;
        const BNodeView& nd = node_view(b, n);
        if (nd.count) {
            for (uint32_t i = 0; i < nd.count; ++i) {
                const uint32_t p = prim_at(b, nd.a + i);
                const float* v = tri_at(b, p);
                double t;
                if (intersect_d(o, d, kx, ky, kz, Sx, Sy, Sz, v, v + 3, v + 6, t_hit, t)) {
                    if (any_hit) {
                        prim = p;
                        t_hit = t;
                        return true;
                    }
                    if (prim == kInvalid || t < t_hit || (t == t_hit && p < prim)) {
                        prim = p;
                        t_hit = t;
                    }
                }
            }
            continue;
        }
        double tl, tr;
        const bool hl = box(nd.a, t_hit, tl), hr = box(nd.a + 1, t_hit, tr);
        if (hl && hr) {
            if (tr < tl) {
                stack.push_back({nd.a, tl});
                stack.push_back({nd.a + 1, tr});
            } else {
                stack.push_back({nd.a + 1, tr});
                stack.push_back({nd.a, tl});
            }
        } else if (hl) {
            stack.push_back({nd.a, tl});
        } else if (hr) {
            stack.push_back({nd.a + 1, tr});
        }
    }
    return prim != kInvalid;
}

void onb(V3 n, V3& t, V3& b) {
    const double sign = std::copysign(1.0, n.z);
    const double a = -1.0 / (sign + n.z);
    const double c = n.x * n.y * a;
    t = {1.0 + sign * n.x * n.x * a, sign * c, -sign * n.x};
    b = {c, sign + n.y * n.y * a, -n.y};
}

double ggx_D(double ch, double a2) {
    const double d = ch * ch * (a2 - 1.0) + 1.0;
    return a2 / (kPi * d * d);
}
double ggx_Lambda(V3 w, double a2) {
    const double z2 = w.z * w.z;
    const double tan2 = std::max(0.0, 1.0 - z2) / z2;
    return 0.5 * (-1.0 + std::sqrt(1.0 + a2 * tan2));
}
V3 schlick(V3 f0, double c) {
    const double m = std::min(std::max(1.0 - c, 0.0), 1.0);
    const double m5 = m * m * m * m * m;
    return f0 + (V3{1, 1, 1} - f0) * m5;
}

void eval_bsdf(uint32_t type, V3 albedo, double alpha, V3 wo, V3 wi, V3& f, double& pdf) {
    f = {0, 0, 0};
    pdf = 0.0;
    if (wo.z <= 0.0 || wi.z <= 0.0) return;
    if (type == 0) {
        f = albedo * (1.0 / kPi);
        pdf = wi.z / kPi;
        return;
    }
    const double a2 = alpha * alpha;
    const V3 h = norm(wo + wi);
    const double D = ggx_D(h.z, a2);
    const double lo = ggx_Lambda(wo, a2), li = ggx_Lambda(wi, a2);
    f = schlick(albedo, dot(wi, h)) * (D / (1.0 + lo + li) / (4.0 * wo.z * wi.z));
    pdf = D / (1.0 + lo) / (4.0 * wo.z);
}

bool sample_bsdf(uint32_t type, V3 albedo, double alpha, V3 wo, double u1, double u2, V3& wi, V3& weight,
                 double& pdf) {
    if (wo.z <= 0.0) return false;
    if (type == 0) {
        const double r = std::sqrt(u1), ph = 2.0 * kPi * u2;
        const double z = std::sqrt(std::max(0.0, 1.0 - u1));
        wi = {r * std::cos(ph), r * std::sin(ph), z};
        pdf = z / kPi;
        weight = albedo;
        return z > 0.0;
    }
    const double a2 = alpha * alpha;
    const V3 vh = norm(V3{alpha * wo.x, alpha * wo.y, wo.z});
    const double lensq = vh.x * vh.x + vh.y * vh.y;
    const V3 T1 = lensq > 0 ? V3{-vh.y, vh.x, 0.0} * (1.0 / std::sqrt(lensq)) : V3{1, 0, 0};
    const V3 T2 = cross(vh, T1);
    const double r = std::sqrt(u1), ph = 2.0 * kPi * u2;
    const double t1 = r * std::cos(ph);
    double t2 = r * std::sin(ph);
    const double s = 0.5 * (1.0 + vh.z);
    t2 = (1.0 - s) * std::sqrt(std::max(0.0, 1.0 - t1 * t1)) + s * t2;
    const V3 nh = T1 * t1 + T2 * t2 + vh * std::sqrt(std::max(0.0, 1.0 - t1 * t1 - t2 * t2));
    const V3 h = norm(V3{alpha * nh.x, alpha * nh.y, std::max(0.0, nh.z)});
    const double woh = dot(wo, h);
    wi = h * (2.0 * woh) - wo;
    if (wi.z <= 0.0 || woh <= 0.0) return false;
    const double D = ggx_D(h.z, a2);
    const double lo = ggx_Lambda(wo, a2), li = ggx_Lambda(wi, a2);
    pdf = D / (1.0 + lo) / (4.0 * wo.z);
    weight = schlick(albedo, dot(wi, h)) * ((1.0 + lo) / (1.0 + lo + li));
    return pdf > 0.0;
}

double power(double a, double b) {
    const double a2 = a * a, b2 = b * b;
    return a2 + b2 > 0.0 ? a2 / (a2 + b2) : 0.0;
}

struct Params {
    uint32_t width, height, spp, max_depth, rr_start;
    uint64_t seed;
    V3 eye, fwd, right, up;
    double tan_half, aspect, eps;
};

V3 radiance(const Scene& S, const Params& P, V3 o, V3 d, Pcg32& rng) {
    V3 L{0, 0, 0}, beta{1, 1, 1};
    double last_pdf = 0.0;
    for (uint32_t bounce = 0; bounce < P.max_depth; ++bounce) {
        uint32_t prim;
        double t;
        if (!trace_d(*S.bvh, o, d, INFINITY, false, prim, t)) {
            L = L + mul(beta, S.sky);
            break;
        }
        const Material& M = S.mats[std::min(S.tri_mat ? S.tri_mat[prim] : 0u, S.nm - 1)];
        const V3 ng = S.normal[prim];
        const double dn = dot(d, ng);
        const V3 p = o + d * t;
        if (M.type == 2) {
            const V3 Le{M.emission[0], M.emission[1], M.emission[2]};
            if (dn < 0.0 && max3(Le) > 0.0) {
                double w = 1.0;
                if (bounce > 0 && M.light >= 0 && (uint32_t)M.light < S.nl) {
                    const QuadLight& q = S.lights[M.light];
                    const V3 eu{q.edge_u[0], q.edge_u[1], q.edge_u[2]}, ev{q.edge_v[0], q.edge_v[1], q.edge_v[2]};
                    const double area = std::sqrt(dot(cross(eu, ev), cross(eu, ev)));
                    w = power(last_pdf, t * t / (-dn * area * S.nl));
                }
                L = L + mul(beta, Le) * w;
            }
            break;
        }
        const V3 n = dn < 0.0 ? ng : ng * -1.0;
        V3 tb, bb;
        onb(n, tb, bb);
        const V3 wo{-dot(d, tb), -dot(d, bb), -dot(d, n)};
        const V3 albedo{M.albedo[0], M.albedo[1], M.albedo[2]};
        const double alpha = M.roughness;
        const V3 po = p + n * P.eps;
        const double ul = rng.next_double(), u1 = rng.next_double(), u2 = rng.next_double();
        if (S.nl > 0) {
            const uint32_t k = std::min((uint32_t)(ul * S.nl), S.nl - 1);
            const QuadLight& q = S.lights[k];
            const V3 c{q.corner[0], q.corner[1], q.corner[2]}, eu{q.edge_u[0], q.edge_u[1], q.edge_u[2]},
                ev{q.edge_v[0], q.edge_v[1], q.edge_v[2]};
            const V3 cr = cross(eu, ev);
            const double area = std::sqrt(dot(cr, cr));
            const V3 nl = cr * (1.0 / area);
            V3 wl = c + eu * u1 + ev * u2 - po;
            const double d2 = dot(wl, wl), dist = std::sqrt(d2);
            wl = wl * (1.0 / dist);
            const double cos_l = -dot(wl, nl), cos_x = dot(wl, n);
            if (cos_l > 0.0 && cos_x > 0.0) {
                V3 f;
                double pdf_b;
                eval_bsdf(M.type, albedo, alpha, wo, V3{dot(wl, tb), dot(wl, bb), cos_x}, f, pdf_b);
                const double pdf_l = d2 / (cos_l * area * S.nl);
                const V3 c2 = mul(mul(beta, f), V3{q.radiance[0], q.radiance[1], q.radiance[2]}) *
                              (cos_x * power(pdf_l, pdf_b) / pdf_l);
                uint32_t sp;
                double st;
                if (max3(c2) > 0.0 && !trace_d(*S.bvh, po, wl, dist * (1.0 - 1e-3), true, sp, st)) L = L + c2;
            }
        }
        if (S.has_sun) {
            const double cos_x = dot(S.sun_dir, n);
            if (cos_x > 0.0) {
                V3 f;
                double pdf_b;
                eval_bsdf(M.type, albedo, alpha, wo, V3{dot(S.sun_dir, tb), dot(S.sun_dir, bb), cos_x}, f, pdf_b);
                const V3 c2 = mul(mul(beta, f), S.sun_E) * cos_x;
                uint32_t sp;
                double st;
                if (max3(c2) > 0.0 && !trace_d(*S.bvh, po, S.sun_dir, INFINITY, true, sp, st)) L = L + c2;
            }
        }
        const double ub1 = rng.next_double(), ub2 = rng.next_double(), urr = rng.next_double();
        if (bounce + 1 >= P.max_depth) break;
        V3 wi, weight;
        double pdf;
        if (!sample_bsdf(M.type, albedo, alpha, wo, ub1, ub2, wi, weight, pdf)) break;
        beta = mul(beta, weight);
        if (!(max3(beta) > 0.0)) break;
        if (bounce >= P.rr_start) {
            const double q = std::min(std::max(max3(beta), 0.05), 1.0);
            if (urr >= q) break;
            beta = beta * (1.0 / q);
        }
        last_pdf = pdf;
        o = po;
        d = tb * wi.x + bb * wi.y + n * wi.z;
    }
    return L;
}

}  // namespace

extern "C" {

// Renders pixels [x0, x0+cw) x [y0, y0+ch) of a width x height image; out:
// cw*ch*3 doubles, mean radiance per pixel. params: see Params (camera
// vectors in world space, unnormalised eye->target direction allowed).
void orc_pt_render(const orc_bvh* b, const uint32_t* tri_mat, const void* materials, uint32_t nm,
                   const void* lights, uint32_t nl, const double* cam /* eye3 target3 up3 vfov_deg */,
                   uint32_t width, uint32_t height, uint32_t spp, uint32_t max_depth, uint32_t rr_start,
                   uint64_t seed, const double* env /* sky3 sun_dir3 sun_E3 */, uint32_t x0, uint32_t y0,
                   uint32_t cw, uint32_t ch, uint32_t threads, double* out) {
    Scene S;
    S.bvh = b;
    const uint32_t nt = tri_count(*b);
    S.normal.resize(nt);
    for (uint32_t t = 0; t < nt; ++t) {
        const float* v = tri_at(*b, t);
        const V3 a{v[0], v[1], v[2]}, e1 = V3{v[3], v[4], v[5]} - a, e2 = V3{v[6], v[7], v[8]} - a;
        const V3 c = cross(e1, e2);
        const double l = std::sqrt(dot(c, c));
        S.normal[t] = l > 0.0 ? c * (1.0 / l) : V3{0, 0, 1};
    }
    S.tri_mat = tri_mat;
    S.mats = static_cast<const Material*>(materials);
    S.nm = nm;
    S.lights = static_cast<const QuadLight*>(lights);
    S.nl = nl;
    S.sky = {env[0], env[1], env[2]};
    const V3 sd{env[3], env[4], env[5]};
    const double sl = std::sqrt(dot(sd, sd));
    S.has_sun = sl > 0.0 && (env[6] > 0 || env[7] > 0 || env[8] > 0);
    S.sun_dir = sl > 0.0 ? sd * (1.0 / sl) : V3{0, 1, 0};
    S.sun_E = {env[6], env[7], env[8]};
    Params P;
    P.width = width;
    P.height = height;
    P.spp = spp;
    P.max_depth = max_depth;
    P.rr_start = rr_start;
    P.seed = seed;
    P.eye = {cam[0], cam[1], cam[2]};
    P.fwd = norm(V3{cam[3], cam[4], cam[5]} - P.eye);
    P.right = norm(cross(P.fwd, V3{cam[6], cam[7], cam[8]}));
    P.up = cross(P.right, P.fwd);
    P.tan_half = std::tan(cam[9] * kPi / 360.0);
    P.aspect = (double)width / height;
    P.eps = 1e-4;
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint32_t> next{0};
    const uint32_t npx = cw * ch;
    auto worker = [&] {
        for (;;) {
            const uint32_t i = next.fetch_add(1);
            if (i >= npx) break;
            const uint32_t px = x0 + i % cw, py = y0 + i / cw;
            const uint32_t pixel = py * width + px;
            V3 acc{0, 0, 0};
            for (uint32_t s = 0; s < spp; ++s) {
                Pcg32 rng(seed * 0x9E3779B97F4A7C15ull + pixel, 0x5EED0000u + s);
                const double a = rng.next_double(), bj = rng.next_double();
                const double sx = (2.0 * (px + a) / width - 1.0) * P.tan_half * P.aspect;
                const double sy = (1.0 - 2.0 * (py + bj) / height) * P.tan_half;
                const V3 d = norm(P.fwd + P.right * sx + P.up * sy);
                acc = acc + radiance(S, P, P.eye, d, rng);
            }
            out[3 * (size_t)i + 0] = acc.x / spp;
            out[3 * (size_t)i + 1] = acc.y / spp;
            out[3 * (size_t)i + 2] = acc.z / spp;
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t i = 0; i < threads; ++i) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
}

}  // extern "C"
