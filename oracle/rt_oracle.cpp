// rt_oracle.cpp — TEST INFRASTRUCTURE ONLY (see oracle_common.hpp header).
//
// Scalar CPU restatement of: binned-SAH binary BVH build (32 bins, <=4
// triangles per leaf), ordered closest-hit / any-hit traversal with FP32
// watertight intersection, brute-force closest / any hit, and PCG32 streams.
// Exposed as a C API for ctypes (oracle/rt_oracle.h). It doubles as the CPU
// baseline that bench.py times (scalar code, one thread per ray chunk).
//
// Binned SAH: I. Wald, "On fast Construction of SAH-based Bounding Volume
// Hierarchies", IEEE RT 2007 — centroid binning into K bins per axis,
// prefix/suffix sweeps of bin bounds, cost C_trav + C_isect *
// (A_L N_L + A_R N_R) / A_node with C_trav = C_isect = 1.
#include "rt_oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "oracle_common.hpp"
#include "rt_oracle_internal.hpp"

using namespace oracle;

namespace {

struct Aabb {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const Aabb& b) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], b.lo[i]);
            hi[i] = std::max(hi[i], b.hi[i]);
        }
    }
    void grow(const float* p) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], p[i]);
            hi[i] = std::max(hi[i], p[i]);
        }
    }
    // half surface area
    float half_area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
};


void tri_bounds(const orc_bvh& b, uint32_t t, Aabb& box) {
    box = Aabb();
    box.grow(&b.tri[9 * t + 0]);
    box.grow(&b.tri[9 * t + 3]);
    box.grow(&b.tri[9 * t + 6]);
}

struct BuildItem {
    uint32_t node, begin, end, depth;
};

void build(orc_bvh& b, uint32_t bins) {
    const uint32_t n = b.nt;
    std::vector<Aabb> tb(n);
    std::vector<float> cen(3 * (size_t)n);
    for (uint32_t t = 0; t < n; ++t) {
        tri_bounds(b, t, tb[t]);
        for (int i = 0; i < 3; ++i) cen[3 * t + i] = (tb[t].lo[i] + tb[t].hi[i]) * 0.5f;
    }
    b.prims.resize(n);
    std::iota(b.prims.begin(), b.prims.end(), 0u);
    b.nodes.clear();
    b.nodes.push_back(BNode{});
    std::vector<BuildItem> stack{{0u, 0u, n, 1u}};
    std::vector<uint32_t> cnt(bins);
    std::vector<Aabb> bb(bins), right_box(bins);
    std::vector<uint32_t> right_cnt(bins);
    b.depth = 0;
    while (!stack.empty()) {
        const BuildItem it = stack.back();
        stack.pop_back();
        b.depth = std::max(b.depth, it.depth);
        Aabb box, cb;
        for (uint32_t i = it.begin; i < it.end; ++i) {
            box.grow(tb[b.prims[i]]);
            cb.grow(&cen[3 * b.prims[i]]);
        }
        BNode& nd = b.nodes[it.node];
        for (int i = 0; i < 3; ++i) {
            nd.lo[i] = box.lo[i];
            nd.hi[i] = box.hi[i];
        }
        const uint32_t cntn = it.end - it.begin;
        const double area = box.half_area();
        // best binned split
        double best = DBL_MAX;
        int best_axis = -1;
        uint32_t best_bin = 0;
        float best_scale = 0.0f;
        if (cntn > 1) {
            for (int ax = 0; ax < 3; ++ax) {
                const float ext = cb.hi[ax] - cb.lo[ax];
                if (!(ext > 0.0f)) continue;
                const float scale = (float)bins / ext;
                std::fill(cnt.begin(), cnt.end(), 0u);
                std::fill(bb.begin(), bb.end(), Aabb());
                for (uint32_t i = it.begin; i < it.end; ++i) {
                    const uint32_t p = b.prims[i];
                    int k = (int)((cen[3 * p + ax] - cb.lo[ax]) * scale);
                    k = std::min(std::max(k, 0), (int)bins - 1);
                    cnt[k]++;
                    bb[k].grow(tb[p]);
                }
                Aabb acc;
                uint32_t c = 0;
                for (int k = (int)bins - 1; k >= 1; --k) {
                    acc.grow(bb[k]);
                    c += cnt[k];
                    right_box[k] = acc;
                    right_cnt[k] = c;
                }
                acc = Aabb();
                c = 0;
                for (uint32_t k = 0; k + 1 < bins; ++k) {
                    acc.grow(bb[k]);
                    c += cnt[k];
                    const uint32_t rc = right_cnt[k + 1];
                    if (c == 0 || rc == 0) continue;
                    const double cost =
                        (double)acc.half_area() * (double)c + (double)right_box[k + 1].half_area() * (double)rc;
                    if (cost < best) {
                        best = cost;
                        best_axis = ax;
                        best_bin = k;
                        best_scale = scale;
                    }
                }
            }
        }
        const double leaf_cost = (double)cntn;
        const double split_cost = best_axis >= 0 ? 1.0 + best / area : DBL_MAX;
        bool make_leaf = cntn <= b.max_leaf && (best_axis < 0 || leaf_cost <= split_cost);
        uint32_t mid = 0;
        if (!make_leaf) {
            if (best_axis >= 0) {
                const int ax = best_axis;
                const float lo = cb.lo[ax];
                auto first_right = std::stable_partition(
                    b.prims.begin() + it.begin, b.prims.begin() + it.end, [&](uint32_t p) {
                        int k = (int)((cen[3 * p + ax] - lo) * best_scale);
                        k = std::min(std::max(k, 0), (int)bins - 1);
                        return (uint32_t)k <= best_bin;
                    });
                mid = (uint32_t)(first_right - b.prims.begin());
            } else {
                // all centroids coincide: split by triangle index at the median
                std::sort(b.prims.begin() + it.begin, b.prims.begin() + it.end);
                mid = it.begin + cntn / 2;
            }
        }
        if (make_leaf) {
            nd.a = it.begin;
            nd.count = cntn;
            b.sah += (double)cntn * area;
            continue;
        }
        b.sah += area;  // C_trav
        const uint32_t left = (uint32_t)b.nodes.size();
        b.nodes[it.node].a = left;
        b.nodes[it.node].count = 0;
        b.nodes.push_back(BNode{});
        b.nodes.push_back(BNode{});
        // right pushed first so the left subtree is built (and laid out) first
        stack.push_back({left + 1, mid, it.end, it.depth + 1});
        stack.push_back({left, it.begin, mid, it.depth + 1});
    }
    const double root_area = b.nodes.empty() ? 0.0 : Aabb{{b.nodes[0].lo[0], b.nodes[0].lo[1], b.nodes[0].lo[2]},
                                                           {b.nodes[0].hi[0], b.nodes[0].hi[1], b.nodes[0].hi[2]}}
                                                          .half_area();
    b.sah = root_area > 0.0 ? b.sah / root_area : 0.0;
}

// Absolute margin added to every box so that the FP32 slab test below is
// conservative for rays whose origin is within ~50x the scene extent.
float scene_margin(const BNode& root) {
    float s = 0.0f;
    for (int i = 0; i < 3; ++i) {
        s = std::max(s, std::fabs(root.lo[i]));
        s = std::max(s, std::fabs(root.hi[i]));
        s = std::max(s, root.hi[i] - root.lo[i]);
    }
    return s * (1.0f / 65536.0f);
}

struct RayBox {
    float o[3], inv[3];
};

inline RayBox ray_box(const Ray& r) {
    RayBox rb;
    for (int i = 0; i < 3; ++i) {
        rb.o[i] = r.org[i];
        float d = r.dir[i];
        if (std::fabs(d) < 1e-20f) d = std::copysign(1e-20f, d);
        rb.inv[i] = 1.0f / d;
    }
    return rb;
}

inline bool box_hit(const RayBox& rb, const BNode& n, float tmin, float tmax, float& tnear) {
    float tn = tmin, tf = tmax;
    for (int i = 0; i < 3; ++i) {
        const float t0 = (n.lo[i] - rb.o[i]) * rb.inv[i];
        const float t1 = (n.hi[i] - rb.o[i]) * rb.inv[i];
        tn = std::max(tn, std::min(t0, t1));
        tf = std::min(tf, std::max(t0, t1));
    }
    tnear = tn;
    return tn <= tf;
}

template <bool kAny>
Hit trace_one(const orc_bvh& b, const Ray& r, uint64_t& nodes, uint64_t& tris) {
    Hit best{kInvalid, INFINITY};
    if (b.nodes.empty() || b.nt == 0) return best;
    const RayPre rp = precompute(r);
    const RayBox rb = ray_box(r);
    float best_t = r.tmax;
    uint32_t best_p = kInvalid;
    struct Entry {
        uint32_t node;
        float tnear;
    };
    thread_local std::vector<Entry> stack_mem;
    if (stack_mem.size() < (size_t)b.depth + 2) stack_mem.resize((size_t)b.depth + 2);
    Entry* stack = stack_mem.data();
    int sp = 0;
    float tn;
    nodes++;
    if (!box_hit(rb, b.nodes[0], r.tmin, best_t, tn)) return best;
    stack[sp++] = {0u, tn};
    while (sp > 0) {
        const Entry e = stack[--sp];
        if (e.tnear > best_t) continue;
        const BNode& nd = b.nodes[e.node];
        if (nd.count) {
            for (uint32_t i = 0; i < nd.count; ++i) {
                const uint32_t p = b.prims[nd.a + i];
                const float* v = &b.tri[9 * (size_t)p];
                tris++;
                float t;
                if (intersect(rp, v, v + 3, v + 6, t)) {
                    if (kAny) return Hit{p, t};
                    if (best_p == kInvalid || closer(t, p, best_t, best_p)) {
                        best_t = t;
                        best_p = p;
                    }
                }
            }
            continue;
        }
        const uint32_t l = nd.a, rr = nd.a + 1;
        float tl, tr;
        nodes += 2;
        const bool hl = box_hit(rb, b.nodes[l], r.tmin, best_t, tl);
        const bool hr = box_hit(rb, b.nodes[rr], r.tmin, best_t, tr);
        if (hl && hr) {
            if (tr < tl) {
                stack[sp++] = {l, tl};
                stack[sp++] = {rr, tr};
            } else {
                stack[sp++] = {rr, tr};
                stack[sp++] = {l, tl};
            }
        } else if (hl) {
            stack[sp++] = {l, tl};
        } else if (hr) {
            stack[sp++] = {rr, tr};
        }
    }
    if (best_p != kInvalid) {
        best.prim = best_p;
        best.t = best_t;
    }
    return best;
}

template <typename F>
void parallel_chunks(uint64_t n, uint32_t threads, F&& f) {
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = 4096;
    auto worker = [&](uint32_t tid) {
        for (;;) {
            const uint64_t s = next.fetch_add(chunk);
            if (s >= n) break;
            f(tid, s, std::min(n, s + chunk));
        }
    };
    if (threads == 1) {
        worker(0);
        return;
    }
    std::vector<std::thread> pool;
    for (uint32_t i = 0; i < threads; ++i) pool.emplace_back(worker, i);
    for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

orc_bvh* orc_bvh_build(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t bins,
                       uint32_t max_leaf) {
    auto* b = new orc_bvh();
    b->nt = nt;
    b->max_leaf = max_leaf ? max_leaf : 4;
    if (bins < 2) bins = 32;
    b->tri.resize(9 * (size_t)nt);
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k) {
            const uint32_t vi = idx[3 * (size_t)t + k];
            for (int c = 0; c < 3; ++c) b->tri[9 * (size_t)t + 3 * k + c] = vi < nv ? verts[3 * (size_t)vi + c] : NAN;
        }
    if (nt == 0) return b;
    build(*b, bins);
    b->margin = scene_margin(b->nodes[0]);
    for (auto& nd : b->nodes)
        for (int i = 0; i < 3; ++i) {
            nd.lo[i] -= b->margin;
            nd.hi[i] += b->margin;
        }
    return b;
}

void orc_bvh_free(orc_bvh* b) { delete b; }

void orc_bvh_stats(const orc_bvh* b, uint64_t* out, double* sah) {
    uint64_t leaves = 0, maxc = 0;
    for (const auto& n : b->nodes)
        if (n.count) {
            leaves++;
            maxc = std::max<uint64_t>(maxc, n.count);
        }
    out[0] = b->nodes.size();
    out[1] = leaves;
    out[2] = b->depth;
    out[3] = maxc;
    *sah = b->sah;
}

int orc_bvh_validate(const orc_bvh* b) {
    if (b->nt == 0) return b->nodes.empty() ? 0 : 1;
    std::vector<uint32_t> seen(b->nt, 0);
    std::vector<uint32_t> st{0};
    while (!st.empty()) {
        const uint32_t i = st.back();
        st.pop_back();
        const BNode& n = b->nodes[i];
        if (n.count) {
            if (n.count > b->max_leaf) return 2;
            for (uint32_t k = 0; k < n.count; ++k) {
                const uint32_t p = b->prims[n.a + k];
                if (p >= b->nt) return 3;
                seen[p]++;
                Aabb tb;
                tri_bounds(*b, p, tb);
                for (int c = 0; c < 3; ++c)
                    if (tb.lo[c] < n.lo[c] || tb.hi[c] > n.hi[c]) return 4;
            }
        } else {
            for (uint32_t ch = n.a; ch < n.a + 2; ++ch) {
                const BNode& c = b->nodes[ch];
                for (int k = 0; k < 3; ++k)
                    if (c.lo[k] < n.lo[k] || c.hi[k] > n.hi[k]) return 5;
                st.push_back(ch);
            }
        }
    }
    for (uint32_t t = 0; t < b->nt; ++t)
        if (seen[t] != 1) return 6;
    return 0;
}

float orc_bvh_margin(const orc_bvh* b) { return b->margin; }

void orc_trace_closest(const orc_bvh* b, const void* rays, uint64_t n, void* hits, uint32_t threads,
                       uint64_t* stats) {
    const Ray* R = (const Ray*)rays;
    Hit* H = (Hit*)hits;
    std::vector<uint64_t> nn(256, 0), tt(256, 0);
    parallel_chunks(n, threads, [&](uint32_t tid, uint64_t s, uint64_t e) {
        uint64_t a = 0, c = 0;
        for (uint64_t i = s; i < e; ++i) H[i] = trace_one<false>(*b, R[i], a, c);
        nn[tid & 255] += a;
        tt[tid & 255] += c;
    });
    if (stats) {
        stats[0] = std::accumulate(nn.begin(), nn.end(), (uint64_t)0);
        stats[1] = std::accumulate(tt.begin(), tt.end(), (uint64_t)0);
    }
}

void orc_trace_any(const orc_bvh* b, const void* rays, uint64_t n, uint8_t* out, uint32_t threads,
                   uint64_t* stats) {
    const Ray* R = (const Ray*)rays;
    std::vector<uint64_t> nn(256, 0), tt(256, 0);
    parallel_chunks(n, threads, [&](uint32_t tid, uint64_t s, uint64_t e) {
        uint64_t a = 0, c = 0;
        for (uint64_t i = s; i < e; ++i) out[i] = trace_one<true>(*b, R[i], a, c).prim != kInvalid ? 1 : 0;
        nn[tid & 255] += a;
        tt[tid & 255] += c;
    });
    if (stats) {
        stats[0] = std::accumulate(nn.begin(), nn.end(), (uint64_t)0);
        stats[1] = std::accumulate(tt.begin(), tt.end(), (uint64_t)0);
    }
}

void orc_brute_closest(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, const void* rays,
                       uint64_t n, void* hits, uint32_t threads) {
    const Ray* R = (const Ray*)rays;
    Hit* H = (Hit*)hits;
    parallel_chunks(n, threads, [&](uint32_t, uint64_t s, uint64_t e) {
        for (uint64_t i = s; i < e; ++i) {
            const RayPre rp = precompute(R[i]);
            float best_t = INFINITY;
            uint32_t best_p = kInvalid;
            for (uint32_t t = 0; t < nt; ++t) {
                float v[9];
                for (int k = 0; k < 3; ++k) {
                    const uint32_t vi = idx[3 * (size_t)t + k];
                    for (int c = 0; c < 3; ++c) v[3 * k + c] = vi < nv ? verts[3 * (size_t)vi + c] : NAN;
                }
                float th;
                if (intersect(rp, v, v + 3, v + 6, th) && (best_p == kInvalid || closer(th, t, best_t, best_p))) {
                    best_t = th;
                    best_p = t;
                }
            }
            H[i] = Hit{best_p, best_p == kInvalid ? INFINITY : best_t};
        }
    });
}

void orc_brute_any(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, const void* rays,
                   uint64_t n, uint8_t* out, uint32_t threads) {
    const Ray* R = (const Ray*)rays;
    parallel_chunks(n, threads, [&](uint32_t, uint64_t s, uint64_t e) {
        for (uint64_t i = s; i < e; ++i) {
            const RayPre rp = precompute(R[i]);
            uint8_t hit = 0;
            for (uint32_t t = 0; t < nt && !hit; ++t) {
                float v[9];
                for (int k = 0; k < 3; ++k) {
                    const uint32_t vi = idx[3 * (size_t)t + k];
                    for (int c = 0; c < 3; ++c) v[3 * k + c] = vi < nv ? verts[3 * (size_t)vi + c] : NAN;
                }
                float th;
                hit = intersect(rp, v, v + 3, v + 6, th) ? 1 : 0;
            }
            out[i] = hit;
        }
    });
}

// Two-level scenes (fnd_rt_instances_upload): every instance's bottom level
// brute-forced in object space. The ray is mapped by the FP32 rounding of
// the FP64 inverse transform (adjugate / determinant, translation
// -inv(A) b), o' = ((m0 ox + m1 oy) + m2 oz) + m3, d' = (m0 dx + m1 dy) + m2 dz
// in FP32; a hit's id is the instance's prim offset plus the bottom-level
// triangle index, ties broken by that id.
// Geometry: bottom level k owns triangles [tri_base[k], tri_base[k] + tri_count[k])
// of idx (indices into verts); instance i uses level inst_level[i].
static void inverse34(const float* m, float* out) {
    const double a00 = m[0], a01 = m[1], a02 = m[2], a10 = m[4], a11 = m[5], a12 = m[6];
    const double a20 = m[8], a21 = m[9], a22 = m[10];
    const double c00 = a11 * a22 - a12 * a21, c01 = a10 * a22 - a12 * a20, c02 = a10 * a21 - a11 * a20;
    const double det = a00 * c00 - a01 * c01 + a02 * c02;
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
}

// An instance whose FP32 inverse is exactly [I | 0] (bit for bit, so no
// negative zeros) keeps the world ray unchanged: the library skips its
// transform, which would only turn -0 components into +0.
static bool identity34(const float* inv) {
    static const float kId[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    return std::memcmp(inv, kId, sizeof(kId)) == 0;
}

static Ray instance_ray(const float* inv, const Ray& r) {
    if (identity34(inv)) return r;
    Ray o = r;
    for (int i = 0; i < 3; ++i) {
        const float* m = inv + 4 * i;
        o.org[i] = ((m[0] * r.org[0] + m[1] * r.org[1]) + m[2] * r.org[2]) + m[3];
        o.dir[i] = (m[0] * r.dir[0] + m[1] * r.dir[1]) + m[2] * r.dir[2];
    }
    return o;
}

void orc_instances_trace(const float* verts, const uint32_t* idx, const uint32_t* tri_base, const uint32_t* tri_count,
                         const uint32_t* inst_level, const float* inst_transform, const uint32_t* inst_offset,
                         uint32_t n_inst, const void* rays, uint64_t n, void* hits, uint8_t* occluded, int any,
                         uint32_t threads) {
    const Ray* R = (const Ray*)rays;
    std::vector<float> invs(12 * (size_t)n_inst);
    for (uint32_t i = 0; i < n_inst; ++i) inverse34(inst_transform + 12 * (size_t)i, &invs[12 * (size_t)i]);
    parallel_chunks(n, threads, [&](uint32_t, uint64_t s, uint64_t e) {
        for (uint64_t q = s; q < e; ++q) {
            float best_t = INFINITY;
            uint32_t best_p = kInvalid;
            for (uint32_t i = 0; i < n_inst && !(any && best_p != kInvalid); ++i) {
                const RayPre rp = precompute(instance_ray(&invs[12 * (size_t)i], R[q]));
                const uint32_t lv = inst_level[i];
                for (uint32_t t = 0; t < tri_count[lv]; ++t) {
                    const uint32_t* f = idx + 3 * ((size_t)tri_base[lv] + t);
                    float th;
                    if (!intersect(rp, verts + 3 * (size_t)f[0], verts + 3 * (size_t)f[1], verts + 3 * (size_t)f[2], th))
                        continue;
                    const uint32_t gid = inst_offset[i] + t;
                    if (best_p == kInvalid || closer(th, gid, best_t, best_p)) {
                        best_t = th;
                        best_p = gid;
                    }
                    if (any) break;
                }
            }
            if (any)
                occluded[q] = best_p != kInvalid ? 1 : 0;
            else
                ((Hit*)hits)[q] = Hit{best_p, best_p == kInvalid ? INFINITY : best_t};
        }
    });
}

int orc_intersect1(const float* ray8, const float* v9, float* out5) {
    Ray r;
    std::memcpy(&r, ray8, sizeof(Ray));
    const RayPre rp = precompute(r);
    float t = 0.0f, uvw[4] = {0, 0, 0, 0};
    const bool h = intersect(rp, v9, v9 + 3, v9 + 6, t, uvw);
    out5[0] = h ? t : INFINITY;
    for (int i = 0; i < 4; ++i) out5[1 + i] = uvw[i];
    return h ? 1 : 0;
}

void orc_pcg32_fill(uint64_t seed, uint64_t seq, uint32_t* out, uint64_t n) {
    Pcg32 g(seed, seq);
    for (uint64_t i = 0; i < n; ++i) out[i] = g.next();
}

double orc_time_build_ms(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t bins,
                         uint32_t max_leaf) {
    const auto t0 = std::chrono::steady_clock::now();
    orc_bvh* b = orc_bvh_build(verts, nv, idx, nt, bins, max_leaf);
    const auto t1 = std::chrono::steady_clock::now();
    orc_bvh_free(b);
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

}  // extern "C"
