// bvh_build.cpp — binned-SAH binary BVH builder (see bvh_build.hpp).
//
// Parallel structure: a shared task stack served by a pool of std::threads.
// A task is one node range; a worker splits it and keeps building the left
// child itself while large right children go back to the shared stack (small
// subtrees stay on the worker). Node pairs come from an atomic counter, so the
// node ORDER depends on timing but the tree (topology, boxes, leaf contents)
// does not: every decision reads only the triangles of its own range, and
// the partition is stable.
#include "bvh_build.hpp"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <condition_variable>
#include <mutex>
#include <numeric>
#include <thread>

#include "../core/core.hpp"

namespace Foundation {
namespace RT {
namespace {

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const Box& b) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], b.lo[i]);
            hi[i] = std::max(hi[i], b.hi[i]);
        }
    }
    void grow_point(const float* p) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], p[i]);
            hi[i] = std::max(hi[i], p[i]);
        }
    }
    float half_area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
};

struct Task {
    uint32_t node, begin, end, depth;
};

constexpr uint32_t kLocalThreshold = 8192;  // subtrees below this stay on one worker

class Builder {
public:
    Builder(const float* tri, uint32_t nt, const BuildParams& p, BinaryBvh& out)
        : m_tri(tri), m_nt(nt), m_p(p), m_out(out) {}

    void Run() {
        const uint32_t threads =
            m_p.threads ? m_p.threads : std::max(1u, (uint32_t)std::thread::hardware_concurrency());
        m_tb.resize(m_nt);
        m_cen.resize(3 * (size_t)m_nt);
        ParallelFor(threads, m_nt, [&](uint32_t s, uint32_t e) {
            for (uint32_t t = s; t < e; ++t) {
                Box b;
                b.grow_point(m_tri + 9 * (size_t)t);
                b.grow_point(m_tri + 9 * (size_t)t + 3);
                b.grow_point(m_tri + 9 * (size_t)t + 6);
                m_tb[t] = b;
                for (int i = 0; i < 3; ++i) m_cen[3 * (size_t)t + i] = (b.lo[i] + b.hi[i]) * 0.5f;
            }
        });
        m_out.prims.resize(m_nt);
        std::iota(m_out.prims.begin(), m_out.prims.end(), 0u);
        m_out.nodes.assign(2 * (size_t)m_nt - 1, BinaryNode{});
        m_next.store(1);
        m_tasks.push_back({0u, 0u, m_nt, 1u});
        m_pending = 1;
        std::vector<std::thread> pool;
        std::vector<double> sah(threads, 0.0);
        std::vector<uint32_t> depth(threads, 0), leaves(threads, 0);
        for (uint32_t i = 0; i < threads; ++i)
            pool.emplace_back([&, i] { Worker(sah[i], depth[i], leaves[i]); });
        for (auto& t : pool) t.join();
        if (m_error) std::rethrow_exception(m_error);
        m_out.nodes.resize(m_next.load());
        double s = 0.0;
        for (double v : sah) s += v;
        m_out.depth = *std::max_element(depth.begin(), depth.end());
        m_out.leaves = 0;
        for (uint32_t v : leaves) m_out.leaves += v;
        const BinaryNode& r = m_out.nodes[0];
        Box rb;
        for (int i = 0; i < 3; ++i) {
            rb.lo[i] = r.lo[i];
            rb.hi[i] = r.hi[i];
        }
        const double ra = rb.half_area();
        m_out.sah_cost = ra > 0.0 ? s / ra : 0.0;
    }

private:
    template <typename F>
    static void ParallelFor(uint32_t threads, uint32_t n, F&& f) {
        const uint32_t chunk = std::max(1u, (n + threads - 1) / threads);
        std::vector<std::thread> pool;
        for (uint32_t s = 0; s < n; s += chunk) pool.emplace_back(f, s, std::min(n, s + chunk));
        for (auto& t : pool) t.join();
    }

    void Worker(double& sah, uint32_t& depth, uint32_t& leaves) {
        std::vector<uint32_t> cnt(m_p.bins), rcnt(m_p.bins);
        std::vector<Box> bb(m_p.bins), rbox(m_p.bins);
        std::vector<Task> local;
        for (;;) {
            Task t;
            {
                std::unique_lock<std::mutex> lk(m_mu);
                m_cv.wait(lk, [&] { return !m_tasks.empty() || m_pending == 0; });
                if (m_tasks.empty()) return;
                t = m_tasks.back();
                m_tasks.pop_back();
            }
            try {
                local.push_back(t);
                while (!local.empty()) {
                    Task cur = local.back();
                    local.pop_back();
                    Task kids[2];
                    const int nk = Split(cur, cnt, rcnt, bb, rbox, sah, depth, leaves, kids);
                    if (nk == 0) continue;
                    // right child: hand big ones to the pool
                    if (kids[1].end - kids[1].begin >= kLocalThreshold) {
                        std::lock_guard<std::mutex> lk(m_mu);
                        m_tasks.push_back(kids[1]);
                        m_pending++;
                        m_cv.notify_one();
                    } else {
                        local.push_back(kids[1]);
                    }
                    local.push_back(kids[0]);
                }
            } catch (...) {
                std::lock_guard<std::mutex> lk(m_mu);
                if (!m_error) m_error = std::current_exception();
                local.clear();
            }
            {
                std::lock_guard<std::mutex> lk(m_mu);
                if (--m_pending == 0) m_cv.notify_all();
            }
        }
    }

    int BinOf(uint32_t p, int ax, float lo, float scale) const {
        int k = (int)((m_cen[3 * (size_t)p + ax] - lo) * scale);
        return std::min(std::max(k, 0), (int)m_p.bins - 1);
    }

    // Returns the number of children (0 = leaf) and fills kids.
    int Split(const Task& t, std::vector<uint32_t>& cnt, std::vector<uint32_t>& rcnt, std::vector<Box>& bb,
              std::vector<Box>& rbox, double& sah, uint32_t& depth, uint32_t& leaves, Task* kids) {
        uint32_t* prims = m_out.prims.data();
        depth = std::max(depth, t.depth);
        Box box, cb;
        for (uint32_t i = t.begin; i < t.end; ++i) {
            box.grow(m_tb[prims[i]]);
            cb.grow_point(&m_cen[3 * (size_t)prims[i]]);
        }
        BinaryNode& nd = m_out.nodes[t.node];
        for (int i = 0; i < 3; ++i) {
            nd.lo[i] = box.lo[i];
            nd.hi[i] = box.hi[i];
        }
        const uint32_t n = t.end - t.begin;
        const double area = box.half_area();
        const uint32_t bins = m_p.bins;
        double best = DBL_MAX;
        int best_axis = -1;
        uint32_t best_bin = 0;
        float best_scale = 0.0f;
        if (n > 1) {
            for (int ax = 0; ax < 3; ++ax) {
                const float ext = cb.hi[ax] - cb.lo[ax];
                if (!(ext > 0.0f)) continue;
                const float scale = (float)bins / ext;
                std::fill(cnt.begin(), cnt.end(), 0u);
                std::fill(bb.begin(), bb.end(), Box());
                for (uint32_t i = t.begin; i < t.end; ++i) {
                    const uint32_t p = prims[i];
                    const int k = BinOf(p, ax, cb.lo[ax], scale);
                    cnt[k]++;
                    bb[k].grow(m_tb[p]);
                }
                Box acc;
                uint32_t c = 0;
                for (int k = (int)bins - 1; k >= 1; --k) {
                    acc.grow(bb[k]);
                    c += cnt[k];
                    rbox[k] = acc;
                    rcnt[k] = c;
                }
                acc = Box();
                c = 0;
                for (uint32_t k = 0; k + 1 < bins; ++k) {
                    acc.grow(bb[k]);
                    c += cnt[k];
                    const uint32_t rc = rcnt[k + 1];
                    if (c == 0 || rc == 0) continue;
                    const double cost = (double)acc.half_area() * (double)c + (double)rbox[k + 1].half_area() * (double)rc;
                    if (cost < best) {
                        best = cost;
                        best_axis = ax;
                        best_bin = k;
                        best_scale = scale;
                    }
                }
            }
        }
        const double split_cost = best_axis >= 0 ? (double)m_p.trav_cost + best / area : DBL_MAX;
        const bool leaf = n <= m_p.max_leaf && (best_axis < 0 || (double)n <= split_cost);
        if (leaf) {
            nd.a = t.begin;
            nd.count = n;
            sah += (double)n * area;
            leaves++;
            return 0;
        }
        uint32_t mid;
        if (best_axis >= 0) {
            const int ax = best_axis;
            const float lo = cb.lo[ax];
            auto it = std::stable_partition(prims + t.begin, prims + t.end,
                                            [&](uint32_t p) { return (uint32_t)BinOf(p, ax, lo, best_scale) <= best_bin; });
            mid = (uint32_t)(it - prims);
        } else {
            std::sort(prims + t.begin, prims + t.end);
            mid = t.begin + n / 2;
        }
        sah += (double)m_p.trav_cost * area;
        const uint32_t left = m_next.fetch_add(2);
        CHECK_CODE(left + 1 < m_out.nodes.size(), FND_ERR_INVALID_SCENE, "BVH node pool exhausted");
        nd.a = left;
        nd.count = 0;
        kids[0] = {left, t.begin, mid, t.depth + 1};
        kids[1] = {left + 1, mid, t.end, t.depth + 1};
        return 2;
    }

    const float* m_tri;
    uint32_t m_nt;
    BuildParams m_p;
    BinaryBvh& m_out;
    std::vector<Box> m_tb;
    std::vector<float> m_cen;
    std::atomic<uint32_t> m_next{0};
    std::mutex m_mu;
    std::condition_variable m_cv;
    std::vector<Task> m_tasks;
    uint64_t m_pending = 0;
    std::exception_ptr m_error;
};

}  // namespace

void BuildBinaryBvh(const float* tri, uint32_t nt, const BuildParams& params, BinaryBvh& out) {
    CHECK(nt > 0);
    CHECK(params.bins >= 2 && params.bins <= 64);
    CHECK(params.max_leaf >= 1 && params.max_leaf <= 4);
    CHECK(params.trav_cost > 0.0f && params.trav_cost <= 64.0f);
    Builder b(tri, nt, params, out);
    b.Run();
}

}  // namespace RT
}  // namespace Foundation
