// bvh_build.cpp — binned-SAH binary BVH builder (see bvh_build.hpp).
//
// Data: one 32-byte record per triangle (box and index) that the partitions
// move, so every pass over a node streams its own contiguous records; a
// triangle's centroid is (lo + hi) / 2, recomputed where it is needed. Each
// task carries its range's box and centroid box, computed while its parent's
// partition wrote the range, and one pass over the records bins all three
// axes at once.
//
// Parallel structure, two phases:
//  1. nodes of more than nt / (4 threads) triangles (and at least 2^16), one
//     at a time with every thread: each bins its chunk of the range into its
//     own bins, the bins are merged, and the stable partition scatters the
//     chunks through per-chunk prefix counts into a second record array;
//  2. the remaining subtrees from a shared task stack served by a pool of
//     std::threads: a worker splits a range and keeps building the left child
//     itself while large right children go back to the stack.
// Node pairs come from a counter, so the node ORDER depends on timing but the
// tree (topology, boxes, leaf contents) does not: every decision reads only
// its own range, bin merging is a min / max / count, and the partition is
// stable. The decisions and their arithmetic are those of the per-node loop
// of Wald 2007 as bvh_build.hpp states them.
#include "bvh_build.hpp"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <condition_variable>
#include <cstring>
#include <mutex>
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
    void grow(const Aabb& b) {
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

// A triangle's box and index: what the partitions move (no default member
// values, so the record arrays are allocated without a fill).
struct Ref {
    Aabb box;
    uint32_t id;
    uint32_t pad;
    void centroid(float c[3]) const {
        for (int i = 0; i < 3; ++i) c[i] = (box.lo[i] + box.hi[i]) * 0.5f;
    }
};
static_assert(sizeof(Ref) == 32, "triangle record");
using RefVector = std::vector<Ref, NoInitAllocator<Ref>>;

struct Task {
    uint32_t node, begin, end, depth;
    Box box, cbox;  // of the range's triangles and of their centroids
};

constexpr uint32_t kLocalThreshold = 8192;  // subtrees below this stay on one worker
constexpr uint32_t kMaxBins = 64;

// Per-axis bins of one range. Only the bins set in occ hold values: a bin
// is written whole by its first triangle, so no bin is cleared.
struct Bins {
    uint64_t occ[3];
    uint32_t cnt[3][kMaxBins];
    Aabb box[3][kMaxBins];
    void clear() { occ[0] = occ[1] = occ[2] = 0; }
    void add(int a, uint32_t k, const Aabb& b) {
        if (occ[a] >> k & 1u) {
            cnt[a][k]++;
            Aabb& d = box[a][k];
            for (int i = 0; i < 3; ++i) {
                d.lo[i] = std::min(d.lo[i], b.lo[i]);
                d.hi[i] = std::max(d.hi[i], b.hi[i]);
            }
        } else {
            occ[a] |= 1ull << k;
            cnt[a][k] = 1;
            box[a][k] = b;
        }
    }
    void merge(const Bins& o) {
        for (int a = 0; a < 3; ++a)
            for (uint64_t m = o.occ[a]; m; m &= m - 1) {
                const uint32_t k = (uint32_t)__builtin_ctzll(m);
                if (occ[a] >> k & 1u) {
                    cnt[a][k] += o.cnt[a][k];
                    Aabb& d = box[a][k];
                    for (int i = 0; i < 3; ++i) {
                        d.lo[i] = std::min(d.lo[i], o.box[a][k].lo[i]);
                        d.hi[i] = std::max(d.hi[i], o.box[a][k].hi[i]);
                    }
                } else {
                    occ[a] |= 1ull << k;
                    cnt[a][k] = o.cnt[a][k];
                    box[a][k] = o.box[a][k];
                }
            }
    }
};

// The split plane of a range: axis (-1: none), bin, grid.
struct Plane {
    int axis = -1;
    uint32_t bin = 0;
    float lo = 0.0f, scale = 0.0f;
    double cost = DBL_MAX;  // A_L N_L + A_R N_R
};

template <typename F>
void ParallelFor(uint32_t threads, uint32_t n, F&& f) {
    const uint32_t parts = std::max(1u, std::min(threads, n));
    const uint32_t chunk = (n + parts - 1) / parts;
    std::vector<std::thread> pool;
    for (uint32_t p = 1; p < parts; ++p) {
        const uint32_t s = p * chunk;
        if (s < n) pool.emplace_back(f, p, s, std::min(n, s + chunk));
    }
    f(0u, 0u, std::min(n, chunk));
    for (auto& t : pool) t.join();
}

class Builder {
public:
    Builder(const float* tri, uint32_t nt, const BuildParams& p, BinaryBvh& out)
        : m_tri(tri), m_nt(nt), m_p(p), m_out(out) {}

    void Run() {
        m_threads = m_p.threads ? m_p.threads : std::max(1u, (uint32_t)std::thread::hardware_concurrency());
        m_refs.resize(m_nt);
        // records, and the root's box and centroid box
        std::vector<Box> pb(m_threads), pc(m_threads);
        ParallelFor(m_threads, m_nt, [&](uint32_t w, uint32_t s, uint32_t e) {
            for (uint32_t t = s; t < e; ++t) {
                Ref& r = m_refs[t];
                Box b;
                b.grow_point(m_tri + 9 * (size_t)t);
                b.grow_point(m_tri + 9 * (size_t)t + 3);
                b.grow_point(m_tri + 9 * (size_t)t + 6);
                for (int i = 0; i < 3; ++i) {
                    r.box.lo[i] = b.lo[i];
                    r.box.hi[i] = b.hi[i];
                }
                r.id = t;
                r.pad = 0;
                float c[3];
                r.centroid(c);
                pb[w].grow(r.box);
                pc[w].grow_point(c);
            }
        });
        Task root{0u, 0u, m_nt, 1u, Box(), Box()};
        for (uint32_t w = 0; w < m_threads; ++w) {
            root.box.grow(pb[w]);
            root.cbox.grow(pc[w]);
        }
        m_out.nodes.resize(2 * (size_t)m_nt - 1);  // every node used is written
        m_next.store(1);
        double sah = 0.0;
        uint32_t depth = 0, leaves = 0;
        // phase 1: large nodes with every thread
        const uint32_t big = std::max<uint32_t>(1u << 16, m_nt / (4 * m_threads));
        std::vector<Task> top{root};
        while (!top.empty()) {
            Task t = top.back();
            top.pop_back();
            if (t.end - t.begin < big || m_threads == 1) {
                m_tasks.push_back(t);
                continue;
            }
            Task kids[2];
            if (SplitWide(t, sah, depth, leaves, kids) == 0) continue;
            top.push_back(kids[1]);
            top.push_back(kids[0]);
        }
        // phase 2: the remaining subtrees
        m_pending = m_tasks.size();
        std::vector<std::thread> pool;
        std::vector<double> wsah(m_threads, 0.0);
        std::vector<uint32_t> wdepth(m_threads, 0), wleaves(m_threads, 0);
        for (uint32_t i = 0; i < m_threads; ++i)
            pool.emplace_back([&, i] { Worker(wsah[i], wdepth[i], wleaves[i]); });
        for (auto& t : pool) t.join();
        if (m_error) std::rethrow_exception(m_error);
        m_out.nodes.resize(m_next.load());
        for (uint32_t i = 0; i < m_threads; ++i) {
            sah += wsah[i];
            depth = std::max(depth, wdepth[i]);
            leaves += wleaves[i];
        }
        m_out.prims.resize(m_nt);
        ParallelFor(m_threads, m_nt, [&](uint32_t, uint32_t s, uint32_t e) {
            for (uint32_t i = s; i < e; ++i) m_out.prims[i] = m_refs[i].id;
        });
        m_out.depth = depth;
        m_out.leaves = leaves;
        const double ra = root.box.half_area();
        m_out.sah_cost = ra > 0.0 ? sah / ra : 0.0;
    }

private:
    int BinOf(float c, const Plane& g) const {
        const int k = (int)((c - g.lo) * g.scale);
        return std::min(std::max(k, 0), (int)m_p.bins - 1);
    }

    // Bins records [s, e) along the axes whose centroid extent is positive.
    void BinRange(uint32_t s, uint32_t e, const Plane* grid, Bins& b) const {
        const bool on[3] = {grid[0].scale > 0.0f, grid[1].scale > 0.0f, grid[2].scale > 0.0f};
        for (uint32_t i = s; i < e; ++i) {
            const Ref& r = m_refs[i];
            float c[3];
            r.centroid(c);
            for (int a = 0; a < 3; ++a)
                if (on[a]) b.add(a, (uint32_t)BinOf(c[a], grid[a]), r.box);
        }
    }

    // The centroid grids of a range (scale 0: the axis is not binned).
    void Grids(const Task& t, Plane* grid) const {
        for (int a = 0; a < 3; ++a) {
            const float ext = t.cbox.hi[a] - t.cbox.lo[a];
            grid[a].lo = t.cbox.lo[a];
            grid[a].scale = ext > 0.0f ? (float)m_p.bins / ext : 0.0f;
        }
    }

    // The sweep over the bins: the least A_L N_L + A_R N_R, axes x, y, z and
    // bins in order, the first minimum winning. Only occupied bins are
    // candidates: after an empty bin the two sides are those of the bin
    // before it, whose equal cost came first; the boxes and counts summed
    // are those of the sweep over all bins.
    static Plane Sweep(const Bins& b, const Plane* grid) {
        Plane best;
        uint32_t rcnt[kMaxBins];
        Box rbox[kMaxBins];
        for (int a = 0; a < 3; ++a) {
            if (!(grid[a].scale > 0.0f)) continue;
            const uint64_t occ = b.occ[a];
            if (!(occ & (occ - 1))) continue;  // fewer than two occupied bins
            Box acc;
            uint32_t c = 0;
            for (uint64_t m = occ; m;) {  // descending
                const uint32_t k = 63u - (uint32_t)__builtin_clzll(m);
                m &= ~(1ull << k);
                acc.grow(b.box[a][k]);
                c += b.cnt[a][k];
                rbox[k] = acc;
                rcnt[k] = c;
            }
            acc = Box();
            c = 0;
            for (uint64_t m = occ; m & (m - 1);) {  // ascending, all but the last
                const uint32_t k = (uint32_t)__builtin_ctzll(m);
                m &= m - 1;
                const uint32_t next = (uint32_t)__builtin_ctzll(m);
                acc.grow(b.box[a][k]);
                c += b.cnt[a][k];
                const double cost =
                    (double)acc.half_area() * (double)c + (double)rbox[next].half_area() * (double)rcnt[next];
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = a;
                    best.bin = k;
                    best.lo = grid[a].lo;
                    best.scale = grid[a].scale;
                }
            }
        }
        return best;
    }

    // The node of t and its split decision; true for a leaf.
    bool Decide(const Task& t, const Plane& plane, double& sah, uint32_t& depth, uint32_t& leaves) {
        depth = std::max(depth, t.depth);
        BinaryNode& nd = m_out.nodes[t.node];
        for (int i = 0; i < 3; ++i) {
            nd.lo[i] = t.box.lo[i];
            nd.hi[i] = t.box.hi[i];
        }
        const uint32_t n = t.end - t.begin;
        const double area = t.box.half_area();
        const double split_cost = plane.axis >= 0 ? (double)m_p.trav_cost + plane.cost / area : DBL_MAX;
        const bool leaf = n <= m_p.max_leaf && (plane.axis < 0 || (double)n <= split_cost);
        if (leaf) {
            nd.a = t.begin;
            nd.count = n;
            sah += (double)n * area;
            leaves++;
        } else {
            sah += (double)m_p.trav_cost * area;
        }
        return leaf;
    }

    void MakeKids(const Task& t, uint32_t mid, const Box* side_box, const Box* side_cbox, Task* kids) {
        const uint32_t left = m_next.fetch_add(2);
        CHECK_CODE(left + 1 < m_out.nodes.size(), FND_ERR_INVALID_SCENE, "BVH node pool exhausted");
        BinaryNode& nd = m_out.nodes[t.node];
        nd.a = left;
        nd.count = 0;
        kids[0] = {left, t.begin, mid, t.depth + 1, side_box[0], side_cbox[0]};
        kids[1] = {left + 1, mid, t.end, t.depth + 1, side_box[1], side_cbox[1]};
    }

    // No axis to bin on (all centroids coincide): the median of the indices.
    void SplitByIndex(const Task& t, Box* side_box, Box* side_cbox, uint32_t& mid) {
        std::sort(m_refs.begin() + t.begin, m_refs.begin() + t.end,
                  [](const Ref& a, const Ref& b) { return a.id < b.id; });
        mid = t.begin + (t.end - t.begin) / 2;
        for (uint32_t i = t.begin; i < t.end; ++i) {
            float c[3];
            m_refs[i].centroid(c);
            side_box[i >= mid].grow(m_refs[i].box);
            side_cbox[i >= mid].grow_point(c);
        }
    }

    // Phase 1: one node with every thread. Returns the number of children.
    int SplitWide(const Task& t, double& sah, uint32_t& depth, uint32_t& leaves, Task* kids) {
        Plane grid[3];
        Grids(t, grid);
        const uint32_t n = t.end - t.begin;
        const uint32_t parts = std::min(m_threads, n);
        std::vector<Bins> bins(parts);
        for (Bins& b : bins) b.clear();
        ParallelFor(m_threads, n, [&](uint32_t w, uint32_t s, uint32_t e) {
            BinRange(t.begin + s, t.begin + e, grid, bins[w]);
        });
        for (uint32_t w = 1; w < parts; ++w) bins[0].merge(bins[w]);
        const Plane plane = n > 1 ? Sweep(bins[0], grid) : Plane();
        if (Decide(t, plane, sah, depth, leaves)) return 0;
        Box side_box[2], side_cbox[2];
        uint32_t mid;
        if (plane.axis < 0) {
            SplitByIndex(t, side_box, side_cbox, mid);
        } else {
            // stable partition: per chunk the left count, then every chunk
            // scatters to its offsets in m_tmp; child boxes per chunk
            if (m_tmp.size() < m_nt) m_tmp.resize(m_nt);
            std::vector<uint32_t> lcount(parts, 0);
            std::vector<Box> cb(4 * parts);
            const uint32_t chunk = (n + parts - 1) / parts;
            ParallelFor(m_threads, n, [&](uint32_t w, uint32_t s, uint32_t e) {
                uint32_t c = 0;
                for (uint32_t i = t.begin + s; i < t.begin + e; ++i) {
                    float cc[3];
                    m_refs[i].centroid(cc);
                    c += (uint32_t)BinOf(cc[plane.axis], plane) <= plane.bin;
                }
                lcount[w] = c;
            });
            uint32_t total_left = 0;
            std::vector<uint32_t> loff(parts), roff(parts);
            for (uint32_t w = 0; w < parts; ++w) {
                loff[w] = total_left;
                total_left += lcount[w];
            }
            uint32_t r = total_left;
            for (uint32_t w = 0; w < parts; ++w) {
                roff[w] = r;
                r += std::min(n, (w + 1) * chunk) - std::min(n, w * chunk) - lcount[w];
            }
            ParallelFor(m_threads, n, [&](uint32_t w, uint32_t s, uint32_t e) {
                uint32_t l = t.begin + loff[w], rr = t.begin + roff[w];
                for (uint32_t i = t.begin + s; i < t.begin + e; ++i) {
                    const Ref& ref = m_refs[i];
                    float cc[3];
                    ref.centroid(cc);
                    const bool left = (uint32_t)BinOf(cc[plane.axis], plane) <= plane.bin;
                    m_tmp[left ? l++ : rr++] = ref;
                    cb[4 * w + (left ? 0 : 1)].grow(ref.box);
                    cb[4 * w + (left ? 2 : 3)].grow_point(cc);
                }
            });
            ParallelFor(m_threads, n, [&](uint32_t, uint32_t s, uint32_t e) {
                std::memcpy(&m_refs[t.begin + s], &m_tmp[t.begin + s], sizeof(Ref) * (size_t)(e - s));
            });
            for (uint32_t w = 0; w < parts; ++w) {
                side_box[0].grow(cb[4 * w]);
                side_box[1].grow(cb[4 * w + 1]);
                side_cbox[0].grow(cb[4 * w + 2]);
                side_cbox[1].grow(cb[4 * w + 3]);
            }
            mid = t.begin + total_left;
        }
        MakeKids(t, mid, side_box, side_cbox, kids);
        return 2;
    }

    // Phase 2: one node on this worker. Returns the number of children.
    int Split(const Task& t, Bins& b, RefVector& tmp, double& sah, uint32_t& depth, uint32_t& leaves,
              Task* kids) {
        const uint32_t n = t.end - t.begin;
        Plane plane;
        Plane grid[3];
        if (n > 1) {
            Grids(t, grid);
            b.clear();
            BinRange(t.begin, t.end, grid, b);
            plane = Sweep(b, grid);
        }
        if (Decide(t, plane, sah, depth, leaves)) return 0;
        Box side_box[2], side_cbox[2];
        uint32_t mid;
        if (plane.axis < 0) {
            SplitByIndex(t, side_box, side_cbox, mid);
        } else {
            // stable partition through tmp: lefts in order, then rights
            if (tmp.size() < n) tmp.resize(n);
            uint32_t l = 0;
            for (uint32_t i = t.begin; i < t.end; ++i) {
                float cc[3];
                m_refs[i].centroid(cc);
                if ((uint32_t)BinOf(cc[plane.axis], plane) <= plane.bin) {
                    m_refs[t.begin + l++] = m_refs[i];
                    side_box[0].grow(m_refs[i].box);
                    side_cbox[0].grow_point(cc);
                } else {
                    tmp[i - t.begin - l] = m_refs[i];
                    side_box[1].grow(m_refs[i].box);
                    side_cbox[1].grow_point(cc);
                }
            }
            std::memcpy(&m_refs[t.begin + l], tmp.data(), sizeof(Ref) * (size_t)(n - l));
            mid = t.begin + l;
        }
        MakeKids(t, mid, side_box, side_cbox, kids);
        return 2;
    }

    void Worker(double& sah, uint32_t& depth, uint32_t& leaves) {
        Bins bins;
        RefVector tmp;
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
                    const int nk = Split(cur, bins, tmp, sah, depth, leaves, kids);
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

    const float* m_tri;
    uint32_t m_nt;
    BuildParams m_p;
    BinaryBvh& m_out;
    uint32_t m_threads = 1;
    RefVector m_refs, m_tmp;
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
    CHECK(params.bins >= 2 && params.bins <= kMaxBins);
    CHECK(params.max_leaf >= 1 && params.max_leaf <= 4);
    CHECK(params.trav_cost > 0.0f && params.trav_cost <= 64.0f);
    Builder b(tri, nt, params, out);
    b.Run();
}

}  // namespace RT
}  // namespace Foundation
