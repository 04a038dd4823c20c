// sbvh_build.cpp — binary BVH with spatial splits (optional build mode).
//
// Method: Stich, Friedrich & Dietrich, "Spatial Splits in Bounding Volume
// Hierarchies", HPG 2009. Leaves hold references (a triangle plus a box that
// may be a clipped part of the triangle's box). At each node the best binned
// object split (SAH over reference-box centroids) is compared with the best
// spatial split when the object split's children overlap by more than
// alpha x the root's half area: the node box is cut into K equal slabs, each
// reference is clipped to every slab it spans (exact triangle / slab
// clipping, intersected with the reference's current box), and a reference
// crossing the chosen plane is duplicated into both children with clipped
// boxes. The duplicates are capped (max_refs_factor x triangles extra
// references, one atomic count shared by the build threads); once the budget
// is used, nodes fall back to object splits, so a build that exhausts it may
// split different nodes from run to run.
// Closest-hit results do not depend on the tree (ties break by triangle
// index), so a duplicated reference cannot change any hit.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <mutex>
#include <thread>
#include <vector>

#include "../core/core.hpp"
#include "bvh_build.hpp"

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
    bool empty() const { return lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]; }
    float half_area() const {
        if (empty()) return 0.0f;
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
    Box intersect(const Box& b) const {
        Box r;
        for (int i = 0; i < 3; ++i) {
            r.lo[i] = std::max(lo[i], b.lo[i]);
            r.hi[i] = std::min(hi[i], b.hi[i]);
        }
        return r;
    }
};

struct Ref {
    uint32_t tri;
    Box box;
    float centroid(int a) const { return (box.lo[a] + box.hi[a]) * 0.5f; }
};

// Box of the part of triangle t inside the slab lo <= x[axis] <= hi.
Box ClipTriangle(const float* tri, int axis, float lo, float hi) {
    Box b;
    const float* v[3] = {tri, tri + 3, tri + 6};
    for (int i = 0; i < 3; ++i) {
        const float* p = v[i];
        const float* q = v[(i + 1) % 3];
        const float pa = p[axis], qa = q[axis];
        if (pa >= lo && pa <= hi) b.grow_point(p);
        // edge crossings of the two slab planes
        for (float plane : {lo, hi}) {
            if ((pa < plane && qa > plane) || (pa > plane && qa < plane)) {
                const float s = (plane - pa) / (qa - pa);
                float x[3];
                for (int c = 0; c < 3; ++c) x[c] = p[c] + (q[c] - p[c]) * s;
                x[axis] = plane;
                b.grow_point(x);
            }
        }
    }
    return b;
}

struct Split {
    double cost = DBL_MAX;
    int axis = -1;
    int bin = 0;
    bool spatial = false;
    float pos = 0.0f;   // spatial: plane position
    float scale = 0.0f; // object: centroid bin scale
    float clo = 0.0f;   // object: centroid bin origin
};

struct Out {
    std::vector<BinaryNode, NoInitAllocator<BinaryNode>> nodes;
    std::vector<uint32_t, NoInitAllocator<uint32_t>> prims;
    uint32_t depth = 0, leaves = 0;
    double sah = 0.0;
};

class SbvhBuilder {
public:
    SbvhBuilder(const float* tri, uint32_t nt, const BuildParams& p, float root_half_area)
        : m_tri(tri), m_nt(nt), m_p(p), m_root_area(root_half_area) {
        m_budget = (uint64_t)(p.max_refs_factor * (double)nt);
    }

    // Builds the subtree of `refs` into `out`, node 0 of `out` its root.
    void Build(std::vector<Ref>&& refs, uint32_t depth0, Out& out) {
        struct Item {
            uint32_t node;
            std::vector<Ref> refs;
            uint32_t depth;
        };
        out.nodes.push_back(BinaryNode{});
        std::vector<Item> stack;
        stack.push_back({0u, std::move(refs), depth0});
        while (!stack.empty()) {
            Item it = std::move(stack.back());
            stack.pop_back();
            out.depth = std::max(out.depth, it.depth);
            std::vector<Ref> L, R;
            if (!SplitNode(it.refs, out, it.node, L, R)) continue;
            const uint32_t left = (uint32_t)out.nodes.size();
            out.nodes[it.node].a = left;
            out.nodes[it.node].count = 0;
            out.nodes.push_back(BinaryNode{});
            out.nodes.push_back(BinaryNode{});
            stack.push_back({left + 1, std::move(R), it.depth + 1});
            stack.push_back({left, std::move(L), it.depth + 1});
        }
    }

    // Splits refs at the root levels until there are enough independent
    // subtrees, then builds those in parallel and stitches them.
    void BuildParallel(std::vector<Ref>&& refs, BinaryBvh& result) {
        const uint32_t threads =
            m_p.threads ? m_p.threads : std::max(1u, (uint32_t)std::thread::hardware_concurrency());
        struct Job {
            uint32_t node;  // placeholder node in `top`
            std::vector<Ref> refs;
            uint32_t depth;
        };
        Out top;
        top.nodes.push_back(BinaryNode{});
        std::vector<Job> frontier;
        frontier.push_back({0u, std::move(refs), 1u});
        std::vector<Job> jobs;
        const size_t want = 4 * (size_t)threads;
        const size_t small = std::max<size_t>(4096, m_nt / (8 * (size_t)threads));
        while (!frontier.empty()) {
            // split the largest frontier item until enough jobs exist
            auto big = std::max_element(frontier.begin(), frontier.end(),
                                        [](const Job& a, const Job& b) { return a.refs.size() < b.refs.size(); });
            if (big->refs.size() <= small || frontier.size() + jobs.size() >= want) break;
            Job j = std::move(*big);
            frontier.erase(big);
            top.depth = std::max(top.depth, j.depth);
            std::vector<Ref> L, R;
            if (!SplitNode(j.refs, top, j.node, L, R)) continue;
            const uint32_t left = (uint32_t)top.nodes.size();
            top.nodes[j.node].a = left;
            top.nodes[j.node].count = 0;
            top.nodes.push_back(BinaryNode{});
            top.nodes.push_back(BinaryNode{});
            frontier.push_back({left, std::move(L), j.depth + 1});
            frontier.push_back({left + 1, std::move(R), j.depth + 1});
        }
        for (auto& f : frontier) jobs.push_back(std::move(f));
        std::vector<Out> outs(jobs.size());
        std::atomic<size_t> next{0};
        std::exception_ptr err;
        std::mutex err_mu;
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < threads; ++t)
            pool.emplace_back([&] {
                for (;;) {
                    const size_t k = next.fetch_add(1);
                    if (k >= jobs.size()) break;
                    try {
                        Build(std::move(jobs[k].refs), jobs[k].depth, outs[k]);
                    } catch (...) {
                        std::lock_guard<std::mutex> lk(err_mu);
                        if (!err) err = std::current_exception();
                    }
                }
            });
        for (auto& t : pool) t.join();
        if (err) std::rethrow_exception(err);
        // stitch: subtree roots replace their placeholders
        result.nodes = std::move(top.nodes);
        result.prims = std::move(top.prims);
        result.depth = top.depth;
        result.leaves = top.leaves;
        double sah = top.sah;
        for (size_t k = 0; k < jobs.size(); ++k) {
            Out& o = outs[k];
            const uint32_t node_base = (uint32_t)result.nodes.size() - 1;  // o.nodes[i] -> node_base + i (i >= 1)
            const uint32_t prim_base = (uint32_t)result.prims.size();
            auto fix = [&](BinaryNode n) {
                if (n.count)
                    n.a += prim_base;
                else
                    n.a += node_base;
                return n;
            };
            result.nodes[jobs[k].node] = fix(o.nodes[0]);
            for (size_t i = 1; i < o.nodes.size(); ++i) result.nodes.push_back(fix(o.nodes[i]));
            result.prims.insert(result.prims.end(), o.prims.begin(), o.prims.end());
            result.depth = std::max(result.depth, o.depth);
            result.leaves += o.leaves;
            sah += o.sah;
        }
        result.sah_cost = m_root_area > 0.0f ? sah / m_root_area : 0.0;
    }

private:
    // Decides leaf or split for `refs` at out.nodes[node]; fills the node box
    // (and leaf contents) and returns true with L / R when it splits.
    bool SplitNode(std::vector<Ref>& refs, Out& out, uint32_t node, std::vector<Ref>& L, std::vector<Ref>& R) {
        Box box, cb;
        for (const Ref& r : refs) {
            box.grow(r.box);
            const float c[3] = {r.centroid(0), r.centroid(1), r.centroid(2)};
            cb.grow_point(c);
        }
        BinaryNode& nd = out.nodes[node];
        for (int i = 0; i < 3; ++i) {
            nd.lo[i] = box.lo[i];
            nd.hi[i] = box.hi[i];
        }
        const uint32_t n = (uint32_t)refs.size();
        const double area = box.half_area();
        Split best = ObjectSplit(refs, cb);
        if (best.axis >= 0 && n > 1 && m_used.load(std::memory_order_relaxed) < m_budget) {
            // overlap of the object split's children decides whether to try spatial splits
            Box lb, rb;
            for (const Ref& r : refs) {
                int k = (int)((r.centroid(best.axis) - best.clo) * best.scale);
                k = std::min(std::max(k, 0), (int)m_p.bins - 1);
                ((uint32_t)k <= (uint32_t)best.bin ? lb : rb).grow(r.box);
            }
            const double overlap = lb.intersect(rb).half_area();
            if (overlap > m_p.spatial_alpha * m_root_area) {
                const Split sp = SpatialSplit(refs, box);
                if (sp.cost < best.cost) best = sp;
            }
        }
        const double split_cost = best.axis >= 0 ? (double)m_p.trav_cost + best.cost / area : DBL_MAX;
        if (n <= m_p.max_leaf && (best.axis < 0 || (double)n <= split_cost)) {
            MakeLeaf(refs, out, node, area);
            return false;
        }
        if (best.axis < 0) {
            // coincident centroids: median split by triangle index
            std::sort(refs.begin(), refs.end(), [](const Ref& a, const Ref& b) { return a.tri < b.tri; });
            L.assign(refs.begin(), refs.begin() + n / 2);
            R.assign(refs.begin() + n / 2, refs.end());
        } else if (!best.spatial) {
            for (const Ref& r : refs) {
                int k = (int)((r.centroid(best.axis) - best.clo) * best.scale);
                k = std::min(std::max(k, 0), (int)m_p.bins - 1);
                ((uint32_t)k <= (uint32_t)best.bin ? L : R).push_back(r);
            }
        } else {
            const int a = best.axis;
            const float pos = best.pos;
            uint64_t dup = 0;
            for (const Ref& r : refs) {
                if (r.box.hi[a] <= pos) {
                    L.push_back(r);
                } else if (r.box.lo[a] >= pos) {
                    R.push_back(r);
                } else {
                    const float* t = m_tri + 9 * (size_t)r.tri;
                    Ref l = r, rr = r;
                    l.box = ClipTriangle(t, a, r.box.lo[a], pos).intersect(r.box);
                    rr.box = ClipTriangle(t, a, pos, r.box.hi[a]).intersect(r.box);
                    if (l.box.empty() && rr.box.empty()) {
                        L.push_back(r);  // numerically empty on both sides: keep it whole
                        continue;
                    }
                    if (!l.box.empty()) L.push_back(l);
                    if (!rr.box.empty()) R.push_back(rr);
                    if (!l.box.empty() && !rr.box.empty()) dup++;
                }
            }
            m_used.fetch_add(dup, std::memory_order_relaxed);
            if (L.empty() || R.empty()) {  // degenerate plane: fall back to halves by index
                std::vector<Ref> all = std::move(L.empty() ? R : L);
                L.clear();
                R.clear();
                std::sort(all.begin(), all.end(), [](const Ref& x, const Ref& y) { return x.tri < y.tri; });
                const size_t h = all.size() / 2;
                L.assign(all.begin(), all.begin() + h);
                R.assign(all.begin() + h, all.end());
                if (L.empty()) {
                    MakeLeaf(all, out, node, area);
                    return false;
                }
            }
        }
        out.sah += (double)m_p.trav_cost * area;
        return true;
    }

    void MakeLeaf(const std::vector<Ref>& refs, Out& out, uint32_t node, double area) {
        BinaryNode& nd = out.nodes[node];
        nd.a = (uint32_t)out.prims.size();
        nd.count = (uint32_t)refs.size();
        CHECK_CODE(nd.count <= 4, FND_ERR_INVALID_SCENE, "spatial-split leaf with %u references", nd.count);
        for (const Ref& r : refs) out.prims.push_back(r.tri);
        out.sah += (double)refs.size() * area;
        out.leaves++;
    }

    Split ObjectSplit(const std::vector<Ref>& refs, const Box& cb) const {
        Split best;
        const uint32_t bins = m_p.bins;
        std::vector<Box> bb(bins), rbox(bins);
        std::vector<uint32_t> cnt(bins), rcnt(bins);
        for (int ax = 0; ax < 3; ++ax) {
            const float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0f)) continue;
            const float scale = (float)bins / ext;
            std::fill(cnt.begin(), cnt.end(), 0u);
            std::fill(bb.begin(), bb.end(), Box());
            for (const Ref& r : refs) {
                int k = (int)((r.centroid(ax) - cb.lo[ax]) * scale);
                k = std::min(std::max(k, 0), (int)bins - 1);
                cnt[k]++;
                bb[k].grow(r.box);
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
                if (c == 0 || rcnt[k + 1] == 0) continue;
                const double cost = (double)acc.half_area() * c + (double)rbox[k + 1].half_area() * rcnt[k + 1];
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = ax;
                    best.bin = (int)k;
                    best.spatial = false;
                    best.scale = scale;
                    best.clo = cb.lo[ax];
                }
            }
        }
        return best;
    }

    Split SpatialSplit(const std::vector<Ref>& refs, const Box& box) const {
        Split best;
        const uint32_t bins = m_p.bins;
        std::vector<Box> bb(bins), rbox(bins);
        std::vector<uint32_t> enter(bins), exit_(bins), rcnt(bins);
        for (int ax = 0; ax < 3; ++ax) {
            const float lo = box.lo[ax], ext = box.hi[ax] - box.lo[ax];
            if (!(ext > 0.0f)) continue;
            const float step = ext / (float)bins;
            std::fill(bb.begin(), bb.end(), Box());
            std::fill(enter.begin(), enter.end(), 0u);
            std::fill(exit_.begin(), exit_.end(), 0u);
            for (const Ref& r : refs) {
                int b0 = (int)((r.box.lo[ax] - lo) / step), b1 = (int)((r.box.hi[ax] - lo) / step);
                b0 = std::min(std::max(b0, 0), (int)bins - 1);
                b1 = std::min(std::max(b1, b0), (int)bins - 1);
                enter[b0]++;
                exit_[b1]++;
                const float* t = m_tri + 9 * (size_t)r.tri;
                for (int b = b0; b <= b1; ++b) {
                    const float slo = lo + step * (float)b, shi = (b == (int)bins - 1) ? box.hi[ax] : slo + step;
                    const Box cbx = (b0 == b1) ? r.box : ClipTriangle(t, ax, slo, shi).intersect(r.box);
                    if (!cbx.empty()) bb[b].grow(cbx);
                }
            }
            Box acc;
            uint32_t c = 0;
            for (int k = (int)bins - 1; k >= 1; --k) {
                acc.grow(bb[k]);
                c += exit_[k];
                rbox[k] = acc;
                rcnt[k] = c;
            }
            acc = Box();
            c = 0;
            for (uint32_t k = 0; k + 1 < bins; ++k) {
                acc.grow(bb[k]);
                c += enter[k];
                if (c == 0 || rcnt[k + 1] == 0) continue;
                const double cost = (double)acc.half_area() * c + (double)rbox[k + 1].half_area() * rcnt[k + 1];
                if (cost < best.cost) {
                    best.cost = cost;
                    best.axis = ax;
                    best.bin = (int)k;
                    best.spatial = true;
                    best.pos = lo + step * (float)(k + 1);
                }
            }
        }
        return best;
    }

    const float* m_tri;
    uint32_t m_nt;
    BuildParams m_p;
    float m_root_area;
    uint64_t m_budget;
    std::atomic<uint64_t> m_used{0};
};

}  // namespace

void BuildBinarySbvh(const float* tri, uint32_t nt, const BuildParams& params, BinaryBvh& out) {
    CHECK(nt > 0);
    CHECK(params.bins >= 2 && params.bins <= 64);
    CHECK(params.max_leaf >= 1 && params.max_leaf <= 4);
    std::vector<Ref> refs(nt);
    Box root;
    for (uint32_t t = 0; t < nt; ++t) {
        refs[t].tri = t;
        refs[t].box.grow_point(tri + 9 * (size_t)t);
        refs[t].box.grow_point(tri + 9 * (size_t)t + 3);
        refs[t].box.grow_point(tri + 9 * (size_t)t + 6);
        root.grow(refs[t].box);
    }
    SbvhBuilder b(tri, nt, params, root.half_area());
    b.BuildParallel(std::move(refs), out);
}

}  // namespace RT
}  // namespace Foundation
