// collapse.cpp — binary BVH -> compressed 8-wide BVH (see collapse.hpp).
//
// Compressed wide nodes after Ylitie, Karras & Laine, "Efficient Incoherent
// Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017: 8 children
// per node, child boxes as 8-bit offsets on a power-of-two grid anchored at
// the node's lower corner, internal children stored contiguously, leaf
// triangles stored contiguously, children placed in slots by octant so a
// fixed per-ray slot order approximates front-to-back.
#include "collapse.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <atomic>
#include <exception>
#include <memory>
#include <mutex>
#include <thread>

#include "../core/core.hpp"

namespace Foundation {
namespace RT {

float SceneMargin(const float lo[3], const float hi[3]) {
    float s = 0.0f;
    for (int i = 0; i < 3; ++i) {
        s = std::max(s, std::fabs(lo[i]));
        s = std::max(s, std::fabs(hi[i]));
        s = std::max(s, hi[i] - lo[i]);
    }
    return s * (1.0f / 65536.0f);
}

namespace {

// A wide node waiting for its record: the binary node it is made of, its
// index in the breadth-first layout and its depth.
struct Item {
    uint32_t bnode;
    uint32_t wnode;
    uint32_t depth;
};

// Everything about one wide node that does not depend on where the
// breadth-first layout puts it: the record without child_base / tri_base,
// its internal children's binary nodes and its leaf triangles, both in slot
// order.
struct NodePlan {
    WideNode nd;
    uint32_t internal[kWidth];
    uint32_t prims[kWidth * kMaxLeafTris];
    uint8_t num_internal;
    uint8_t num_tris;
    uint8_t num_leaves;
};

// f(i) for i in [0, n) on up to `threads` threads, `chunk` indices at a
// time; the first exception is rethrown on the caller's thread.
template <class F>
void ParallelFor(size_t n, uint32_t threads, size_t chunk, const F& f) {
    if (threads <= 1 || n <= chunk) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::exception_ptr err;
    std::mutex err_mu;
    auto work = [&] {
        for (;;) {
            const size_t b = next.fetch_add(chunk);
            if (b >= n) return;
            try {
                for (size_t i = b; i < std::min(n, b + chunk); ++i) f(i);
            } catch (...) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (!err) err = std::current_exception();
                next.store(n);
                return;
            }
        }
    };
    std::vector<std::thread> pool;
    const uint32_t t = (uint32_t)std::min<size_t>(threads, (n + chunk - 1) / chunk);
    for (uint32_t k = 1; k < t; ++k) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    if (err) std::rethrow_exception(err);
}

float HalfArea(const BinaryNode& n) {
    const float dx = n.hi[0] - n.lo[0], dy = n.hi[1] - n.lo[1], dz = n.hi[2] - n.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// A child of a wide node: a binary subtree that becomes either an internal
// wide node or one leaf slot holding all of the subtree's triangles.
struct Kid {
    uint32_t bnode;
    bool leaf;
};

// SAH-optimal collapse (after Ylitie, Karras & Laine 2017): bottom-up over the
// binary tree, C(n, i) is the least cost of representing n's subtree by at most
// i roots (wide nodes or leaf slots of at most kMaxLeafTris triangles), with a
// wide node costing c_node x its half area and a leaf c_tri x half area x its
// triangles; a wide node's children are the best split of 8 roots between
// the two binary children.
class SahCollapse {
public:
    // Solves C(n, i) for every node reachable from the root: the subtrees
    // below a breadth-first top part in parallel, each in reverse pre-order,
    // then the top part in reverse breadth-first order, so every node's
    // children are solved before it.
    SahCollapse(const BinaryBvh& bin, double c_node, double c_tri, uint32_t threads, int width)
        : m_bin(bin), m_c_node(c_node), m_c_tri(c_tri), m_width(width) {
        const size_t n = bin.nodes.size();
        m_cost.assign(8 * n, 0.0f);
        m_choice.assign(8 * n, 0);
        m_node_j.assign(n, 0);
        m_as_leaf.assign(n, 0);
        m_tris.assign(n, 0);
        std::vector<uint32_t> top, frontier{0u}, grow;
        while (!frontier.empty() && frontier.size() < 8 * (size_t)threads) {
            grow.clear();
            for (uint32_t k : frontier) {
                top.push_back(k);
                if (!bin.nodes[k].count) {
                    CheckChildren(k);
                    grow.push_back(bin.nodes[k].a);
                    grow.push_back(bin.nodes[k].a + 1);
                }
            }
            frontier.swap(grow);
        }
        ParallelFor(frontier.size(), threads, 1, [&](size_t i) { SolveSubtree(frontier[i]); });
        for (size_t i = top.size(); i-- > 0;) Solve(top[i]);
    }

    // C(root, 1): the cost of the whole wide tree.
    float RootCost() const { return m_cost[0]; }

    // The children of a wide node made of binary node n.
    void NodeKids(uint32_t n, Kid* kids, int& nk) const {
        nk = 0;
        const BinaryNode& b = m_bin.nodes[n];
        if (b.count) {
            kids[nk++] = {n, true};
            return;
        }
        Gather(b.a, m_node_j[n], kids, nk);
        Gather(b.a + 1, m_width - m_node_j[n], kids, nk);
    }

private:
    void CheckChildren(uint32_t k) const {
        const uint32_t l = m_bin.nodes[k].a;
        CHECK_CODE(l > k && (size_t)l + 1 < m_bin.nodes.size(), FND_ERR_INVALID_SCENE,
                   "binary tree not in parent-before-child order");
    }

    void SolveSubtree(uint32_t root) {
        std::vector<uint32_t> order{root}, stack{root};
        while (!stack.empty()) {
            const uint32_t k = stack.back();
            stack.pop_back();
            if (m_bin.nodes[k].count) continue;
            CheckChildren(k);
            const uint32_t l = m_bin.nodes[k].a;
            for (uint32_t c : {l, l + 1}) {
                order.push_back(c);
                stack.push_back(c);
            }
        }
        for (size_t i = order.size(); i-- > 0;) Solve(order[i]);
    }

    // C(k, 1..8) from the children's costs
    void Solve(uint32_t k) {
        const BinaryNode& b = m_bin.nodes[k];
        const double area = (double)HalfArea(b);
        float* c = &m_cost[8 * (size_t)k];
        if (b.count) {
            m_tris[k] = b.count;
            for (int i = 0; i < 8; ++i) c[i] = (float)(area * m_c_tri * b.count);
            m_as_leaf[k] = 1;
            return;
        }
        const uint32_t l = b.a, r = b.a + 1;
        m_tris[k] = m_tris[l] + m_tris[r];
        const float* cl = &m_cost[8 * (size_t)l];
        const float* cr = &m_cost[8 * (size_t)r];
        float split[9];
        uint8_t split_j[9];
        for (int i = 2; i <= 8; ++i) {
            split[i] = FLT_MAX;
            split_j[i] = 1;
            for (int j = 1; j < i; ++j) {
                const float v = cl[j - 1] + cr[i - j - 1];
                if (v < split[i]) {
                    split[i] = v;
                    split_j[i] = (uint8_t)j;
                }
            }
        }
        // a wide node: its children are the best split of m_width roots
        const float node_cost = (float)(area * m_c_node) + split[m_width];
        m_node_j[k] = split_j[m_width];
        c[0] = node_cost;
        if (m_tris[k] <= (uint32_t)kMaxLeafTris) {
            const float leaf_cost = (float)(area * m_c_tri * m_tris[k]);
            if (leaf_cost <= node_cost) {
                c[0] = leaf_cost;
                m_as_leaf[k] = 1;
            }
        }
        for (int i = 2; i <= 8; ++i) {
            if (split[i] < c[i - 2]) {
                c[i - 1] = split[i];
                m_choice[8 * (size_t)k + i - 1] = split_j[i];
            } else {
                c[i - 1] = c[i - 2];
            }
        }
    }

    void Gather(uint32_t n, int k, Kid* kids, int& nk) const {
        const BinaryNode& b = m_bin.nodes[n];
        while (k >= 2 && !b.count && m_choice[8 * (size_t)n + k - 1] == 0) --k;
        if (k >= 2 && !b.count) {
            const int j = m_choice[8 * (size_t)n + k - 1];
            Gather(b.a, j, kids, nk);
            Gather(b.a + 1, k - j, kids, nk);
            return;
        }
        CHECK(nk < kWidth);
        kids[nk++] = {n, m_as_leaf[n] != 0};
    }

    const BinaryBvh& m_bin;
    const double m_c_node, m_c_tri;
    const int m_width;               // children per wide node
    std::vector<uint32_t> m_tris;    // triangles (leaf slots) under n
    std::vector<float> m_cost;       // [8 n + i - 1]: C(n, i)
    std::vector<uint8_t> m_choice;   // [8 n + i - 1], i >= 2: 0 = C(n, i - 1), else roots given to the left child
    std::vector<uint8_t> m_node_j;   // roots given to the left child when n is a wide node
    std::vector<uint8_t> m_as_leaf;  // C(n, 1) is a leaf slot
};

// The triangles (leaf slots) of binary subtree n, in leaf order.
void SubtreePrims(const BinaryBvh& bin, uint32_t n, uint32_t* out, uint32_t& cnt) {
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = n;
    while (sp) {
        const BinaryNode& b = bin.nodes[stack[--sp]];
        if (b.count) {
            for (uint32_t i = 0; i < b.count; ++i) {
                CHECK_CODE(cnt < (uint32_t)kMaxLeafTris, FND_ERR_INVALID_SCENE, "leaf larger than 4 triangles");
                out[cnt++] = bin.prims[b.a + i];
            }
        } else {
            CHECK(sp + 2 <= 64);
            stack[sp++] = b.a + 1;
            stack[sp++] = b.a;
        }
    }
}

// The wide node made of binary node `bnode`: its children (SAH-optimal or
// greedy), inflated child boxes, octant slots, quantised boxes and leaf
// triangles. Depends on nothing outside the subtree of `bnode`.
void PlanNode(const BinaryBvh& bin, const SahCollapse* sah, float margin, int width, uint32_t bnode,
              NodePlan& plan) {
    Kid kids[kWidth];
    int nk = 0;
    if (sah) {
        sah->NodeKids(bnode, kids, nk);
    } else {
        // gather up to `width` children by expanding the largest internal child
        nk = 1;
        kids[0] = {bnode, bin.nodes[bnode].count > 0};
        for (;;) {
            int pick = -1;
            float best = -1.0f;
            for (int k = 0; k < nk; ++k) {
                const BinaryNode& c = bin.nodes[kids[k].bnode];
                if (c.count) continue;
                const float a = HalfArea(c);
                if (a > best) {
                    best = a;
                    pick = k;
                }
            }
            if (pick < 0 || nk == width) break;
            const uint32_t l = bin.nodes[kids[pick].bnode].a;
            kids[pick] = {l, bin.nodes[l].count > 0};
            kids[nk++] = {l + 1, bin.nodes[l + 1].count > 0};
        }
    }
    // inflated child boxes and the node box
    float clo[kWidth][3], chi[kWidth][3], nlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, nhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int k = 0; k < nk; ++k) {
        const BinaryNode& c = bin.nodes[kids[k].bnode];
        for (int a = 0; a < 3; ++a) {
            clo[k][a] = c.lo[a] - margin;
            chi[k][a] = c.hi[a] + margin;
            // subtraction can round back to the uninflated value for
            // huge coordinates; step one ulp outward in that case
            if (!(clo[k][a] < c.lo[a])) clo[k][a] = std::nextafter(c.lo[a], -INFINITY);
            if (!(chi[k][a] > c.hi[a])) chi[k][a] = std::nextafter(c.hi[a], INFINITY);
            nlo[a] = std::min(nlo[a], clo[k][a]);
            nhi[a] = std::max(nhi[a], chi[k][a]);
        }
    }
    // octant slot assignment (greedy on the score table)
    int child_in_slot[kWidth];
    for (int s = 0; s < kWidth; ++s) child_in_slot[s] = -1;
    {
        float score[kWidth][kWidth];
        const float cx = 0.5f * (nlo[0] + nhi[0]), cy = 0.5f * (nlo[1] + nhi[1]), cz = 0.5f * (nlo[2] + nhi[2]);
        for (int k = 0; k < nk; ++k) {
            const float dx = 0.5f * (clo[k][0] + chi[k][0]) - cx;
            const float dy = 0.5f * (clo[k][1] + chi[k][1]) - cy;
            const float dz = 0.5f * (clo[k][2] + chi[k][2]) - cz;
            for (int s = 0; s < kWidth; ++s)
                score[k][s] = ((s & 1) ? dx : -dx) + ((s & 2) ? dy : -dy) + ((s & 4) ? dz : -dz);
        }
        bool used_k[kWidth] = {}, used_s[kWidth] = {};
        for (int round = 0; round < nk; ++round) {
            int bk = -1, bs = -1;
            float bv = -FLT_MAX;
            for (int k = 0; k < nk; ++k) {
                if (used_k[k]) continue;
                for (int s = 0; s < kWidth; ++s) {
                    if (used_s[s]) continue;
                    if (score[k][s] > bv || bk < 0) {
                        bv = score[k][s];
                        bk = k;
                        bs = s;
                    }
                }
            }
            used_k[bk] = used_s[bs] = true;
            child_in_slot[bs] = bk;
        }
    }
    // quantisation grid
    WideNode& nd = plan.nd;
    std::memset(&nd, 0, sizeof(nd));
    double step[3];
    for (int a = 0; a < 3; ++a) {
        nd.p[a] = nlo[a];
        const double ext = (double)nhi[a] - (double)nlo[a];
        int e = ext > 0.0 ? (int)std::ceil(std::log2(ext / 255.0)) : -100;
        while (std::ldexp(255.0, e) < ext) e++;
        while (e > -100 && std::ldexp(255.0, e - 1) >= ext) e--;
        CHECK_CODE(e >= -100 && e <= 100, FND_ERR_INVALID_SCENE, "scene extent out of the node format range");
        nd.e[a] = (uint8_t)(e + 127);
        step[a] = std::ldexp(1.0, e);
    }
    plan.num_internal = 0;
    plan.num_leaves = 0;
    uint32_t tri_off = 0;
    // slots in increasing order so internal children and leaf triangles are
    // laid out in slot order
    for (int s = 0; s < kWidth; ++s) {
        const int k = child_in_slot[s];
        if (k < 0) continue;
        for (int a = 0; a < 3; ++a) {
            const double p = nd.p[a];
            double ql = std::floor(((double)clo[k][a] - p) / step[a]);
            double qh = std::ceil(((double)chi[k][a] - p) / step[a]);
            ql = std::min(std::max(ql, 0.0), 255.0);
            qh = std::min(std::max(qh, 0.0), 255.0);
            while (ql > 0.0 && p + ql * step[a] > (double)clo[k][a]) ql -= 1.0;
            while (qh < 255.0 && p + qh * step[a] < (double)chi[k][a]) qh += 1.0;
            CHECK_CODE(p + ql * step[a] <= (double)clo[k][a] && p + qh * step[a] >= (double)chi[k][a],
                       FND_ERR_INVALID_SCENE, "child box quantisation failed");
            nd.qlo[a][s] = (uint8_t)ql;
            nd.qhi[a][s] = (uint8_t)qh;
        }
        if (kids[k].leaf) {
            uint32_t lp[kMaxLeafTris], lc = 0;
            SubtreePrims(bin, kids[k].bnode, lp, lc);
            CHECK_CODE(lc >= 1, FND_ERR_INVALID_SCENE, "empty leaf");
            CHECK_CODE(tri_off + lc <= 32, FND_ERR_INVALID_SCENE, "more than 32 triangles under one wide node");
            nd.meta[s] = (uint8_t)(kMetaLeafFlag | ((lc - 1) << 5) | tri_off);
            for (uint32_t i = 0; i < lc; ++i) plan.prims[tri_off + i] = lp[i];
            tri_off += lc;
            plan.num_leaves++;
        } else {
            nd.imask |= (uint8_t)(1u << s);
            nd.meta[s] = kMetaInternal;
            plan.internal[plan.num_internal++] = kids[k].bnode;
        }
    }
    plan.num_tris = (uint8_t)tri_off;
}

}  // namespace

// Breadth-first layout, one level at a time: the nodes of a level are planned
// in parallel, a pass in breadth-first order gives each its child and
// triangle bases (children in the order the parents and their slots come),
// and the records and triangle planes are then written in parallel. The
// result is the same as visiting the nodes one by one from a FIFO queue.
void CollapseToWide(const BinaryBvh& bin, const float* tri, uint32_t nt, WideBvh& out, float margin_scale,
                    const CollapseOptions& opt) {
    CHECK(!bin.nodes.empty());
    const uint32_t threads =
        opt.threads ? opt.threads : std::max(1u, (uint32_t)std::thread::hardware_concurrency());
    std::unique_ptr<SahCollapse> sah;
    CHECK_CODE(opt.width >= 2 && opt.width <= (uint32_t)kWidth, FND_ERR_INVALID_ARG, "node width %u not in 2..%d",
               opt.width, kWidth);
    if (opt.sah) sah = std::make_unique<SahCollapse>(bin, opt.c_node, opt.c_tri, threads, (int)opt.width);
    const BinaryNode& root = bin.nodes[0];
    for (int i = 0; i < 3; ++i) {
        out.lo[i] = root.lo[i];
        out.hi[i] = root.hi[i];
    }
    const float margin = SceneMargin(root.lo, root.hi) * margin_scale;
    if (sah) {
        const double ra = (double)(root.hi[0] - root.lo[0]) * (root.hi[1] - root.lo[1]) +
                          (double)(root.hi[1] - root.lo[1]) * (root.hi[2] - root.lo[2]) +
                          (double)(root.hi[2] - root.lo[2]) * (root.hi[0] - root.lo[0]);
        LOG_RUNTIME(FndRt, INFO, "SAH-optimal collapse: wide-tree cost %.4f (root half-area normalised)",
                    ra > 0.0 ? sah->RootCost() / ra : 0.0);
    }
    out.margin = margin;
    out.nodes.assign(1, WideNode{});
    const size_t nrefs = bin.prims.size();  // == nt unless spatial splits duplicated references
    out.v0 = PlaneVector(4 * nrefs);  // every element is written below
    out.v1 = PlaneVector(4 * nrefs);
    out.v2 = PlaneVector(4 * nrefs);
    out.depth = 0;
    out.leaves = 0;
    uint64_t next_tri = 0;

    constexpr size_t kLevelChunk = 256;  // wide nodes per task; smaller levels run on this thread
    std::vector<Item> level{{0u, 0u, 1u}}, next;
    std::vector<NodePlan> plans;
    while (!level.empty()) {
        plans.resize(level.size());
        ParallelFor(level.size(), threads, kLevelChunk,
                    [&](size_t i) { PlanNode(bin, sah.get(), margin, (int)opt.width, level[i].bnode, plans[i]); });
        next.clear();
        uint64_t child = out.nodes.size();
        for (size_t i = 0; i < level.size(); ++i) {
            NodePlan& p = plans[i];
            out.depth = std::max(out.depth, level[i].depth);
            CHECK_CODE(child + p.num_internal <= UINT32_MAX && next_tri + p.num_tris <= nrefs, FND_ERR_INVALID_SCENE,
                       "collapse layout overflow");
            p.nd.child_base = (uint32_t)child;
            p.nd.tri_base = (uint32_t)next_tri;
            for (int j = 0; j < p.num_internal; ++j)
                next.push_back({p.internal[j], (uint32_t)(child + j), level[i].depth + 1});
            child += p.num_internal;
            next_tri += p.num_tris;
            out.leaves += p.num_leaves;
        }
        out.nodes.resize(child);
        ParallelFor(level.size(), threads, kLevelChunk, [&](size_t i) {
            const NodePlan& p = plans[i];
            out.nodes[level[i].wnode] = p.nd;
            for (uint32_t k = 0; k < p.num_tris; ++k) {
                const uint32_t id = p.prims[k];
                const size_t d = 4 * ((size_t)p.nd.tri_base + k);
                const float* v = tri + 9 * (size_t)id;
                out.v0[d + 0] = v[0];
                out.v0[d + 1] = v[1];
                out.v0[d + 2] = v[2];
                std::memcpy(&out.v0[d + 3], &id, 4);
                out.v1[d + 0] = v[3];
                out.v1[d + 1] = v[4];
                out.v1[d + 2] = v[5];
                out.v1[d + 3] = 0.0f;
                out.v2[d + 0] = v[6];
                out.v2[d + 1] = v[7];
                out.v2[d + 2] = v[8];
                out.v2[d + 3] = 0.0f;
            }
        });
        level.swap(next);
    }
    CHECK_CODE(next_tri == nrefs, FND_ERR_INVALID_SCENE, "collapse lost references (%llu of %zu)",
               (unsigned long long)next_tri, nrefs);
    (void)nt;
}

}  // namespace RT
}  // namespace Foundation
