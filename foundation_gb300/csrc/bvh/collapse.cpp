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
#include <deque>
#include <memory>

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

struct Item {
    uint32_t bnode;
    uint32_t wnode;
    uint32_t depth;
};

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
    SahCollapse(const BinaryBvh& bin, double c_node, double c_tri) : m_bin(bin) {
        const size_t n = bin.nodes.size();
        m_cost.assign(8 * n, 0.0f);
        m_choice.assign(8 * n, 0);
        m_node_j.assign(n, 0);
        m_as_leaf.assign(n, 0);
        std::vector<uint32_t> tris(n, 0);
        for (size_t k = n; k-- > 0;) {
            const BinaryNode& b = bin.nodes[k];
            const double area = (double)HalfArea(b);
            float* c = &m_cost[8 * k];
            if (b.count) {
                tris[k] = b.count;
                for (int i = 0; i < 8; ++i) c[i] = (float)(area * c_tri * b.count);
                m_as_leaf[k] = 1;
                continue;
            }
            const uint32_t l = b.a, r = b.a + 1;
            CHECK_CODE(l > k && r < n, FND_ERR_INVALID_SCENE, "binary tree not in parent-before-child order");
            tris[k] = tris[l] + tris[r];
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
            const float node_cost = (float)(area * c_node) + split[8];
            m_node_j[k] = split_j[8];
            c[0] = node_cost;
            if (tris[k] <= (uint32_t)kMaxLeafTris) {
                const float leaf_cost = (float)(area * c_tri * tris[k]);
                if (leaf_cost <= node_cost) {
                    c[0] = leaf_cost;
                    m_as_leaf[k] = 1;
                }
            }
            for (int i = 2; i <= 8; ++i) {
                if (split[i] < c[i - 2]) {
                    c[i - 1] = split[i];
                    m_choice[8 * k + i - 1] = split_j[i];
                } else {
                    c[i - 1] = c[i - 2];
                }
            }
        }
    }

    // The children of a wide node made of binary node n.
    void NodeKids(uint32_t n, Kid* kids, int& nk) const {
        nk = 0;
        const BinaryNode& b = m_bin.nodes[n];
        if (b.count) {
            kids[nk++] = {n, true};
            return;
        }
        Gather(b.a, m_node_j[n], kids, nk);
        Gather(b.a + 1, 8 - m_node_j[n], kids, nk);
    }

private:
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

}  // namespace

void CollapseToWide(const BinaryBvh& bin, const float* tri, uint32_t nt, WideBvh& out, float margin_scale,
                    const CollapseOptions& opt) {
    CHECK(!bin.nodes.empty());
    std::unique_ptr<SahCollapse> sah;
    if (opt.sah) sah = std::make_unique<SahCollapse>(bin, opt.c_node, opt.c_tri);
    const BinaryNode& root = bin.nodes[0];
    for (int i = 0; i < 3; ++i) {
        out.lo[i] = root.lo[i];
        out.hi[i] = root.hi[i];
    }
    const float margin = SceneMargin(root.lo, root.hi) * margin_scale;
    out.margin = margin;
    out.nodes.clear();
    out.nodes.reserve(bin.nodes.size() / 4 + 1);
    const size_t nrefs = bin.prims.size();  // == nt unless spatial splits duplicated references
    out.v0.assign(4 * nrefs, 0.0f);
    out.v1.assign(4 * nrefs, 0.0f);
    out.v2.assign(4 * nrefs, 0.0f);
    out.depth = 0;
    out.leaves = 0;
    uint32_t next_tri = 0;

    out.nodes.push_back(WideNode{});
    std::deque<Item> queue{{0u, 0u, 1u}};
    while (!queue.empty()) {
        const Item it = queue.front();
        queue.pop_front();
        out.depth = std::max(out.depth, it.depth);
        Kid kids[kWidth];
        int nk = 0;
        if (sah) {
            sah->NodeKids(it.bnode, kids, nk);
        } else {
            // gather up to 8 children by expanding the largest internal child
            nk = 1;
            kids[0] = {it.bnode, bin.nodes[it.bnode].count > 0};
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
                if (pick < 0 || nk == kWidth) break;
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
        int slot_of[kWidth];
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
                slot_of[bk] = bs;
                child_in_slot[bs] = bk;
            }
        }
        // quantisation grid
        WideNode nd;
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
        nd.child_base = (uint32_t)out.nodes.size();
        nd.tri_base = next_tri;
        uint32_t tri_off = 0;
        // slots in increasing order so internal children and leaf triangles
        // are laid out in slot order
        for (int s = 0; s < kWidth; ++s) {
            const int k = child_in_slot[s];
            if (k < 0) continue;
            const BinaryNode& c = bin.nodes[kids[k].bnode];
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
                nd.meta[s] = (uint8_t)(kMetaLeafFlag | ((lc - 1) << 5) | tri_off);
                for (uint32_t i = 0; i < lc; ++i) {
                    const uint32_t p = lp[i];
                    const size_t d = 4 * (size_t)(next_tri + tri_off + i);
                    const float* v = tri + 9 * (size_t)p;
                    uint32_t pid = p;
                    out.v0[d + 0] = v[0];
                    out.v0[d + 1] = v[1];
                    out.v0[d + 2] = v[2];
                    std::memcpy(&out.v0[d + 3], &pid, 4);
                    out.v1[d + 0] = v[3];
                    out.v1[d + 1] = v[4];
                    out.v1[d + 2] = v[5];
                    out.v2[d + 0] = v[6];
                    out.v2[d + 1] = v[7];
                    out.v2[d + 2] = v[8];
                }
                tri_off += lc;
                out.leaves++;
            } else {
                nd.imask |= (uint8_t)(1u << s);
                nd.meta[s] = kMetaInternal;
                const uint32_t w = (uint32_t)out.nodes.size();
                out.nodes.push_back(WideNode{});
                queue.push_back({kids[k].bnode, w, it.depth + 1});
            }
        }
        CHECK_CODE(tri_off <= 32, FND_ERR_INVALID_SCENE, "more than 32 triangles under one wide node");
        next_tri += tri_off;
        out.nodes[it.wnode] = nd;
    }
    CHECK_CODE(next_tri == nrefs, FND_ERR_INVALID_SCENE, "collapse lost references (%u of %zu)", next_tri, nrefs);
    (void)nt;
}

}  // namespace RT
}  // namespace Foundation
