// bvh_build.cpp — host build of the compressed 8-wide BVH.
//
// Replaces the driver-side BLAS build the reference requests through
// AccelerationStructure (bisemutum/src/graphics/accel.cpp:11-159,
// graphics_manager.cpp:616-654).  Steps:
//   1. binary BVH by binned SAH (Wald 2007, "On fast construction of SAH-based
//      bounding volume hierarchies"): 32 bins per axis, leaves of <= 3
//      triangles, subtrees built on parallel threads;
//   2. collapse to 8 children per node by repeatedly opening the child with
//      the largest surface area;
//   3. assign children to slots by octant (Ylitie et al. 2017) so that the
//      traversal's bit order visits near children first;
//   4. quantise child boxes outward to 8 bits per plane in the node's frame.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace bsm {
namespace {

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void grow(const float p[3]) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    double area() const {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = std::max(0.0, (double)hi[k] - (double)lo[k]);
        return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
    bool valid() const { return lo[0] <= hi[0]; }
};

struct BNode {
    Box box;
    uint32_t left = 0, right = 0;   // children (internal)
    uint32_t first = 0, count = 0;  // primitive range in the reference array
    bool leaf = false;
};

struct Builder {
    const std::vector<Box>& tri_box;
    const std::vector<float>& cen;  // 3 per triangle
    std::vector<uint32_t>& refs;
    std::vector<BNode>& nodes;
    std::atomic<uint32_t> node_count{0};
    std::atomic<int> threads_free{0};
    uint32_t bins = 0;       // set by the caller before build()
    uint32_t max_leaf = 0;

    uint32_t alloc() { return node_count.fetch_add(1); }

    void build(uint32_t ni, uint32_t begin, uint32_t end) {
        BNode& n = nodes[ni];
        Box bb, cb;
        for (uint32_t i = begin; i < end; ++i) {
            uint32_t r = refs[i];
            bb.grow(tri_box[r]);
            cb.grow(&cen[3 * (size_t)r]);
        }
        n.box = bb;
        n.first = begin;
        n.count = end - begin;
        uint32_t cnt = end - begin;
        if (cnt <= 1) { n.leaf = true; return; }

        // binned SAH over the three axes
        double best_cost = INFINITY;
        int best_axis = -1;
        uint32_t best_split = 0;
        const uint32_t B = bins;
        std::vector<Box> bin_box(B);
        std::vector<uint32_t> bin_cnt(B);
        std::vector<double> right_area(B);
        std::vector<uint32_t> right_cnt(B);
        for (int axis = 0; axis < 3; ++axis) {
            float ext = cb.hi[axis] - cb.lo[axis];
            if (!(ext > 0.0f)) continue;
            double scale = (double)B / (double)ext;
            std::fill(bin_box.begin(), bin_box.end(), Box());
            std::fill(bin_cnt.begin(), bin_cnt.end(), 0u);
            for (uint32_t i = begin; i < end; ++i) {
                uint32_t r = refs[i];
                int b = (int)(((double)cen[3 * (size_t)r + axis] - cb.lo[axis]) * scale);
                b = std::min(std::max(b, 0), (int)B - 1);
                bin_box[b].grow(tri_box[r]);
                bin_cnt[b]++;
            }
            Box acc;
            uint32_t c = 0;
            for (int b = (int)B - 1; b > 0; --b) {
                acc.grow(bin_box[b]);
                c += bin_cnt[b];
                right_area[b] = acc.valid() ? acc.area() : 0.0;
                right_cnt[b] = c;
            }
            acc = Box();
            c = 0;
            for (uint32_t b = 1; b < B; ++b) {
                acc.grow(bin_box[b - 1]);
                c += bin_cnt[b - 1];
                if (c == 0 || right_cnt[b] == 0) continue;
                double cost = acc.area() * c + right_area[b] * right_cnt[b];
                if (cost < best_cost) { best_cost = cost; best_axis = axis; best_split = b; }
            }
        }
        double parent_area = bb.area();
        double leaf_cost = (double)cnt;
        double split_cost = parent_area > 0.0 ? 1.0 + best_cost / parent_area : INFINITY;
        uint32_t mid;
        if (best_axis < 0) {
            if (cnt <= max_leaf) { n.leaf = true; return; }
            mid = begin + cnt / 2;  // all centroids coincide: split by index
        } else {
            if (cnt <= max_leaf && leaf_cost <= split_cost) { n.leaf = true; return; }
            double scale = (double)B / (double)(cb.hi[best_axis] - cb.lo[best_axis]);
            auto it = std::partition(refs.begin() + begin, refs.begin() + end, [&](uint32_t r) {
                int b = (int)(((double)cen[3 * (size_t)r + best_axis] - cb.lo[best_axis]) * scale);
                b = std::min(std::max(b, 0), (int)B - 1);
                return (uint32_t)b < best_split;
            });
            mid = (uint32_t)(it - refs.begin());
            if (mid == begin || mid == end) mid = begin + cnt / 2;
        }
        uint32_t l = alloc(), r = alloc();
        n.left = l;
        n.right = r;
        n.leaf = false;
        uint32_t lcnt = mid - begin, rcnt = end - mid;
        if (lcnt + rcnt > 65536 && threads_free.fetch_sub(1) > 0) {
            std::thread t([this, l, begin, mid] { build(l, begin, mid); });
            build(r, mid, end);
            t.join();
            threads_free.fetch_add(1);
        } else {
            if (lcnt + rcnt > 65536) threads_free.fetch_add(1);
            build(l, begin, mid);
            build(r, mid, end);
        }
    }
};

double sah_cost(const std::vector<BNode>& nodes, uint32_t root) {
    double ra = nodes[root].box.area();
    if (!(ra > 0.0)) return 0.0;
    double c = 0.0;
    std::vector<uint32_t> st{root};
    while (!st.empty()) {
        uint32_t i = st.back();
        st.pop_back();
        const BNode& n = nodes[i];
        if (n.leaf) c += n.box.area() / ra * n.count;
        else { c += n.box.area() / ra; st.push_back(n.left); st.push_back(n.right); }
    }
    return c;
}

// SAH-optimal collapse of a binary BVH into an 8-wide one (Ylitie, Karras,
// Laine 2017, section 3.1): cost(n, i) is the least SAH cost of representing
// n's subtree as at most i child slots of a wide node,
//   cost(n, 1) = min(leaf(n), internal(n)),
//   cost(n, i) = min(cost(n, i - 1), dist(n, i))               for i > 1,
//   dist(n, j) = min over k of cost(left, k) + cost(right, j - k),
//   internal(n) = area(n) * kNodeCost + dist(n, 8),
//   leaf(n) = area(n) * count(n) * kTriCost   (count <= max_leaf).
// The decisions are kept to expand each wide node's children afterwards.
struct Collapse {
    static constexpr double kNodeCost = 1.0;
    double kTriCost = 1.0;                    // a triangle test against an 8-child node test (measured optimum
                                              // 0.7-1.4 on the 1.48 M-triangle terrain)
    static constexpr uint8_t kLeaf = 0xff, kInner = 0xfe, kSame = 0xfd;
    std::vector<double> cost;                 // 8 per binary node
    std::vector<uint8_t> dec;                 // 8 per binary node: kLeaf / kInner (slot 0), kSame or k (left share)
    std::vector<uint8_t> inner_split;         // k of dist(n, 8) for wide nodes

    void run(const std::vector<BNode>& nodes, uint32_t max_leaf) {
        const size_t n = nodes.size();
        cost.assign(8 * n, INFINITY);
        dec.assign(8 * n, kSame);
        inner_split.assign(n, 4);
        // children are allocated after their parent: reverse index order is a post-order
        for (size_t x = n; x-- > 0;) {
            const BNode& b = nodes[x];
            double a = b.box.area();
            double leaf = b.count <= max_leaf ? a * b.count * kTriCost : INFINITY;
            double* c = &cost[8 * x];
            uint8_t* d = &dec[8 * x];
            if (b.leaf) {
                for (int i = 0; i < 8; ++i) { c[i] = leaf; d[i] = i == 0 ? kLeaf : kSame; }
                continue;
            }
            const double* cl = &cost[8 * (size_t)b.left];
            const double* cr = &cost[8 * (size_t)b.right];
            double dist[9];
            uint8_t arg[9];
            for (int j = 2; j <= 8; ++j) {
                dist[j] = INFINITY;
                arg[j] = 1;
                for (int k = 1; k < j; ++k) {
                    double v = cl[k - 1] + cr[j - k - 1];
                    if (v < dist[j]) { dist[j] = v; arg[j] = (uint8_t)k; }
                }
            }
            double inner = a * kNodeCost + dist[8];
            inner_split[x] = arg[8];
            if (leaf <= inner) { c[0] = leaf; d[0] = kLeaf; }
            else { c[0] = inner; d[0] = kInner; }
            for (int i = 2; i <= 8; ++i) {
                if (c[i - 2] <= dist[i]) { c[i - 1] = c[i - 2]; d[i - 1] = kSame; }
                else { c[i - 1] = dist[i]; d[i - 1] = arg[i]; }
            }
        }
    }
    // the binary nodes that fill up to i slots for subtree x
    void gather(const std::vector<BNode>& nodes, uint32_t x, int i, std::vector<uint32_t>& out) const {
        while (i > 1 && dec[8 * (size_t)x + i - 1] == kSame) --i;
        if (i == 1) { out.push_back(x); return; }
        int k = dec[8 * (size_t)x + i - 1];
        gather(nodes, nodes[x].left, k, out);
        gather(nodes, nodes[x].right, i - k, out);
    }
    bool is_leaf(uint32_t x) const { return dec[8 * (size_t)x] == kLeaf; }
};

// smallest e with 253 * 2^e >= extent (two steps of margin for the outward
// padding); returns the biased exponent byte
int quant_exponent(float extent) {
    double ext = std::max((double)extent, 1e-30);
    int e;
    std::frexp(ext / 253.0, &e);
    while (std::ldexp(253.0, e - 1) >= ext) --e;
    while (std::ldexp(253.0, e) < ext) ++e;
    int biased = e + 127;
    return std::min(std::max(biased, 1), 254);
}

}  // namespace

bool build_cwbvh(const float* positions, const uint32_t* indices, uint32_t num_tris, const uint32_t* material_ids,
                 const bsm_bvh_opts* opts_in, BvhBuildResult& out, std::string& err) {
    auto t0 = std::chrono::steady_clock::now();
    if (num_tris == 0) { err = "scene has no triangles"; return false; }
    // node and triangle bases share their top bit with the traversal's triangle-group flag
    if (num_tris >= kTriGroupFlag) { err = "more than 2^31 - 1 triangles in one BVH"; return false; }
    bsm_bvh_opts opts{};
    if (opts_in) opts = *opts_in;
    uint32_t bins = opts.sah_bins ? std::min(std::max(opts.sah_bins, 4u), 256u) : 32u;
    uint32_t max_leaf = opts.max_leaf_tris ? std::min(opts.max_leaf_tris, kMaxLeafTris) : kMaxLeafTris;
    const bool optimal = opts.collapse == BSM_COLLAPSE_SAH_OPTIMAL;
    uint32_t threads = opts.num_threads ? opts.num_threads : std::max(1u, std::thread::hardware_concurrency());

    auto vtx = [&](uint32_t t, int c, float p[3]) {
        size_t vi = indices ? indices[3 * (size_t)t + c] : 3 * (size_t)t + c;
        p[0] = positions[3 * vi]; p[1] = positions[3 * vi + 1]; p[2] = positions[3 * vi + 2];
    };

    std::vector<Box> tri_box(num_tris);
    std::vector<float> cen(3 * (size_t)num_tris);
    for (uint32_t t = 0; t < num_tris; ++t) {
        float p[3];
        Box b;
        for (int c = 0; c < 3; ++c) { vtx(t, c, p); b.grow(p); }
        for (int k = 0; k < 3; ++k) {
            if (!std::isfinite(b.lo[k]) || !std::isfinite(b.hi[k])) { err = "non-finite vertex position"; return false; }
            cen[3 * (size_t)t + k] = 0.5f * (b.lo[k] + b.hi[k]);
        }
        tri_box[t] = b;
    }
    std::vector<uint32_t> refs(num_tris);
    for (uint32_t i = 0; i < num_tris; ++i) refs[i] = i;
    std::vector<BNode> nodes(2 * (size_t)num_tris);
    Builder bld{tri_box, cen, refs, nodes};
    bld.bins = bins;
    bld.max_leaf = optimal ? 1u : max_leaf;  // the collapse chooses the leaves itself
    bld.threads_free = (int)threads - 1;
    uint32_t root = bld.alloc();
    bld.build(root, 0, num_tris);
    nodes.resize(bld.node_count.load());
    out.sah_cost = sah_cost(nodes, root);
    Collapse dp;
    if (opts.tri_cost > 0.0f) dp.kTriCost = opts.tri_cost;
    if (optimal) dp.run(nodes, max_leaf);
    // a binary node becomes one leaf slot
    auto as_leaf_node = [&](uint32_t x) {
        return optimal ? dp.is_leaf(x) : (nodes[x].leaf || nodes[x].count <= max_leaf);
    };

    // subtree triangle counts (count is set for every node by build())
    // collapse into 8-wide nodes, breadth first
    out.nodes.clear();
    out.tris.clear();
    out.nodes.reserve(num_tris / 3 + 16);
    out.tris.reserve(num_tris);
    struct Item { uint32_t bnode; uint32_t wnode; uint32_t depth; };
    std::vector<Item> queue;
    out.nodes.emplace_back();
    queue.push_back({root, 0, 1});
    uint32_t max_depth = 1;
    auto emit_leaf_tris = [&](uint32_t bi) {
        const BNode& n = nodes[bi];
        for (uint32_t i = 0; i < n.count; ++i) {
            uint32_t t = refs[n.first + i];
            CwTri ct{};
            float p[3];
            vtx(t, 0, p); ct.v0x = p[0]; ct.v0y = p[1]; ct.v0z = p[2];
            vtx(t, 1, p); ct.v1x = p[0]; ct.v1y = p[1]; ct.v1z = p[2];
            vtx(t, 2, p); ct.v2x = p[0]; ct.v2y = p[1]; ct.v2z = p[2];
            ct.prim = t;
            ct.material = material_ids ? material_ids[t] : 0u;
            ct.pad = 0;
            out.tris.push_back(ct);
        }
    };
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        Item it = queue[qi];
        max_depth = std::max(max_depth, it.depth);
        // gather up to 8 children
        std::vector<uint32_t> ch;
        const BNode& bn = nodes[it.bnode];
        if (as_leaf_node(it.bnode)) {
            ch.push_back(it.bnode);  // root that is a single leaf
        } else if (optimal) {
            dp.gather(nodes, bn.left, dp.inner_split[it.bnode], ch);
            dp.gather(nodes, bn.right, 8 - dp.inner_split[it.bnode], ch);
        } else {
            ch.push_back(bn.left);
            ch.push_back(bn.right);
        }
        while (!optimal && ch.size() < 8) {
            int best = -1;
            double best_area = -1.0;
            for (size_t i = 0; i < ch.size(); ++i) {
                const BNode& c = nodes[ch[i]];
                if (c.leaf || c.count <= max_leaf) continue;
                double a = c.box.area();
                if (a > best_area) { best_area = a; best = (int)i; }
            }
            if (best < 0) break;
            uint32_t open = ch[best];
            ch[best] = nodes[open].left;
            ch.push_back(nodes[open].right);
        }
        // node box and octant slot assignment
        Box nb;
        for (uint32_t c : ch) nb.grow(nodes[c].box);
        float ctr[3];
        for (int k = 0; k < 3; ++k) ctr[k] = 0.5f * (nb.lo[k] + nb.hi[k]);
        int slot_of[8];
        bool slot_used[8] = {false};
        bool child_done[8] = {false};
        for (size_t i = 0; i < ch.size(); ++i) slot_of[i] = -1;
        for (size_t round = 0; round < ch.size(); ++round) {
            double best = -INFINITY;
            int bi = -1, bs = -1;
            for (size_t i = 0; i < ch.size(); ++i) {
                if (child_done[i]) continue;
                const Box& b = nodes[ch[i]].box;
                double d[3];
                for (int k = 0; k < 3; ++k) d[k] = 0.5 * ((double)b.lo[k] + b.hi[k]) - ctr[k];
                for (int s = 0; s < 8; ++s) {
                    if (slot_used[s]) continue;
                    double cost = ((s & 1) ? d[0] : -d[0]) + ((s & 2) ? d[1] : -d[1]) + ((s & 4) ? d[2] : -d[2]);
                    if (cost > best) { best = cost; bi = (int)i; bs = s; }
                }
            }
            slot_of[bi] = bs;
            slot_used[bs] = true;
            child_done[bi] = true;
        }
        int child_at[8];
        for (int s = 0; s < 8; ++s) child_at[s] = -1;
        for (size_t i = 0; i < ch.size(); ++i) child_at[slot_of[i]] = (int)i;

        CwNode node;
        std::memset(&node, 0, sizeof(node));
        // quantisation frame: origin one step below the node box, so every
        // child box can be padded outward by one step on every side
        int e[3];
        float org_f[3];
        for (int k = 0; k < 3; ++k) {
            e[k] = quant_exponent(nb.hi[k] - nb.lo[k]);
            double step = std::ldexp(1.0, e[k] - 127);
            float o = (float)((double)nb.lo[k] - step);
            while ((double)o > (double)nb.lo[k] - step) o = std::nextafter(o, -INFINITY);
            org_f[k] = o;
        }
        node.px = org_f[0]; node.py = org_f[1]; node.pz = org_f[2];
        node.ex = (uint8_t)e[0]; node.ey = (uint8_t)e[1]; node.ez = (uint8_t)e[2];
        node.child_base = (uint32_t)out.nodes.size();
        node.tri_base = (uint32_t)out.tris.size();
        uint32_t tri_off = 0;
        std::vector<uint32_t> internal_children;
        for (int s = 0; s < 8; ++s) {
            if (child_at[s] < 0) continue;
            uint32_t ci = ch[child_at[s]];
            const BNode& c = nodes[ci];
            // outward quantisation, checked in double against the float box
            uint8_t* qlo[3] = {node.qlo_x, node.qlo_y, node.qlo_z};
            uint8_t* qhi[3] = {node.qhi_x, node.qhi_y, node.qhi_z};
            const float org[3] = {node.px, node.py, node.pz};
            for (int k = 0; k < 3; ++k) {
                double sc = std::ldexp(1.0, e[k] - 127);
                double lo = std::floor(((double)c.box.lo[k] - org[k]) / sc) - 1.0;
                double hi = std::ceil(((double)c.box.hi[k] - org[k]) / sc) + 1.0;
                lo = std::min(std::max(lo, 0.0), 255.0);
                hi = std::min(std::max(hi, 0.0), 255.0);
                while (lo > 0.0 && (double)org[k] + lo * sc > (double)c.box.lo[k]) lo -= 1.0;
                while (hi < 255.0 && (double)org[k] + hi * sc < (double)c.box.hi[k]) hi += 1.0;
                qlo[k][s] = (uint8_t)lo;
                qhi[k][s] = (uint8_t)hi;
            }
            bool as_leaf = as_leaf_node(ci);
            if (as_leaf) {
                uint32_t cnt = c.count;
                if (cnt == 0 || cnt > kMaxLeafTris) { err = "internal error: leaf size"; return false; }
                // gather the subtree's triangles (a small internal subtree becomes one leaf)
                std::vector<uint32_t> st{ci};
                while (!st.empty()) {
                    uint32_t x = st.back();
                    st.pop_back();
                    if (nodes[x].leaf) emit_leaf_tris(x);
                    else { st.push_back(nodes[x].right); st.push_back(nodes[x].left); }
                }
                node.tri_mask |= (uint16_t)(((1u << cnt) - 1u) << (2 * s));
                tri_off += cnt;
            } else {
                node.imask |= (uint8_t)(1u << s);
                internal_children.push_back(ci);
            }
        }
        if (tri_off > 2 * 8) { err = "internal error: more than 16 triangles in a node"; return false; }
        for (uint32_t ci : internal_children) {
            uint32_t wi = (uint32_t)out.nodes.size();
            out.nodes.emplace_back();
            queue.push_back({ci, wi, it.depth + 1});
        }
        out.nodes[it.wnode] = node;
    }
    if (out.tris.size() != num_tris) { err = "internal error: triangle count mismatch"; return false; }
    out.max_depth = max_depth;
    out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return true;
}

}  // namespace bsm
