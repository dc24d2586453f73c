#include "flatten.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>

namespace pray_gpu {

namespace {

constexpr float kPadRel = 1.0f / 65536.0f;
// Every padded box also grows by this fraction of the scene's diagonal D, and
// only rays whose origin lies within kCullReach diagonals of the scene's
// centre use padded boxes (the others take the exact copy). Float errors grow
// with the distance travelled, not with a box's coordinates: for an origin at
// distance R from the centre, each endpoint of a slab test errs by at most
// 3u(R + D) (u = 2^-24), and a hit that Moeller-Trumbore reports can lie off
// its triangle by about u(R + D) / (sin a sin b), a the triangle's smallest
// angle and b the ray's angle to its plane. The pad, 2^8 u D, keeps such hits
// inside their boxes for sin a sin b down to 1/50 at the reach limit (1/170
// for origins inside the scene). The warp-packet walk's FMA form of the slab
// test (p * inv - o * inv) adds at most 1/25 of the pad.
constexpr float kPadScene = 1.0f / 65536.0f;
constexpr float kCullReach = 4.0f;
// deepest node the flattened hierarchy may have (the kernels' traversal stack
// holds one entry per level)
constexpr int kMaxDeviceDepth = kMaxTraversalDepth;

struct Item {
    uint32_t pos;  // depth-first position of the reference (tie-break key)
    uint32_t tri;  // triangle id
};

struct Tight {
    float lo[3], hi[3];
};

struct Flattener {
    const BuiltTree &t;
    const std::vector<TriPre> &pre;
    int refine;
    DeviceImage &out;
    float pad_scene = 0.f;                            // kPadScene x the scene's diagonal
    std::vector<std::pair<uint32_t, Tight>> tight{};  // interior reference nodes: slot, padded triangle bounds
    std::vector<std::pair<uint32_t, GNode>> linear{};  // refined reference leaves: slot, linear leaf over the same range

    uint32_t alloc_pair() {
        const uint32_t pair = (uint32_t)out.nodes.size();
        out.nodes.resize(out.nodes.size() + 2);
        return pair;
    }

    void put_tri(const Item &it) {
        const TriPre &p = pre[it.tri];
        GTri g;
        uint32_t idbits = it.tri, key = it.pos;
        float idf, keyf;
        std::memcpy(&idf, &idbits, 4);
        std::memcpy(&keyf, &key, 4);
        g.v0[0] = p.a[0], g.v0[1] = p.a[1], g.v0[2] = p.a[2], g.v0[3] = idf;
        g.e1[0] = p.ab[0], g.e1[1] = p.ab[1], g.e1[2] = p.ab[2], g.e1[3] = keyf;
        g.e2[0] = p.ac[0], g.e2[1] = p.ac[1], g.e2[2] = p.ac[2], g.e2[3] = 0.f;
        out.tris.push_back(g);
    }

    // Linear leaf over items[lo, hi) in their current order.
    void linear_leaf(GNode &g, const std::vector<Item> &items, size_t lo, size_t hi) {
        g.a = (uint32_t)out.tris.size();
        g.b = kLeafFlag | (uint32_t)(hi - lo);
        for (size_t i = lo; i < hi; i++) put_tri(items[i]);
    }

    // Padded bounds of the triangles items[lo, hi); an empty range gives the
    // empty box (+inf, -inf), unpadded, which a union ignores.
    void padded_box(const std::vector<Item> &items, size_t lo, size_t hi, float blo[3], float bhi[3]) {
        for (int k = 0; k < 3; k++) blo[k] = INFINITY, bhi[k] = -INFINITY;
        for (size_t i = lo; i < hi; i++) {
            const Aabb &b = pre[items[i].tri].box;
            for (int k = 0; k < 3; k++) blo[k] = std::min(blo[k], b.lo[k]), bhi[k] = std::max(bhi[k], b.hi[k]);
        }
        if (lo >= hi) return;
        for (int k = 0; k < 3; k++) {
            const float pad =
                (std::fabs(blo[k]) + std::fabs(bhi[k]) + (bhi[k] - blo[k])) * kPadRel + pad_scene + 1e-30f;
            blo[k] -= pad;
            bhi[k] += pad;
        }
    }

    // Median split of items[lo, hi) along the longest axis of the centroid
    // bounds; the halves become a new node pair, whose index is returned.
    uint32_t split_pair(std::vector<Item> &items, size_t lo, size_t hi, int depth) {
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = lo; i < hi; i++)
            for (int k = 0; k < 3; k++) {
                const float c = pre[items[i].tri].mid[k];
                clo[k] = std::min(clo[k], c);
                chi[k] = std::max(chi[k], c);
            }
        int axis = 0;
        for (int k = 1; k < 3; k++)
            if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
        const size_t mid = lo + (hi - lo) / 2;
        std::nth_element(items.begin() + lo, items.begin() + mid, items.begin() + hi,
                         [&](const Item &x, const Item &y) {
                             const float a = pre[x.tri].mid[axis], b = pre[y.tri].mid[axis];
                             return a < b || (a == b && x.pos < y.pos);
                         });
        const uint32_t pair = alloc_pair();
        out.sub_nodes += 2;
        sub_tree(items, lo, mid, pair, depth + 1);
        sub_tree(items, mid, hi, pair + 1, depth + 1);
        return pair;
    }

    // Sub-hierarchy node over items[lo, hi) (padded box) written into slot.
    void sub_tree(std::vector<Item> &items, size_t lo, size_t hi, uint32_t slot, int depth) {
        GNode g;
        padded_box(items, lo, hi, g.lo, g.hi);
        if ((int64_t)(hi - lo) <= refine || depth >= kMaxDeviceDepth) {
            linear_leaf(g, items, lo, hi);
            out.nodes[slot] = g;
            return;
        }
        g.a = 0;
        g.b = 0;
        out.nodes[slot] = g;
        const uint32_t pair = split_pair(items, lo, hi, depth);
        out.nodes[slot].a = pair;
    }

    // Reference node p into slot (the box is the reference's, unpadded).
    // Returns the padded bounds of the triangles below it; for an interior
    // node they are recorded in tight[slot].
    Tight put(int32_t p, uint32_t slot, int depth) {
        const FlatNode &n = t.nodes[p];
        GNode g;
        for (int k = 0; k < 3; k++) g.lo[k] = n.box.lo[k], g.hi[k] = n.box.hi[k];
        g.a = 0;
        g.b = 0;
        if (n.left < 0) {
            std::vector<Item> items(n.count);
            for (uint32_t i = 0; i < n.count; i++) items[i] = Item{n.first + i, t.refs[n.first + i]};
            Tight b;
            padded_box(items, 0, items.size(), b.lo, b.hi);
            if (refine <= 0 || (int64_t)n.count <= refine || depth >= kMaxDeviceDepth) {
                linear_leaf(g, items, 0, items.size());
                out.nodes[slot] = g;
                return b;
            }
            out.refined_leaves++;
            out.nodes[slot] = g;
            const uint32_t first = (uint32_t)out.tris.size();
            const uint32_t pair = split_pair(items, 0, items.size(), depth);
            out.nodes[slot].a = pair;
            // the sub-hierarchy's leaves hold the leaf's references, contiguous
            GNode flat = g;
            flat.a = first;
            flat.b = kLeafFlag | (uint32_t)(out.tris.size() - first);
            linear.push_back({slot, flat});
            return b;
        }
        out.nodes[slot] = g;
        const uint32_t pair = alloc_pair();
        out.nodes[slot].a = pair;
        const Tight l = put(n.left, pair, depth + 1);
        const Tight r = put(n.right, pair + 1, depth + 1);
        Tight b;
        for (int k = 0; k < 3; k++) b.lo[k] = std::min(l.lo[k], r.lo[k]), b.hi[k] = std::max(l.hi[k], r.hi[k]);
        tight.push_back({slot, b});
        return b;
    }
};

}  // namespace

void flatten_for_device(const BuiltTree &t, const std::vector<TriPre> &pre, int leaf_refine, DeviceImage &out) {
    out.nodes.assign(2, GNode{});
    out.tris.clear();
    out.tris.reserve(t.refs.size());
    out.refined_leaves = 0;
    out.sub_nodes = 0;
    Flattener f{t, pre, leaf_refine, out};
    const Aabb &root = t.nodes[0].box;
    double d2 = 0.0;
    for (int k = 0; k < 3; k++) d2 += ((double)root.hi[k] - root.lo[k]) * ((double)root.hi[k] - root.lo[k]);
    const bool sized = !t.refs.empty() && std::isfinite(d2);
    const float diag = sized ? (float)std::sqrt(d2) : 0.f;
    f.pad_scene = diag * kPadScene;
    for (int k = 0; k < 3; k++) out.cull_center[k] = sized ? 0.5f * (root.lo[k] + root.hi[k]) : 0.f;
    out.cull_radius2 = sized ? (kCullReach * diag) * (kCullReach * diag) : -1.f;
    f.put(0, 0, 0);
    // the culling copy: same topology; an interior reference node takes the
    // padded bounds of its triangles where they are smaller (by surface area,
    // the chance a ray crosses them) than the reference's box. Either box alone
    // culls conservatively for finite-direction rays; triangle bounds win for
    // fine meshes in voxels with empty space, voxels for coarse meshes whose
    // straddling triangles reach far outside them.
    auto area = [](const float lo[3], const float hi[3]) {
        const double x = (double)hi[0] - lo[0], y = (double)hi[1] - lo[1], z = (double)hi[2] - lo[2];
        return x * y + y * z + z * x;
    };
    out.nodes_tight = out.nodes;
    // the exact copy scans refined leaves linearly: no padded box decides
    // anything for the rays that use it
    for (const auto &[slot, g] : f.linear) out.nodes[slot] = g;
    for (const auto &[slot, b] : f.tight) {
        bool usable = true;  // finite and non-empty (no triangles below: keep the reference's box)
        for (int k = 0; k < 3; k++)
            usable = usable && std::isfinite(b.lo[k]) && std::isfinite(b.hi[k]) && b.lo[k] <= b.hi[k];
        GNode &g = out.nodes_tight[slot];
        if (!usable || !(area(b.lo, b.hi) < area(g.lo, g.hi))) continue;
        for (int k = 0; k < 3; k++) g.lo[k] = b.lo[k], g.hi[k] = b.hi[k];
    }
}

namespace {

bool validate_nodes(const std::vector<GNode> &nodes, uint64_t nt, std::string &why, int &deepest, uint64_t &refs) {
    const uint64_t nn = nodes.size();
    if (nn < 2) {
        why = "device image has no root";
        return false;
    }
    // iterative walk from the root: every child pair and leaf range in
    // bounds, every node reached once, depth within the traversal stack
    std::vector<uint8_t> seen(nn, 0);
    std::vector<std::pair<uint32_t, int>> todo{{0u, 0}};
    seen[0] = 1;
    while (!todo.empty()) {
        const auto [i, d] = todo.back();
        todo.pop_back();
        if (d > kMaxTraversalDepth) {
            why = "device hierarchy deeper than the traversal stack";
            return false;
        }
        deepest = std::max(deepest, d);
        const GNode &g = nodes[i];
        if (g.b & kLeafFlag) {
            const uint64_t cnt = g.b & ~kLeafFlag;
            if ((uint64_t)g.a + cnt > nt) {
                why = "leaf range out of bounds";
                return false;
            }
            refs += cnt;
            continue;
        }
        if (g.b != 0 || (g.a & 1u) || (uint64_t)g.a + 1 >= nn || g.a < 2) {
            why = "child pair out of bounds";
            return false;
        }
        for (uint32_t c = g.a; c <= g.a + 1; c++) {
            if (seen[c]) {
                why = "node reached twice";
                return false;
            }
            seen[c] = 1;
            todo.push_back({c, d + 1});
        }
    }
    return true;
}

}  // namespace

bool validate_device_image(const DeviceImage &img, std::string &why, int *max_depth) {
    int deepest = 0;
    if (img.nodes_tight.size() != img.nodes.size()) {
        why = "node copies differ in size";
        return false;
    }
    uint64_t exact_refs = 0, cull_refs = 0;
    if (!validate_nodes(img.nodes, img.tris.size(), why, deepest, exact_refs) ||
        !validate_nodes(img.nodes_tight, img.tris.size(), why, deepest, cull_refs))
        return false;
    // each copy reaches every triangle reference exactly once
    if (exact_refs != img.tris.size() || cull_refs != img.tris.size()) {
        why = "a node copy does not reach every triangle reference once";
        return false;
    }
    if (max_depth) *max_depth = deepest;
    return true;
}

}  // namespace pray_gpu
