// Host KD-tree builders (median and SAH) producing the reference's trees.
// Independent subtrees are built on separate threads; the result does not
// depend on the schedule.
#include "kdtree.h"

#include <algorithm>
#include <future>
#include <memory>
#include <thread>

namespace pray_gpu {

namespace {

struct BNode {
    Aabb box;
    std::unique_ptr<BNode> left, right;
    int axis = 255;
    float split = 0.f;
    std::vector<uint32_t> tris;
    bool leaf() const { return !tris.empty() || (!left && !right); }
};

int hw_threads(int requested) {
    if (requested > 0) return requested;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

// Depth up to which the two subtrees of a node are built concurrently.
int parallel_depth(int threads) {
    int d = 0;
    while ((1 << d) < 2 * threads && d < 8) d++;
    return d;
}

// ---------------------------------------------------------------- median

struct MedianBuilder {
    const std::vector<TriPre> &tris;
    const TreeOptions &opt;
    int par_depth;

    std::unique_ptr<BNode> build(std::vector<uint32_t> &idx, int depth) {
        auto node = std::make_unique<BNode>();
        Aabb b = tris[idx[0]].box;
        for (size_t i = 1; i < idx.size(); i++) b = b.grown(tris[idx[i]].box);
        node->box = b;
        const int axis = b.longest();
        if ((int64_t)idx.size() <= opt.leaf_size || depth >= opt.max_depth) {
            node->tris = idx;
            return node;
        }
        const size_t half = idx.size() / 2;
        // Same call, comparator and input order as the reference, so the
        // libstdc++ selection permutes the indices identically.
        std::nth_element(idx.begin(), idx.begin() + half, idx.end(),
                         [&](uint32_t l, uint32_t r) { return tris[l].mid[axis] < tris[r].mid[axis]; });
        std::vector<uint32_t> li(idx.begin(), idx.begin() + half), ri(idx.begin() + half, idx.end());
        if (depth < par_depth) {
            auto fut = std::async(std::launch::async, [&] { return build(li, depth + 1); });
            node->right = build(ri, depth + 1);
            node->left = fut.get();
        } else {
            node->left = build(li, depth + 1);
            node->right = build(ri, depth + 1);
        }
        node->axis = axis;
        node->split = tris[idx[half]].mid[axis];
        return node;
    }
};

// ---------------------------------------------------------------- SAH

enum : uint8_t { kEvEnd = 0, kEvLie = 1, kEvStart = 2 };
struct Ev {
    float d;
    uint32_t tri;
    uint8_t axis, type;
};
// Event ordering of include/kd_tree_sah.h:33-36: plane position, then axis,
// then type (end < lying < start). Events equal in all three are
// interchangeable for the sweep and the classification.
inline bool ev_less(const Ev &a, const Ev &b) {
    return (a.d < b.d) || (a.d == b.d && a.axis < b.axis) || (a.d == b.d && a.axis == b.axis && a.type < b.type);
}

// Sorts events by ev_less on up to `threads` threads: a power-of-two number
// of chunks sorted concurrently, then merged pairwise. Events that compare
// equal are interchangeable, so the tree does not depend on their order.
void sort_events(std::vector<Ev> &ev, int threads) {
    const size_t n = ev.size();
    int parts = 1;
    while (2 * parts <= threads && n / (2 * (size_t)parts) >= ((size_t)1 << 16)) parts *= 2;
    if (parts == 1) {
        std::sort(ev.begin(), ev.end(), ev_less);
        return;
    }
    std::vector<size_t> cut(parts + 1);
    for (int i = 0; i <= parts; i++) cut[i] = n * (size_t)i / (size_t)parts;
    {
        std::vector<std::thread> pool;
        for (int i = 0; i < parts; i++)
            pool.emplace_back([&, i] { std::sort(ev.begin() + cut[i], ev.begin() + cut[i + 1], ev_less); });
        for (auto &t : pool) t.join();
    }
    std::vector<Ev> tmp(n);
    std::vector<Ev> *src = &ev, *dst = &tmp;
    for (int w = 1; w < parts; w *= 2) {
        std::vector<std::thread> pool;
        for (int i = 0; i < parts; i += 2 * w) {
            const size_t a = cut[i], m = cut[i + w], b = cut[i + 2 * w];
            pool.emplace_back([=] {
                std::merge(src->begin() + a, src->begin() + m, src->begin() + m, src->begin() + b, dst->begin() + a,
                           ev_less);
            });
        }
        for (auto &t : pool) t.join();
        std::swap(src, dst);
    }
    if (src != &ev) ev.swap(tmp);
}

enum : int8_t { kLeftOnly = -1, kBoth = 0, kRightOnly = 1 };

struct SahBuilder {
    const std::vector<TriPre> &tris;
    const TreeOptions &opt;
    int par_depth;
    size_t ntris;

    void events_of(uint32_t t, const Aabb &vox, std::vector<Ev> &ev) const {
        Aabb eb = tris[t].box.clipped(vox);
        for (int k = 0; k < 3; k++) {
            if (eb.lo[k] - eb.hi[k] == 0) {
                ev.push_back(Ev{eb.lo[k], t, (uint8_t)k, kEvLie});
            } else {
                ev.push_back(Ev{eb.lo[k], t, (uint8_t)k, kEvStart});
                ev.push_back(Ev{eb.hi[k], t, (uint8_t)k, kEvEnd});
            }
        }
    }

    // Cost of one candidate plane (KDTreeSAH::sah, src/kd_tree_sah.cpp:141-166;
    // cost and empty-side bias of include/kd_tree_sah.h:52-71).
    void plane_cost(int axis, float d, const Aabb &b, uint64_t nl, uint64_t nr, uint64_t np, float &c,
                    int &side) const {
        c = std::numeric_limits<float>::max();
        Aabb bl = b, br = b;
        bl.hi[axis] = d;
        br.lo[axis] = d;
        const float ab = b.area();
        const float pl = bl.area() / ab, pr = br.area() / ab;
        if (pl == 0 || pr == 0) return;
        if (b.hi[axis] - b.lo[axis] == 0) return;
        auto cost = [&](uint64_t l, uint64_t r) {
            float lambda = ((l == 0 || r == 0) && !(pl == 1 || pr == 1)) ? 0.8f : 1.0f;
            return lambda * (opt.sah_ct + opt.sah_ci * (pl * (float)l + pr * (float)r));
        };
        const float cl = cost(nl + np, nr), cr = cost(nl, np + nr);
        if (cl < cr) {
            c = cl;
            side = -1;
        } else {
            c = cr;
            side = 1;
        }
    }

    // Plane sweep (KDTreeSAH::findPlane, src/kd_tree_sah.cpp:169-207). After
    // each group of events on one plane the reference's loop index advances
    // once more, so the first event of the following group is not counted;
    // the sweep below keeps that behaviour because the tree depends on it.
    void sweep(uint64_t n, const std::vector<Ev> &ev, const Aabb &b, int &axis, float &d, float &cbest,
               int &side) const {
        cbest = std::numeric_limits<float>::max();
        uint64_t nl[3] = {0, 0, 0}, np[3] = {0, 0, 0}, nr[3] = {n, n, n};
        const size_t m = ev.size();
        size_t i = 0;
        while (i < m) {
            const int pa = ev[i].axis;
            const float pd = ev[i].d;
            uint64_t cnt[3] = {0, 0, 0};
            for (uint8_t ty = kEvEnd; ty <= kEvStart; ty++)
                while (i < m && ev[i].axis == pa && ev[i].d == pd && ev[i].type == ty) cnt[ty]++, i++;
            np[pa] = cnt[kEvLie];
            nr[pa] -= cnt[kEvLie];
            nr[pa] -= cnt[kEvEnd];
            float c;
            int sd = 0;
            plane_cost(pa, pd, b, nl[pa], nr[pa], np[pa], c, sd);
            if (c < cbest) {
                cbest = c;
                axis = pa;
                d = pd;
                side = sd;
            }
            nl[pa] += cnt[kEvStart];
            nl[pa] += cnt[kEvLie];
            np[pa] = 0;
            i++;  // the reference's extra advance
        }
    }

    std::unique_ptr<BNode> build(std::vector<uint32_t> &idx, const Aabb &b, std::vector<Ev> ev, int prev_axis,
                                 float prev_d, int depth, std::vector<int8_t> &side) {
        auto node = std::make_unique<BNode>();
        node->box = b;
        int axis = 255, pside = 0;
        float d = 0.f, c;
        sweep(idx.size(), ev, b, axis, d, c, pside);
        const bool same_plane = (axis == prev_axis && d == prev_d);
        if ((int64_t)idx.size() <= opt.leaf_size || depth >= opt.max_depth || same_plane ||
            c > opt.sah_ci * (float)idx.size()) {
            node->tris = idx;
            return node;
        }
        // classifyLeftRightBoth (src/kd_tree_sah.cpp:209-232)
        for (uint32_t t : idx) side[t] = kBoth;
        for (const Ev &e : ev) {
            if (e.axis != axis) continue;
            if (e.type == kEvEnd && e.d <= d)
                side[e.tri] = kLeftOnly;
            else if (e.type == kEvStart && e.d >= d)
                side[e.tri] = kRightOnly;
            else if (e.type == kEvLie) {
                if (e.d < d || (e.d == d && pside == -1))
                    side[e.tri] = kLeftOnly;
                else if (e.d > d || (e.d == d && pside == 1))
                    side[e.tri] = kRightOnly;
            }
        }
        Aabb vl = b, vr = b;
        vl.hi[axis] = d;
        vr.lo[axis] = d;
        // splitAndGenerate (src/kd_tree_sah.cpp:250-270)
        std::vector<uint32_t> tl, tr;
        std::vector<Ev> bl, br;
        for (uint32_t t : idx) {
            if (side[t] == kLeftOnly) {
                tl.push_back(t);
            } else if (side[t] == kRightOnly) {
                tr.push_back(t);
            } else {
                events_of(t, vl, bl);
                events_of(t, vr, br);
                tl.push_back(t);
                tr.push_back(t);
            }
        }
        // splitEvents + mergeStrains (src/kd_tree_sah.cpp:235-248, 286-296):
        // one-sided events keep their sorted order, new straddler events are
        // sorted and merged in.
        std::sort(bl.begin(), bl.end(), ev_less);
        std::sort(br.begin(), br.end(), ev_less);
        std::vector<Ev> le, re;
        {
            std::vector<Ev> lo, ro;
            lo.reserve(ev.size());
            ro.reserve(ev.size());
            for (const Ev &e : ev) {
                if (side[e.tri] == kLeftOnly)
                    lo.push_back(e);
                else if (side[e.tri] == kRightOnly)
                    ro.push_back(e);
            }
            std::vector<Ev>().swap(ev);
            le.resize(lo.size() + bl.size());
            re.resize(ro.size() + br.size());
            std::merge(lo.begin(), lo.end(), bl.begin(), bl.end(), le.begin(), ev_less);
            std::merge(ro.begin(), ro.end(), br.begin(), br.end(), re.begin(), ev_less);
        }
        std::vector<Ev>().swap(bl);
        std::vector<Ev>().swap(br);
        if (depth < par_depth) {
            auto fut = std::async(std::launch::async, [&] {
                std::vector<int8_t> own(ntris, kBoth);
                return build(tl, vl, std::move(le), axis, d, depth + 1, own);
            });
            node->right = build(tr, vr, std::move(re), axis, d, depth + 1, side);
            node->left = fut.get();
        } else {
            node->left = build(tl, vl, std::move(le), axis, d, depth + 1, side);
            node->right = build(tr, vr, std::move(re), axis, d, depth + 1, side);
        }
        node->axis = axis;
        node->split = d;
        return node;
    }
};

// ---------------------------------------------------------------- flatten

struct Stats {
    uint64_t sub_nodes = 0, depth_to_leaf = 0, sub_leaves = 0, sub_empty = 0;
};

Stats flatten(const BNode *n, BuiltTree &out) {
    const int32_t me = (int32_t)out.nodes.size();
    out.nodes.emplace_back();
    out.nodes[me].box = n->box;
    Stats s;
    if (n->leaf()) {
        out.nodes[me].first = (uint32_t)out.refs.size();
        out.nodes[me].count = (uint32_t)n->tris.size();
        out.refs.insert(out.refs.end(), n->tris.begin(), n->tris.end());
        return s;
    }
    out.nodes[me].axis = n->axis;
    out.nodes[me].split = n->split;
    out.nodes[me].first = (uint32_t)out.refs.size();
    out.nodes[me].left = (int32_t)out.nodes.size();
    Stats l = flatten(n->left.get(), out);
    out.nodes[me].right = (int32_t)out.nodes.size();
    Stats r = flatten(n->right.get(), out);
    // KDTreeElement::log (include/kd_tree.h:122-132)
    const bool ll = n->left->leaf(), rl = n->right->leaf();
    s.sub_nodes = l.sub_nodes + r.sub_nodes + 2;
    s.depth_to_leaf = std::max(l.depth_to_leaf, r.depth_to_leaf) + 1;
    s.sub_leaves = (ll ? 1 : l.sub_leaves) + (rl ? 1 : r.sub_leaves);
    s.sub_empty = (ll ? (n->left->tris.empty() ? 1 : 0) : l.sub_empty) +
                  (rl ? (n->right->tris.empty() ? 1 : 0) : r.sub_empty);
    return s;
}

}  // namespace

std::vector<TriPre> precompute_triangles(const float *verts, uint64_t n, int threads) {
    std::vector<TriPre> out(n);
    const int nt = std::max(1, std::min<int>(hw_threads(threads), (int)(n / 65536) + 1));
    std::vector<std::thread> pool;
    for (int w = 0; w < nt; w++)
        pool.emplace_back([&, w] {
            for (uint64_t i = w; i < n; i += nt) out[i] = precompute_triangle(verts + 9 * i);
        });
    for (auto &t : pool) t.join();
    return out;
}

BuiltTree build_tree(const std::vector<TriPre> &tris, const TreeOptions &opt) {
    BuiltTree out;
    if (tris.empty()) {
        out.nodes.emplace_back();  // empty root leaf (src/kd_tree.cpp:26-29)
        return out;
    }
    const int threads = hw_threads(opt.threads);
    std::vector<uint32_t> idx(tris.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (uint32_t)i;
    std::unique_ptr<BNode> root;
    if (opt.kind == kTreeMedian) {
        MedianBuilder mb{tris, opt, parallel_depth(threads)};
        root = mb.build(idx, 0);
    } else {
        Aabb rb = tris[0].box;
        for (size_t i = 0; i < tris.size(); i++) rb = rb.grown(tris[i].box);
        SahBuilder sb{tris, opt, parallel_depth(threads), tris.size()};
        std::vector<Ev> ev;
        ev.reserve(tris.size() * 6);
        for (uint32_t t : idx) sb.events_of(t, rb, ev);
        sort_events(ev, threads);
        std::vector<int8_t> side(tris.size(), kBoth);
        root = sb.build(idx, rb, std::move(ev), 255, 0.f, 0, side);
    }
    out.nodes.reserve(1024);
    Stats s = flatten(root.get(), out);
    out.maxdepth = s.depth_to_leaf;
    out.leaf_nodes = s.sub_leaves;
    out.empty_leaves = s.sub_empty;
    return out;
}

}  // namespace pray_gpu
