// ORACLE — test infrastructure, not product code.
//
// A plain C++ restatement of the reference's hot path, used only by tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg to check (never to
// produce) the results of the CUDA path. Compiled with -ffp-contract=off so
// that every float operation rounds exactly as in the reference's scalar build.
// Parity is pinned against the reference's own code built from source
// (build_ref.sh, ref_harness.cpp): tests/golden/ holds the fixtures that the
// reference produced, and tests/test_oracle_golden.py checks this file against
// them.
//
// Each function cites the reference code whose arithmetic it restates
// (paths relative to the reference project root).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

#include <omp.h>

#include "../include/nostrum_pray_sampling.h"


namespace {

constexpr float kMax = std::numeric_limits<float>::max();
constexpr float kLowest = std::numeric_limits<float>::lowest();

// std::min / std::max select semantics (first argument on ties and NaN).
inline float smin(float a, float b) { return (b < a) ? b : a; }
inline float smax(float a, float b) { return (a < b) ? b : a; }

struct V3 {
    float x, y, z;
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 scale(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// Vec3::normalize, include/geometry.h:29-35
inline V3 normalized(V3 v) {
    float n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (n2 > 0) {
        float inv = 1 / std::sqrt(n2);
        v.x *= inv, v.y *= inv, v.z *= inv;
    }
    return v;
}

struct Ray {
    V3 o, d, inv;
};
// Ray ctor, include/geometry.h:82-87
inline Ray make_ray(V3 o, V3 d) {
    Ray r;
    r.o = o;
    r.d = normalized(d);
    r.inv = {1 / r.d.x, 1 / r.d.y, 1 / r.d.z};
    return r;
}

struct Box {
    V3 lo, hi;
};
// BoundingBox::expand, include/geometry.h:110-117
inline Box expand(const Box &a, const Box &b) {
    return {{smin(a.lo.x, b.lo.x), smin(a.lo.y, b.lo.y), smin(a.lo.z, b.lo.z)},
            {smax(a.hi.x, b.hi.x), smax(a.hi.y, b.hi.y), smax(a.hi.z, b.hi.z)}};
}
// BoundingBox::clip, include/geometry.h:119-126
inline Box clip(const Box &a, const Box &b) {
    return {{smax(a.lo.x, b.lo.x), smax(a.lo.y, b.lo.y), smax(a.lo.z, b.lo.z)},
            {smin(a.hi.x, b.hi.x), smin(a.hi.y, b.hi.y), smin(a.hi.z, b.hi.z)}};
}
// BoundingBox::getLongestAxis, include/geometry.h:132-149
inline int longest_axis(const Box &b) {
    float x = b.hi.x - b.lo.x, y = b.hi.y - b.lo.y, z = b.hi.z - b.lo.z;
    if (x >= y && x >= z) return 0;
    if (y >= x && y >= z) return 1;
    return 2;
}
// BoundingBox::surfaceArea, include/geometry.h:186-192
inline float area(const Box &b) {
    float dx = b.hi.x - b.lo.x, dy = b.hi.y - b.lo.y, dz = b.hi.z - b.lo.z;
    return 2.f * (dx * dy + dx * dz + dy * dz);
}
inline float &comp(V3 &v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
// BoundingBox::split, include/geometry.h:195-213
inline void split_box(const Box &b, int axis, float d, Box &l, Box &r) {
    l = b;
    r = b;
    comp(l.hi, axis) = d;
    comp(r.lo, axis) = d;
}
// BoundingBox::intersect (infinite-line slab test), include/geometry.h:151-164
inline bool slab(const Box &b, const Ray &r) {
    V3 t1 = mul(sub(b.lo, r.o), r.inv);
    V3 t2 = mul(sub(b.hi, r.o), r.inv);
    float n = smax(smax(smin(t1.x, t2.x), smin(t1.y, t2.y)), smax(smin(t1.z, t2.z), kLowest));
    float f = smin(smin(smax(t1.x, t2.x), smax(t1.y, t2.y)), smin(smax(t1.z, t2.z), kMax));
    return n <= f;
}

struct Tri {
    V3 a, b, c, color;
    bool emit;
    V3 normal, ab, ac, mid;
    Box box;
};
// Moeller-Trumbore, one-sided, include/geometry.h:242-262 (eps = det threshold)
inline bool intersect_tri(const Tri &t, const Ray &r, float eps, float &dist) {
    V3 p = cross(r.d, t.ac);
    float det = dot(t.ab, p);
    if (det < eps) return false;
    float inv = 1 / det;
    V3 tv = sub(r.o, t.a);
    float u = dot(tv, p) * inv;
    if (u < 0.f || u > 1.f) return false;
    V3 q = cross(tv, t.ab);
    float v = dot(r.d, q) * inv;
    if (v < 0.f || u + v > 1.f) return false;
    dist = dot(t.ac, q) * inv;
    return true;
}

struct Node {
    Box box;
    int left = -1, right = -1;  // child node indices (-1: none)
    int axis = 255;
    float split = 0.f;
    std::vector<int64_t> tris;  // leaf triangle indices
    bool leaf() const { return !tris.empty() || (left < 0 && right < 0); }
    // statistics of KDTreeElement::log, include/kd_tree.h:122-132
    uint64_t sub_nodes = 0, depth_to_leaf = 0, sub_leaves = 0, sub_empty = 0;
};

struct Scene {
    std::vector<Tri> tris;
    std::vector<Node> nodes;  // nodes[0] is the root
    int leaf_size = 32, max_depth = 20;
    float ct = 5.f, ci = 1.5f;
    uint64_t nnodes = 0, maxdepth = 0, leaf_nodes = 0, empty_leaves = 0;
};

void log_stats(Scene &s, int id) {
    Node &n = s.nodes[id];
    const Node &l = s.nodes[n.left];
    const Node &r = s.nodes[n.right];
    n.sub_nodes = l.sub_nodes + r.sub_nodes + 2;
    n.depth_to_leaf = std::max(l.depth_to_leaf, r.depth_to_leaf) + 1;
    n.sub_leaves += l.leaf() ? 1 : l.sub_leaves;
    n.sub_leaves += r.leaf() ? 1 : r.sub_leaves;
    n.sub_empty += l.leaf() ? (l.tris.empty() ? 1 : 0) : l.sub_empty;
    n.sub_empty += r.leaf() ? (r.tris.empty() ? 1 : 0) : r.sub_empty;
}

// ---- median tree: KDTree::buildRecursive, src/kd_tree.cpp:48-84 ----------
int build_median(Scene &s, std::vector<int64_t> &idx, int depth) {
    Box b = s.tris[idx[0]].box;
    for (size_t i = 1; i < idx.size(); i++) b = expand(b, s.tris[idx[i]].box);
    int axis = longest_axis(b);
    int me = (int)s.nodes.size();
    s.nodes.emplace_back();
    s.nodes[me].box = b;
    if ((int64_t)idx.size() <= s.leaf_size || depth >= s.max_depth) {
        s.nodes[me].tris = idx;
        return me;
    }
    size_t half = idx.size() / 2;
    std::nth_element(idx.begin(), idx.begin() + half, idx.end(), [&](int64_t l, int64_t r) {
        return s.tris[l].mid[axis] < s.tris[r].mid[axis];
    });
    std::vector<int64_t> li(idx.begin(), idx.begin() + half), ri(idx.begin() + half, idx.end());
    int l = build_median(s, li, depth + 1);
    int r = build_median(s, ri, depth + 1);
    Node &n = s.nodes[me];
    n.left = l;
    n.right = r;
    n.axis = axis;
    n.split = s.tris[idx[half]].mid[axis];
    log_stats(s, me);
    return me;
}

// ---- SAH kd tree: KDTreeSAH, src/kd_tree_sah.cpp:32-296 --------------------
enum EvType : int { kEnd = 0, kLie = 1, kStart = 2 };
struct Event {
    int64_t tri;
    int axis;
    float d;
    int type;
    // Event::operator<, include/kd_tree_sah.h:33-36
    bool operator<(const Event &e) const {
        return (d < e.d) || (d == e.d && axis < e.axis) || (d == e.d && axis == e.axis && type < e.type);
    }
};
enum Side : int8_t { kLeftOnly = -1, kBoth = 0, kRightOnly = 1 };

// KDTreeSAH::generateEvents, src/kd_tree_sah.cpp:272-284
void gen_events(const Scene &s, int64_t t, const Box &vox, std::vector<Event> &ev) {
    Box eb = clip(s.tris[t].box, vox);
    for (int k = 0; k < 3; k++) {
        if (eb.lo[k] - eb.hi[k] == 0) {
            ev.push_back({t, k, eb.lo[k], kLie});
        } else {
            ev.push_back({t, k, eb.lo[k], kStart});
            ev.push_back({t, k, eb.hi[k], kEnd});
        }
    }
}

// KDTreeSAH::sah, src/kd_tree_sah.cpp:141-166, with cost/lambda of
// include/kd_tree_sah.h:52-71
void sah_cost(const Scene &s, int axis, float d, const Box &b, uint64_t nl, uint64_t nr, uint64_t np,
              float &c, int &side) {
    c = kMax;
    Box bl, br;
    split_box(b, axis, d, bl, br);
    float pl = area(bl) / area(b);
    float pr = area(br) / area(b);
    if (pl == 0 || pr == 0) return;
    if (b.hi[axis] - b.lo[axis] == 0) return;
    auto cost = [&](uint64_t l, uint64_t r) {
        float lambda = ((l == 0 || r == 0) && !(pl == 1 || pr == 1)) ? 0.8f : 1.0f;
        return lambda * (s.ct + s.ci * (pl * (float)l + pr * (float)r));
    };
    float cl = cost(nl + np, nr);
    float cr = cost(nl, np + nr);
    if (cl < cr) {
        c = cl;
        side = -1;
    } else {
        c = cr;
        side = 1;
    }
}

// KDTreeSAH::findPlane, src/kd_tree_sah.cpp:169-207. The sweep advances one
// extra event after each plane group, exactly as the reference's loop does.
void find_plane(const Scene &s, uint64_t n, const std::vector<Event> &ev, const Box &b, int &axis,
                float &d, float &cbest, int &side) {
    cbest = kMax;
    uint64_t nl[3] = {0, 0, 0}, np[3] = {0, 0, 0}, nr[3] = {n, n, n};
    for (size_t i = 0; i < ev.size(); i++) {
        const int pa = ev[i].axis;
        const float pd = ev[i].d;
        uint64_t lie = 0, start = 0, end = 0;
        while (i < ev.size() && ev[i].axis == pa && ev[i].d == pd && ev[i].type == kEnd) end++, i++;
        while (i < ev.size() && ev[i].axis == pa && ev[i].d == pd && ev[i].type == kLie) lie++, i++;
        while (i < ev.size() && ev[i].axis == pa && ev[i].d == pd && ev[i].type == kStart) start++, i++;
        np[pa] = lie;
        nr[pa] -= lie;
        nr[pa] -= end;
        float c;
        int sd = 0;
        sah_cost(s, pa, pd, b, nl[pa], nr[pa], np[pa], c, sd);
        if (c < cbest) {
            cbest = c;
            axis = pa;
            d = pd;
            side = sd;
        }
        nl[pa] += start;
        nl[pa] += lie;
        np[pa] = 0;
    }
}

int build_sah(Scene &s, std::vector<int64_t> &idx, const Box &b, const std::vector<Event> &ev, int prev_axis,
              float prev_d, int depth, std::vector<int8_t> &side_of) {
    int axis = 255;
    float d = 0.f, c;
    int pside = 0;
    find_plane(s, idx.size(), ev, b, axis, d, c, pside);
    int me = (int)s.nodes.size();
    s.nodes.emplace_back();
    s.nodes[me].box = b;
    // termination, src/kd_tree_sah.cpp:102 and include/kd_tree_sah.h:75-77
    bool same_plane = (axis == prev_axis && d == prev_d);
    if ((int64_t)idx.size() <= s.leaf_size || depth >= s.max_depth || same_plane || c > s.ci * (float)idx.size()) {
        s.nodes[me].tris = idx;
        return me;
    }
    // classifyLeftRightBoth, src/kd_tree_sah.cpp:209-232
    for (int64_t t : idx) side_of[t] = kBoth;
    for (const Event &e : ev) {
        if (e.axis != axis) continue;
        if (e.type == kEnd && e.d <= d) {
            side_of[e.tri] = kLeftOnly;
        } else if (e.type == kStart && e.d >= d) {
            side_of[e.tri] = kRightOnly;
        } else if (e.type == kLie) {
            if (e.d < d || (e.d == d && pside == -1))
                side_of[e.tri] = kLeftOnly;
            else if (e.d > d || (e.d == d && pside == 1))
                side_of[e.tri] = kRightOnly;
        }
    }
    // splitEvents, src/kd_tree_sah.cpp:235-248
    std::vector<Event> lo, ro;
    for (const Event &e : ev) {
        if (side_of[e.tri] == kLeftOnly)
            lo.push_back(e);
        else if (side_of[e.tri] == kRightOnly)
            ro.push_back(e);
    }
    Box vl, vr;
    split_box(b, axis, d, vl, vr);
    // splitAndGenerate, src/kd_tree_sah.cpp:250-270
    std::vector<Event> bl, br;
    std::vector<int64_t> tl, tr;
    for (int64_t t : idx) {
        if (side_of[t] == kLeftOnly) {
            tl.push_back(t);
        } else if (side_of[t] == kRightOnly) {
            tr.push_back(t);
        } else {
            gen_events(s, t, vl, bl);
            gen_events(s, t, vr, br);
            tl.push_back(t);
            tr.push_back(t);
        }
    }
    // mergeStrains, src/kd_tree_sah.cpp:286-296
    std::sort(bl.begin(), bl.end());
    std::sort(br.begin(), br.end());
    std::vector<Event> le(lo.size() + bl.size()), re(ro.size() + br.size());
    std::merge(lo.begin(), lo.end(), bl.begin(), bl.end(), le.begin());
    std::merge(ro.begin(), ro.end(), br.begin(), br.end(), re.begin());
    lo.clear(); lo.shrink_to_fit();
    ro.clear(); ro.shrink_to_fit();
    int l = build_sah(s, tl, vl, le, axis, d, depth + 1, side_of);
    int r = build_sah(s, tr, vr, re, axis, d, depth + 1, side_of);
    Node &n = s.nodes[me];
    n.left = l;
    n.right = r;
    n.axis = axis;
    n.split = d;
    log_stats(s, me);
    return me;
}

// initialiseTriangles, src/scene_preprocessor.cpp:74-96
void precompute(Tri &t) {
    t.box.lo = {smin(t.a.x, smin(t.b.x, t.c.x)), smin(t.a.y, smin(t.b.y, t.c.y)), smin(t.a.z, smin(t.b.z, t.c.z))};
    t.box.hi = {smax(t.a.x, smax(t.b.x, t.c.x)), smax(t.a.y, smax(t.b.y, t.c.y)), smax(t.a.z, smax(t.b.z, t.c.z))};
    V3 s3 = add(add(t.a, t.b), t.c);
    t.mid = {s3.x / 3, s3.y / 3, s3.z / 3};
    t.ab = sub(t.b, t.a);
    t.ac = sub(t.c, t.a);
    t.normal = normalized(cross(t.ab, t.ac));
}

// KDTree::intersectRecursive, src/kd_tree.cpp:237-279: depth-first over every
// node whose box the ray's line crosses, left child before right; the first
// visited triangle wins ties.
bool trace_dfs(const Scene &s, int id, const Ray &r, float eps, int64_t &best, float &dist) {
    const Node &n = s.nodes[id];
    if (!slab(n.box, r)) return false;
    if (n.left >= 0 || n.right >= 0) {
        bool hl = false, hr = false;
        if (n.left >= 0) hl = trace_dfs(s, n.left, r, eps, best, dist);
        if (n.right >= 0) hr = trace_dfs(s, n.right, r, eps, best, dist);
        return hl || hr;
    }
    bool hit = false;
    float md = kMax;
    int64_t mi = 0;
    for (int64_t t : n.tris) {
        float td;
        if (intersect_tri(s.tris[t], r, eps, td)) {
            if (td < md && td > 0) {
                hit = true;
                md = td;
                mi = t;
            }
        }
    }
    if (hit && md < dist) {
        best = mi;
        dist = md;
        return true;
    }
    return false;
}

bool closest(const Scene &s, const Ray &r, float eps, int64_t &id, float &dist) {
    dist = kMax;
    id = -1;
    if (s.tris.empty()) return false;
    return trace_dfs(s, 0, r, eps, id, dist);
}

// Matrix44::inverse (Gauss-Jordan with partial pivoting), include/geometry.h:322-403
void invert44(const float m[4][4], float s[4][4]) {
    float t[4][4];
    std::memcpy(t, m, sizeof(t));
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) s[i][j] = (i == j) ? 1.f : 0.f;
    auto identity = [&]() {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) s[i][j] = (i == j) ? 1.f : 0.f;
    };
    for (int i = 0; i < 3; i++) {
        int piv = i;
        float best = t[i][i] < 0 ? -t[i][i] : t[i][i];
        for (int j = i + 1; j < 4; j++) {
            float a = t[j][i] < 0 ? -t[j][i] : t[j][i];
            if (a > best) piv = j, best = a;
        }
        if (best == 0) return identity();
        if (piv != i)
            for (int j = 0; j < 4; j++) std::swap(t[i][j], t[piv][j]), std::swap(s[i][j], s[piv][j]);
        for (int j = i + 1; j < 4; j++) {
            float f = t[j][i] / t[i][i];
            for (int k = 0; k < 4; k++) t[j][k] -= f * t[i][k], s[j][k] -= f * s[i][k];
        }
    }
    for (int i = 3; i >= 0; --i) {
        float f = t[i][i];
        if (f == 0) return identity();
        for (int j = 0; j < 4; j++) t[i][j] /= f, s[i][j] /= f;
        for (int j = 0; j < i; j++) {
            f = t[j][i];
            for (int k = 0; k < 4; k++) t[j][k] -= f * t[i][k], s[j][k] -= f * s[i][k];
        }
    }
}

struct Camera {
    float inv[4][4];
    float inv_w, inv_h, aspect, angle;
    V3 pos;
    uint64_t w, h;
};
// calculatePrimRays set-up, src/scene_preprocessor.cpp:98-120
Camera make_camera(uint64_t w, uint64_t h, uint64_t fov, V3 pos, V3 look) {
    Camera c;
    V3 target = add(pos, look);
    V3 up{0, 1, 0};
    V3 z = normalized(sub(target, pos));
    V3 x = normalized(cross(up, z));
    V3 y = cross(z, x);
    float view[4][4] = {{x.x, y.x, z.x, 0},
                        {x.y, y.y, z.y, 0},
                        {x.z, y.z, z.z, 0},
                        {-dot(x, pos), -dot(y, pos), -dot(z, pos), 1}};
    invert44(view, c.inv);
    c.inv_w = 1 / float(w);
    c.inv_h = 1 / float(h);
    c.aspect = w / float(h);
    const float pi = static_cast<float>(std::acos(-1));
    c.angle = std::tan(pi * 0.5f * fov / 180.f);
    c.pos = pos;
    c.w = w;
    c.h = h;
    return c;
}
// per-pixel ray, src/scene_preprocessor.cpp:124-134 and Matrix44::multDirMatrix,
// include/geometry.h:312-320
Ray primary(const Camera &c, uint64_t px, uint64_t py) {
    float x = (2 * ((px + 0.5f) * c.inv_w) - 1) * c.angle;
    float y = (1 - 2 * ((py + 0.5f) * c.inv_h)) * c.angle / c.aspect;
    const float(*m)[4] = c.inv;
    V3 d{x * m[0][0] + y * m[1][0] + 1 * m[2][0], x * m[0][1] + y * m[1][1] + 1 * m[2][1],
         x * m[0][2] + y * m[1][2] + 1 * m[2][2]};
    return make_ray(c.pos, d);
}

struct Light {
    V3 pos, color;
};

// evaluateRay (scalar), src/pray.cpp:17-55; returns the unclamped background on
// a miss exactly like the reference.
V3 shade_rt(const Scene &s, const Ray &r, const std::vector<Light> &lights, V3 bg, float eps,
            uint64_t &shadow_rays) {
    int64_t id;
    float dist;
    if (!closest(s, r, eps, id, dist)) return bg;
    const Tri &t = s.tris[id];
    V3 color{0.f, 0.f, 0.f};
    V3 hit = add(r.o, scale(r.d, dist));
    for (const Light &l : lights) {
        V3 L = sub(l.pos, hit);
        float d2 = L.x * L.x + L.y * L.y + L.z * L.z;
        L = normalized(L);
        float lambert = dot(L, t.normal);
        if (lambert < 0.f) continue;
        int64_t sid;
        float sd;
        shadow_rays++;
        if (closest(s, make_ray(hit, L), eps, sid, sd) && d2 > sd * sd) continue;
        color = add(color, scale(scale(mul(t.color, l.color), lambert), 1 / d2));
        if (color.x >= 1.f && color.y >= 1.f && color.z >= 1.f) break;
    }
    auto cl = [](float v) { return smax(0.f, smin(1.f, v)); };
    return {cl(color.x), cl(color.y), cl(color.z)};
}

// static_cast<uint8_t>(c * 255.f + 0.5f) of src/pray.cpp:470-476 for values in
// [0, 255.5]; outside that range the C++ conversion is undefined, and this
// takes the low byte of the truncated integer.
inline uint8_t quantise(float c) {
    float v = c * 255.f + 0.5f;
    return (uint8_t)(uint32_t)(int32_t)v;
}

// ---- path tracing -----------------------------------------------------------
// Kajiya mode restates evaluatePathRecursive / evaluatePath
// (src/pray.cpp:342-378) with the PCG32 streams and hemisphere sampling of
// include/nostrum_pray_sampling.h in place of the reference's clock-seeded
// mt19937_64. NEE mode is this project's next-event-estimation variant (no
// reference counterpart); branching mode restates the reference's
// evaluatePathRecursiveDiffuse. The CUDA kernels must match this code's float
// operation order.

struct Emitters {
    std::vector<int64_t> ids;
    std::vector<float> cdf;
    float area = 0.f;
};

Emitters collect_emitters(const Scene &s) {
    Emitters e;
    double acc = 0.0;
    for (size_t i = 0; i < s.tris.size(); i++) {
        const Tri &t = s.tris[i];
        if (!t.emit) continue;
        const V3 c = cross(t.ab, t.ac);
        const double a = 0.5 * std::sqrt((double)c.x * c.x + (double)c.y * c.y + (double)c.z * c.z);
        if (!(a > 0.0)) continue;
        acc += a;
        e.ids.push_back((int64_t)i);
        e.cdf.push_back((float)acc);
    }
    e.area = e.cdf.empty() ? 0.f : e.cdf.back();
    return e;
}

V3 path_kajiya(const Scene &s, Ray r, V3 bg, uint32_t max_depth, float eps, pray_pcg32 &g, uint64_t &segs) {
    std::vector<V3> albedo;
    V3 L;
    while (true) {
        int64_t id;
        float t;
        segs++;
        if (!closest(s, r, eps, id, t)) {
            L = bg;
            break;
        }
        const Tri &tri = s.tris[id];
        if (tri.emit) {
            L = tri.color;
            break;
        }
        if (albedo.size() >= max_depth) {
            L = {0.f, 0.f, 0.f};
            break;
        }
        albedo.push_back(tri.color);
        V3 hit = add(r.o, scale(r.d, t));
        const float u1 = pray_uniform(&g), u2 = pray_uniform(&g);
        const float n[3] = {tri.normal.x, tri.normal.y, tri.normal.z};
        float d[3];
        pray_sample_hemisphere(n, u1, u2, d);
        r = make_ray(hit, {d[0], d[1], d[2]});
    }
    for (size_t k = albedo.size(); k-- > 0;) L = mul(L, albedo[k]);
    return L;
}

// The reference's branching recursion (evaluatePathRecursiveDiffuse,
// src/pray.cpp:315-340): num_samples bounce rays at every non-emitting hit
// above max_depth, (sum of their values * albedo) / num_samples. The two
// uniforms of each bounce come from one PCG32 stream in depth-first order
// (the reference draws from a clock-seeded mt19937_64 per call).
V3 path_diffuse(const Scene &s, const Ray &r, V3 bg, uint32_t max_depth, uint32_t n, float eps, pray_pcg32 &g,
                uint64_t &segs, uint32_t depth) {
    int64_t id;
    float t;
    segs++;
    if (!closest(s, r, eps, id, t)) return bg;
    const Tri &tri = s.tris[id];
    if (tri.emit) return tri.color;
    if (depth >= max_depth) return {0.f, 0.f, 0.f};
    const V3 hit = add(r.o, scale(r.d, t));
    const float nrm[3] = {tri.normal.x, tri.normal.y, tri.normal.z};
    V3 sum{0.f, 0.f, 0.f};
    for (uint32_t i = 0; i < n; i++) {
        const float u1 = pray_uniform(&g), u2 = pray_uniform(&g);
        float d[3];
        pray_sample_hemisphere(nrm, u1, u2, d);
        sum = add(sum, path_diffuse(s, make_ray(hit, {d[0], d[1], d[2]}), bg, max_depth, n, eps, g, segs, depth + 1));
    }
    const V3 m = mul(sum, tri.color);
    const float nf = (float)n;
    return {m.x / nf, m.y / nf, m.z / nf};
}

V3 path_nee(const Scene &s, const Emitters &em, Ray r, V3 bg, uint32_t max_depth, uint32_t rr_depth, float eps,
            pray_pcg32 &g, uint64_t &segs) {
    V3 T{1.f, 1.f, 1.f}, L{0.f, 0.f, 0.f};
    const float inv_pi = 0.318309886183790671538f;
    for (uint32_t depth = 0;; depth++) {
        int64_t id;
        float t;
        segs++;
        if (!closest(s, r, eps, id, t)) {
            L = add(L, mul(T, bg));
            break;
        }
        const Tri &tri = s.tris[id];
        if (tri.emit) {
            if (depth == 0) L = add(L, mul(T, tri.color));
            break;
        }
        if (depth >= max_depth) break;
        const V3 hit = add(r.o, scale(r.d, t));
        if (!em.ids.empty()) {
            const float ue = pray_uniform(&g), ua = pray_uniform(&g), ub = pray_uniform(&g);
            const float target = ue * em.area;
            size_t lo = 0, hi = em.ids.size() - 1;
            while (lo < hi) {
                const size_t mid = (lo + hi) >> 1;
                if (em.cdf[mid] > target) hi = mid;
                else lo = mid + 1;
            }
            const Tri &E = s.tris[em.ids[lo]];
            const float su = std::sqrt(ua);
            const float b1 = su * (1.f - ub), b2 = su * ub;
            const V3 y{E.a.x + E.ab.x * b1 + E.ac.x * b2, E.a.y + E.ab.y * b1 + E.ac.y * b2,
                       E.a.z + E.ab.z * b1 + E.ac.z * b2};
            V3 w = sub(y, hit);
            const float d2 = w.x * w.x + w.y * w.y + w.z * w.z;
            if (d2 > 0.f) {
                const float inv = 1.0f / std::sqrt(d2);
                w = {w.x * inv, w.y * inv, w.z * inv};
                const float cx = dot(tri.normal, w);
                const float cy = -dot(E.normal, w);
                if (cx > 0.f && cy > 0.f) {
                    segs++;
                    int64_t sid;
                    float st;
                    const bool blocked = closest(s, make_ray(hit, w), eps, sid, st) && d2 * 0.999f > st * st;
                    if (!blocked) {
                        const float gterm = ((cx * cy) * em.area) * inv_pi / d2;
                        L = {L.x + ((T.x * tri.color.x) * E.color.x) * gterm, L.y + ((T.y * tri.color.y) * E.color.y) * gterm,
                             L.z + ((T.z * tri.color.z) * E.color.z) * gterm};
                    }
                }
            }
        }
        const float u1 = pray_uniform(&g), u2 = pray_uniform(&g);
        const float n[3] = {tri.normal.x, tri.normal.y, tri.normal.z};
        float d[3];
        pray_sample_hemisphere(n, u1, u2, d);
        r = make_ray(hit, {d[0], d[1], d[2]});
        T = mul(T, tri.color);
        if (depth >= rr_depth) {
            const float q = smin(smax(smax(T.x, T.y), T.z), 0.95f);
            if (!(pray_uniform(&g) < q)) break;
            T = {T.x / q, T.y / q, T.z / q};
        }
    }
    return L;
}

// Threads of the most recent parallel frame loop, as OpenMP ran it (not as
// requested): the CPU baselines report this count.
int g_last_threads = 0;
inline void note_threads() {
    if (omp_get_thread_num() == 0) g_last_threads = omp_get_num_threads();
}

}  // namespace

extern "C" {

int orc_last_threads() { return g_last_threads; }

// cos/sin(2 pi u) of the shared sampling header, for accuracy tests.
void orc_sincos_turns(const float *u, uint64_t n, float *s_out, float *c_out) {
    for (uint64_t i = 0; i < n; i++) pray_sincos_turns(u[i], s_out + i, c_out + i);
}

void orc_sample_hemisphere(const float *normals, const float *u, uint64_t n, float *dirs) {
    for (uint64_t i = 0; i < n; i++) pray_sample_hemisphere(normals + 3 * i, u[2 * i], u[2 * i + 1], dirs + 3 * i);
}

// Path-traced rows [row0, row1): out_rgb width*(row1-row0)*3 bytes, out_rad
// (may be NULL) the mean radiance per pixel. Returns the ray segments cast.
// sample_offset selects the first PCG stream (sample index); out_sum64 (may
// be NULL) is added to, one sample at a time in sample order, in double.
uint64_t orc_render_pt(void *h, uint64_t w, uint64_t hh, uint64_t fov, const float *pos, const float *look,
                       const float *bg, uint32_t max_depth, uint32_t spp, uint64_t seed, float eps, int mode,
                       uint32_t rr_depth, uint64_t row0, uint64_t row1, uint8_t *out_rgb, float *out_rad,
                       int threads, uint32_t sample_offset, double *out_sum64) {
    auto &s = *static_cast<Scene *>(h);
    Camera c = make_camera(w, hh, fov, {pos[0], pos[1], pos[2]}, {look[0], look[1], look[2]});
    const Emitters em = collect_emitters(s);
    const V3 b{bg[0], bg[1], bg[2]};
    uint64_t segs = 0;
    const int64_t npx = (int64_t)((row1 - row0) * w);
    // pixels, not rows, are the unit of work, so that a band of a few rows
    // still keeps every thread busy
#pragma omp parallel for schedule(dynamic, 2) reduction(+ : segs) num_threads(threads > 0 ? threads : 1)
    for (int64_t k = 0; k < npx; k++) {
        note_threads();
        {
            const uint64_t py = row0 + (uint64_t)k / w, px = (uint64_t)k % w;
            const uint64_t pixel = py * w + px;
            const Ray prim = primary(c, px, py);
            V3 sum{0.f, 0.f, 0.f};
            const uint64_t o = (py - row0) * w + px;
            double *acc = out_sum64 ? out_sum64 + 3 * o : nullptr;
            if (mode == 2) {
                // branching mode: one tree per pixel, spp = bounce rays per hit (evaluatePath,
                // src/pray.cpp:366-378, returns the tree's value without a further average)
                pray_pcg32 g = pray_pcg32_stream(seed, pixel, sample_offset);
                sum = path_diffuse(s, prim, b, max_depth, spp, eps, g, segs, 0);
                if (acc) acc[0] += (double)sum.x, acc[1] += (double)sum.y, acc[2] += (double)sum.z;
            }
            for (uint32_t k = 0; k < (mode == 2 ? 0u : spp); k++) {
                pray_pcg32 g = pray_pcg32_stream(seed, pixel, sample_offset + k);
                const V3 L = mode == 0 ? path_kajiya(s, prim, b, max_depth, eps, g, segs)
                                       : path_nee(s, em, prim, b, max_depth, rr_depth, eps, g, segs);
                sum = add(sum, L);
                if (acc) acc[0] += (double)L.x, acc[1] += (double)L.y, acc[2] += (double)L.z;
            }
            const float ns = (float)spp;
            const V3 mean = mode == 2 ? sum : V3{sum.x / ns, sum.y / ns, sum.z / ns};
            if (out_rad) {
                out_rad[3 * o] = mean.x;
                out_rad[3 * o + 1] = mean.y;
                out_rad[3 * o + 2] = mean.z;
            }
            auto cl = [](float v) { return smax(0.f, smin(1.f, v)); };
            out_rgb[3 * o] = quantise(cl(mean.x));
            out_rgb[3 * o + 1] = quantise(cl(mean.y));
            out_rgb[3 * o + 2] = quantise(cl(mean.z));
        }
    }
    return segs;
}


void *orc_scene_new(const float *verts, const float *colors, const uint8_t *emit, uint64_t n) {
    auto *s = new Scene();
    s->tris.resize(n);
    for (uint64_t i = 0; i < n; i++) {
        const float *v = verts + 9 * i;
        Tri &t = s->tris[i];
        t.a = {v[0], v[1], v[2]};
        t.b = {v[3], v[4], v[5]};
        t.c = {v[6], v[7], v[8]};
        t.color = {colors[3 * i], colors[3 * i + 1], colors[3 * i + 2]};
        t.emit = emit ? emit[i] != 0 : false;
    }
    return s;
}

void orc_scene_free(void *h) { delete static_cast<Scene *>(h); }

// Precompute and build. kind 0 = median tree, 1 = SAH kd tree.
void orc_scene_build(void *h, int kind, int leaf_size, int max_depth, float ct, float ci) {
    auto &s = *static_cast<Scene *>(h);
    s.leaf_size = leaf_size;
    s.max_depth = max_depth;
    s.ct = ct;
    s.ci = ci;
    s.nodes.clear();
    for (Tri &t : s.tris) precompute(t);
    if (s.tris.empty()) {
        s.nodes.emplace_back();  // empty root, src/kd_tree.cpp:26-29
        s.nnodes = 1;
        return;
    }
    std::vector<int64_t> idx(s.tris.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (int64_t)i;
    if (kind == 0) {
        build_median(s, idx, 0);
    } else {
        Box root = s.tris[0].box;
        for (size_t i = 0; i < s.tris.size(); i++) root = expand(root, s.tris[i].box);
        std::vector<Event> ev;
        ev.reserve(s.tris.size() * 6);
        for (int64_t t : idx) gen_events(s, t, root, ev);
        std::sort(ev.begin(), ev.end());
        std::vector<int8_t> side(s.tris.size(), kBoth);
        build_sah(s, idx, root, ev, 255, 0.f, 0, side);
    }
    const Node &r = s.nodes[0];
    s.nnodes = r.sub_nodes + 1;
    s.leaf_nodes = r.sub_leaves;
    s.empty_leaves = r.sub_empty;
    s.maxdepth = r.depth_to_leaf;
}

void orc_triangle_precompute(void *h, float *out) {
    auto &s = *static_cast<Scene *>(h);
    for (size_t i = 0; i < s.tris.size(); i++) {
        const Tri &t = s.tris[i];
        const V3 *vs[6] = {&t.box.lo, &t.box.hi, &t.mid, &t.ab, &t.ac, &t.normal};
        for (int k = 0; k < 6; k++) {
            out[18 * i + 3 * k] = vs[k]->x;
            out[18 * i + 3 * k + 1] = vs[k]->y;
            out[18 * i + 3 * k + 2] = vs[k]->z;
        }
    }
}

// nnodes, maxdepth, leafNodes, emptyLeafNodes, total leaf references
void orc_tree_stats(void *h, uint64_t *out) {
    auto &s = *static_cast<Scene *>(h);
    uint64_t refs = 0;
    for (const Node &n : s.nodes) refs += n.tris.size();
    out[0] = s.nodes.size();
    out[1] = s.maxdepth;
    out[2] = s.leaf_nodes;
    out[3] = s.empty_leaves;
    out[4] = refs;
}

// Nodes are stored in DFS pre-order already (each build appends the node
// before its subtrees), matching ref_tree_dump's layout.
void orc_tree_dump(void *h, float *boxes, float *split, int32_t *info, int64_t *refs) {
    auto &s = *static_cast<Scene *>(h);
    int64_t r = 0;
    for (size_t i = 0; i < s.nodes.size(); i++) {
        const Node &n = s.nodes[i];
        float *b = boxes + 6 * i;
        b[0] = n.box.lo.x; b[1] = n.box.lo.y; b[2] = n.box.lo.z;
        b[3] = n.box.hi.x; b[4] = n.box.hi.y; b[5] = n.box.hi.z;
        split[i] = n.split;
        info[4 * i] = n.leaf() ? 1 : 0;
        info[4 * i + 1] = n.axis;
        info[4 * i + 2] = (int32_t)n.tris.size();
        info[4 * i + 3] = (int32_t)r;
        for (int64_t t : n.tris) refs[r++] = t;
    }
}

void orc_primary_rays(uint64_t w, uint64_t h, uint64_t fov, const float *pos, const float *look, float *out) {
    Camera c = make_camera(w, h, fov, {pos[0], pos[1], pos[2]}, {look[0], look[1], look[2]});
    for (uint64_t py = 0; py < h; py++)
        for (uint64_t px = 0; px < w; px++) {
            Ray r = primary(c, px, py);
            float *o = out + 9 * (py * w + px);
            o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z;
            o[3] = r.d.x; o[4] = r.d.y; o[5] = r.d.z;
            o[6] = r.inv.x; o[7] = r.inv.y; o[8] = r.inv.z;
        }
}

// Camera constants the GPU kernels are given: inverse view matrix rows 0-2
// (cols 0-2), inv_w, inv_h, aspect, angle.
void orc_camera(uint64_t w, uint64_t h, uint64_t fov, const float *pos, const float *look, float *out) {
    Camera c = make_camera(w, h, fov, {pos[0], pos[1], pos[2]}, {look[0], look[1], look[2]});
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[3 * i + j] = c.inv[i][j];
    out[9] = c.inv_w;
    out[10] = c.inv_h;
    out[11] = c.aspect;
    out[12] = c.angle;
}

void orc_trace(void *h, const float *rays, uint64_t n, float eps, int64_t *ids, float *ts, int threads) {
    auto &s = *static_cast<Scene *>(h);
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : 1)
    for (uint64_t i = 0; i < n; i++) {
        const float *r = rays + 9 * i;
        Ray ray{{r[0], r[1], r[2]}, {r[3], r[4], r[5]}, {r[6], r[7], r[8]}};
        int64_t id;
        float d;
        closest(s, ray, eps, id, d);
        ids[i] = id;
        ts[i] = d;
    }
}

// Ray-tracing render (src/pray.cpp:380-590 semantics) of the pixel rows
// [row0, row1). out holds width*(row1-row0)*3 bytes. Returns the number of
// shadow rays cast.
uint64_t orc_render_rt(void *h, uint64_t w, uint64_t hh, uint64_t fov, const float *pos, const float *look,
                       const float *lights, int n_lights, const float *bg, float eps, uint64_t row0,
                       uint64_t row1, uint8_t *out, int threads) {
    auto &s = *static_cast<Scene *>(h);
    Camera c = make_camera(w, hh, fov, {pos[0], pos[1], pos[2]}, {look[0], look[1], look[2]});
    std::vector<Light> ls(n_lights);
    for (int i = 0; i < n_lights; i++)
        ls[i] = {{lights[6 * i], lights[6 * i + 1], lights[6 * i + 2]},
                 {lights[6 * i + 3], lights[6 * i + 4], lights[6 * i + 5]}};
    V3 b{bg[0], bg[1], bg[2]};
    uint64_t shadows = 0;
    const bool empty = s.tris.empty();
    const int64_t npx = (int64_t)((row1 - row0) * w);
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : shadows) num_threads(threads > 0 ? threads : 1)
    for (int64_t k = 0; k < npx; k++) {
        note_threads();
        {
            const uint64_t py = row0 + (uint64_t)k / w, px = (uint64_t)k % w;
            V3 col = empty ? b : shade_rt(s, primary(c, px, py), ls, b, eps, shadows);
            uint8_t *o = out + 3 * ((py - row0) * w + px);
            o[0] = quantise(col.x);
            o[1] = quantise(col.y);
            o[2] = quantise(col.z);
        }
    }
    return shadows;
}

}  // extern "C"
