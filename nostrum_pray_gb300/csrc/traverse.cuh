// Device-side ray traversal and intersection shared by the tracing kernels.
//
// Every translation unit that includes this file is built with --fmad=false
// and IEEE division / square root, so each float operation rounds as in the
// reference's scalar build compiled without FMA contraction.
//
// Traversal: one ray per thread, iterative, with a short per-thread stack.
// Both children of a node are fetched together (one 64-byte pair) and tested
// with the reference's infinite-line slab test (BoundingBox::intersect,
// include/geometry.h:151-164); the nearer is entered first and the farther
// pushed. Instead of the reference's visit-everything depth-first order
// (KDTree::intersectRecursive, src/kd_tree.cpp:237-279), boxes that start
// beyond the best hit found so far are skipped: the result is the
// lexicographic minimum of (distance, depth-first reference position) over
// the references the reference itself tests, which is exactly the triangle
// it returns. The skip bounds keep a relative margin (kPruneRel) and an
// absolute margin (DevScene::tol) so that rounding in a box's entry or exit
// distance never drops a box holding the winning triangle.
#pragma once

#include <cfloat>
#include <cstdint>

#include "device_layout.h"
#include "host/camera.h"

namespace pray_gpu {
namespace dev {

constexpr float kPruneRel = 1.0f + 1.0f / 4096.0f;
constexpr int kStack = 64;
static_assert(kStack > kMaxTraversalDepth, "stack must hold a full root-to-leaf path");

struct RayF {
    float ox, oy, oz;
    float dx, dy, dz;
    float ix, iy, iz;
};

__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// Ray ctor of include/geometry.h:82-87: normalise, then 1/direction.
__device__ __forceinline__ RayF make_ray(float ox, float oy, float oz, float dx, float dy, float dz) {
    RayF r;
    r.ox = ox, r.oy = oy, r.oz = oz;
    const float n2 = dx * dx + dy * dy + dz * dz;
    if (n2 > 0) {
        const float inv = 1.0f / sqrtf(n2);
        dx *= inv, dy *= inv, dz *= inv;
    }
    r.dx = dx, r.dy = dy, r.dz = dz;
    r.ix = 1.0f / dx, r.iy = 1.0f / dy, r.iz = 1.0f / dz;
    return r;
}

// Three-input minimum / maximum (one instruction on sm_100 and later). Like
// fminf / fmaxf, a NaN operand is ignored unless all are NaN.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// BoundingBox::intersect, include/geometry.h:151-164. `finite`: all three
// inverse direction components are finite, so no slab value can be NaN; then
// fminf/fmaxf return the same values as the reference's std::min/std::max
// selects (they can differ only in the sign of a zero, which no comparison
// sees), at one instruction each. Otherwise the select form reproduces the
// reference's NaN behaviour.
__device__ __forceinline__ bool slab(const float4 &lo, const float4 &hi, const RayF &r, bool finite, float &tn,
                                     float &tf) {
    const float t1x = (lo.x - r.ox) * r.ix, t2x = (hi.x - r.ox) * r.ix;
    const float t1y = (lo.y - r.oy) * r.iy, t2y = (hi.y - r.oy) * r.iy;
    const float t1z = (lo.z - r.oz) * r.iz, t2z = (hi.z - r.oz) * r.iz;
    if (finite) {
        // the same values as fmaxf(fmaxf(a, b), fmaxf(c, -FLT_MAX)) and its mirror
        tn = max3f(fminf(t1x, t2x), fminf(t1y, t2y), fmaxf(fminf(t1z, t2z), -FLT_MAX));
        tf = min3f(fmaxf(t1x, t2x), fmaxf(t1y, t2y), fminf(fmaxf(t1z, t2z), FLT_MAX));
    } else {
        tn = smax(smax(smin(t1x, t2x), smin(t1y, t2y)), smax(smin(t1z, t2z), -FLT_MAX));
        tf = smin(smin(smax(t1x, t2x), smax(t1y, t2y)), smin(smax(t1z, t2z), FLT_MAX));
    }
    return tn <= tf;
}

__device__ __forceinline__ bool slab(const float4 &lo, const float4 &hi, const RayF &r, float &tn, float &tf) {
    return slab(lo, hi, r, false, tn, tf);
}

// The slab test on the culling copy's padded boxes as one FMA per plane:
// (p - o) * inv computed as p * inv + (-o * inv), with no = -o * inv rounded
// once per ray (finite: the caller checks). Its error against the exact
// plane distance is below 2^-24 (2 |o| + |p|) |inv| per axis. The padding
// of a culling box moves each plane by at least 2^-16 (|p| + D) (D the
// scene's diagonal) and culling origins lie within 4 D of the scene's
// centre, so |o| < |p| + 4.5 D and the error is below 1/25 of the pad, on
// entry and exit alike: the pad still holds the triangle hits it was sized
// for (host/flatten.cpp), so no box that the exact ray crosses around a hit
// fails the test or the pruning bound.
//
// Entry and exit take the three-input min / max and drop the reference's clamps to
// -FLT_MAX / FLT_MAX: with a finite inverse direction and finite o * inv no
// plane distance of a finite box is NaN, so the clamps change only an
// infinite entry or exit into FLT_MAX, which no comparison here sees. Boxes of
// empty leaves (infinite or NaN coordinates, no triangles) may then fail where
// they passed before, which drops no triangle.
__device__ __forceinline__ bool slab_fma(const float4 &lo, const float4 &hi, const RayF &r, float nox, float noy,
                                         float noz, float &tn, float &tf) {
    const float t1x = fmaf(lo.x, r.ix, nox), t2x = fmaf(hi.x, r.ix, nox);
    const float t1y = fmaf(lo.y, r.iy, noy), t2y = fmaf(hi.y, r.iy, noy);
    const float t1z = fmaf(lo.z, r.iz, noz), t2z = fmaf(hi.z, r.iz, noz);
    tn = max3f(fminf(t1x, t2x), fminf(t1y, t2y), fminf(t1z, t2z));
    tf = min3f(fmaxf(t1x, t2x), fmaxf(t1y, t2y), fmaxf(t1z, t2z));
    return tn <= tf;
}

// One-sided Moeller-Trumbore, include/geometry.h:242-262, with the det
// threshold as a parameter (the reference's EPSILON is 1e-4).
__device__ __forceinline__ bool intersect_tri(const float4 &v0, const float4 &e1, const float4 &e2, const RayF &r,
                                              float eps, float &t) {
    const float px = r.dy * e2.z - r.dz * e2.y;
    const float py = r.dz * e2.x - r.dx * e2.z;
    const float pz = r.dx * e2.y - r.dy * e2.x;
    const float det = e1.x * px + e1.y * py + e1.z * pz;
    if (det < eps) return false;
    const float tx = r.ox - v0.x, ty = r.oy - v0.y, tz = r.oz - v0.z;
    const float un = tx * px + ty * py + tz * pz;
    // Early out before the division, only where the reference's
    // u = un * (1 / det) is certainly < 0 or > 1: un below -2^-125.6 * det
    // keeps the product a negative normal number; un above det * (1 + 2^-20)
    // keeps it above 1 whatever the two roundings.
    if (un < -(det * 2.4e-38f) || un > det * 1.00000095367431640625f) return false;
    const float inv = 1.0f / det;
    const float u = un * inv;
    if (u < 0.f || u > 1.f) return false;
    const float qx = ty * e1.z - tz * e1.y;
    const float qy = tz * e1.x - tx * e1.z;
    const float qz = tx * e1.y - ty * e1.x;
    const float v = (r.dx * qx + r.dy * qy + r.dz * qz) * inv;
    if (v < 0.f || u + v > 1.f) return false;
    t = (e2.x * qx + e2.y * qy + e2.z * qz) * inv;
    return true;
}

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

// One node (box lo + payload a, box hi + payload b) in one 256-bit read-only
// load: nodes are 32-byte aligned, so a lane's node is one 32-byte sector and
// one load instruction instead of two 16-byte ones (half the L1 wavefronts
// of the incoherent per-lane walks, half the load instructions of the packet
// walk).
__device__ __forceinline__ void ldg_node(const GNode *n, float4 &lo, float4 &hi) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z), "=f"(hi.w)
        : "l"(n));
}

// Closest hit (kAny = false): returns the reference position of the winning
// triangle or -1, and its distance in t.
// Any hit (kAny = true): returns >= 0 as soon as a triangle with t > 0 and
// t * t < d2 is found (the occlusion test of src/pray.cpp:42).
// Fetch counts of one traversal (only maintained when kCount is set).
struct FetchCount {
    uint32_t pairs = 0, tris = 0;
};

// Pops the next stacked node that can still hold a closer hit.
__device__ __forceinline__ bool pop_node(const uint32_t *stk_a, const uint32_t *stk_b, const float *stk_t, int &sp,
                                         float limit, uint32_t &a, uint32_t &b, float &tn) {
    while (sp > 0) {
        sp--;
        if (stk_t[sp] <= limit) {
            a = stk_a[sp];
            b = stk_b[sp];
            tn = stk_t[sp];
            return true;
        }
    }
    return false;
}

// Warp-collective traversal: every lane of the warp must call it together
// (inactive lanes pass valid = false). Structure after Aila & Laine,
// "Understanding the Efficiency of Ray Traversal on GPUs" (HPG 2009): the
// warp first walks interior nodes until every lane holds a leaf ("postponing"
// the first leaf it meets and speculatively continuing), then intersects the
// postponed leaves together, so lanes do the same kind of work at the same
// time.
//
// The per-lane state lives in Trav, so that a kernel can also run the
// traversal round by round and hand a lane whose ray is done a new ray
// (dynamic fetch): trav_start tests the root, trav_round runs one interior
// phase and one leaf phase for the whole warp, and a lane is done when
// active() turns false.
//
// Closest hit: best = index of the winning triangle record or -1, its
// distance in best_t. Any hit: best >= 0 once a triangle with t > 0 and
// t * t < d2 is found (the occlusion test of src/pray.cpp:42). A traversal
// looks for one or the other for the whole warp (kClosest, kAnyHit), or per
// lane as Trav::any says (kPerLane: a warp mixing extension and occlusion
// rays).
enum TravMode { kClosest = 0, kAnyHit = 1, kPerLane = 2 };

struct Trav {
    uint32_t a, b, la, lb;
    uint32_t node_off;  // 0: the exact copy; n_nodes: the culling copy (finite inverse direction, near origin)
    float cur_tn, leaf_tn, limit, back, best_t;
    int best, sp;
    uint32_t best_key;
    bool have_node, have_leaf, finite, any;
    __device__ __forceinline__ bool active() const { return have_node || have_leaf; }
};

// The traversal stack of one lane (kept apart from Trav so that the scalar
// state stays in registers).
template <int kStackN>
struct TravStack {
    uint32_t a[kStackN], b[kStackN];
    float t[kStackN];
};

// `any` (kPerLane only): this lane's ray looks for any occluder.
template <int kMode>
__device__ __forceinline__ void trav_start(const DevScene &s, const RayF &r, float d2, bool valid, Trav &T,
                                           bool any = false) {
    T.any = kMode == kAnyHit || (kMode == kPerLane && any);
    T.best_t = FLT_MAX;
    T.best = -1;
    T.best_key = 0xFFFFFFFFu;
    T.limit = T.any ? sqrtf(d2) * kPruneRel : FLT_MAX;
    T.back = -s.tol;
    T.a = T.b = T.la = T.lb = 0;
    T.cur_tn = T.leaf_tn = 0.f;
    T.have_node = T.have_leaf = false;
    T.sp = 0;
    T.finite = isfinite(r.ix) && isfinite(r.iy) && isfinite(r.iz);
    const float cx = r.ox - s.cull_c[0], cy = r.oy - s.cull_c[1], cz = r.oz - s.cull_c[2];
    T.node_off = (T.finite && cx * cx + cy * cy + cz * cz <= s.cull_r2) ? s.n_nodes : 0u;
    if (valid) {
        float tn, tf;
        const GNode *root = s.nodes + T.node_off;
        float4 rlo, rhi;
        ldg_node(root, rlo, rhi);
        if (slab(rlo, rhi, r, tn, tf)) {
            T.a = __float_as_uint(rlo.w);
            T.b = __float_as_uint(rhi.w);
            T.cur_tn = tn;
            T.have_node = true;
        }
    }
}

template <int kMode, bool kCount, int kStackN>
__device__ __forceinline__ void trav_round(const DevScene &s, const RayF &r, float eps, float d2, Trav &T,
                                           TravStack<kStackN> &S, FetchCount *fc) {
    static_assert(kStackN >= 2 && kStackN <= kStack, "stack entries");
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const bool any_hit = kMode == kAnyHit || (kMode == kPerLane && T.any);
    // 1. interior nodes, until every lane has found a leaf
    while (true) {
        const bool interior = T.have_node && !(T.b & kLeafFlag);
        if (!__any_sync(kFull, interior && !T.have_leaf)) break;
        if (interior) {
            if (kCount) fc->pairs++;
            // culling copy: boxes around the triangles (same topology; the
            // reference's leaf boxes decide which leaves count)
            const GNode *c = s.nodes + (T.a + T.node_off);
            float4 l0, h0, l1, h1;
            ldg_node(c, l0, h0);
            ldg_node(c + 1, l1, h1);
            float tn0, tf0, tn1, tf1;
            const bool v0 = slab(l0, h0, r, T.finite, tn0, tf0) && tn0 <= T.limit && tf0 >= T.back;
            const bool v1 = slab(l1, h1, r, T.finite, tn1, tf1) && tn1 <= T.limit && tf1 >= T.back;
            if (v0 && v1) {
                const bool first0 = tn0 <= tn1;
                S.a[T.sp] = __float_as_uint(first0 ? l1.w : l0.w);
                S.b[T.sp] = __float_as_uint(first0 ? h1.w : h0.w);
                S.t[T.sp] = first0 ? tn1 : tn0;
                T.sp++;
                T.a = __float_as_uint(first0 ? l0.w : l1.w);
                T.b = __float_as_uint(first0 ? h0.w : h1.w);
                T.cur_tn = first0 ? tn0 : tn1;
            } else if (v0 || v1) {
                T.a = __float_as_uint(v0 ? l0.w : l1.w);
                T.b = __float_as_uint(v0 ? h0.w : h1.w);
                T.cur_tn = v0 ? tn0 : tn1;
            } else {
                T.have_node = pop_node(S.a, S.b, S.t, T.sp, T.limit, T.a, T.b, T.cur_tn);
            }
            if (T.have_node && (T.b & kLeafFlag) && !T.have_leaf) {
                // first leaf: postpone it and keep walking
                T.la = T.a, T.lb = T.b, T.leaf_tn = T.cur_tn;
                T.have_leaf = true;
                T.have_node = pop_node(S.a, S.b, S.t, T.sp, T.limit, T.a, T.b, T.cur_tn);
            }
        }
    }
    // 2. leaves: the postponed one, then any leaf the walk stopped on
    while (true) {
        const bool work = T.have_leaf || (T.have_node && (T.b & kLeafFlag));
        if (!__any_sync(kFull, work)) break;
        if (work) {
            uint32_t fa, fb;
            float ftn;
            if (T.have_leaf) {
                fa = T.la, fb = T.lb, ftn = T.leaf_tn;
                T.have_leaf = false;
            } else {
                fa = T.a, fb = T.b, ftn = T.cur_tn;
                T.have_node = pop_node(S.a, S.b, S.t, T.sp, T.limit, T.a, T.b, T.cur_tn);
            }
            if (ftn <= T.limit) {
                const uint32_t end = fa + (fb & ~kLeafFlag);
                for (uint32_t i = fa; i < end; i++) {
                    if (kCount) fc->tris++;
                    const GTri *Tr = s.tris + i;
                    const float4 v0 = ldg4(Tr->v0), e1 = ldg4(Tr->e1), e2 = ldg4(Tr->e2);
                    float t;
                    if (intersect_tri(v0, e1, e2, r, eps, t) && t > 0) {
                        if (any_hit) {
                            if (d2 > t * t) {
                                T.best = (int)i;
                                T.have_node = T.have_leaf = false;
                                T.sp = 0;
                                break;
                            }
                        } else {
                            // depth-first position in the reference's leaf order
                            const uint32_t key = __float_as_uint(e1.w);
                            if (t < T.best_t || (T.best >= 0 && t == T.best_t && key < T.best_key)) {
                                T.best_t = t;
                                T.best = (int)i;
                                T.best_key = key;
                                T.limit = t * kPruneRel;
                            }
                        }
                    }
                }
            }
        }
    }
}

template <bool kAny, bool kCount = false, int kStackN = kStack>
__device__ __forceinline__ int traverse(const DevScene &s, const RayF &r, float eps, float d2, bool valid,
                                        float &best_t, FetchCount *fc = nullptr) {
    constexpr int kMode = kAny ? kAnyHit : kClosest;
    Trav T;
    TravStack<kStackN> S;
    trav_start<kMode>(s, r, d2, valid, T);
    while (__any_sync(0xFFFFFFFFu, T.active())) trav_round<kMode, kCount>(s, r, eps, d2, T, S, fc);
    best_t = T.best_t;
    return T.best;
}

// Warp-packet traversal for coherent rays (the primary and occlusion rays of
// a pixel tile), after the packet traversals of Wald et al. (EG 2001) and
// Garanzha & Loop (2010): the warp walks one node sequence of the culling
// copy with a mask of the lanes whose own box tests passed, so node and
// triangle loads are warp-uniform (one broadcast each) and the traversal
// stack is one shared stack per warp (`stk`: 3 x kStackN words of shared
// memory: node payload, lane mask) instead of one per lane. Every lane still
// applies its own slab test (with its own pruning bound) to every box on its
// way and its own triangle test to every reference of the leaves it reaches,
// so it returns the same lexicographic minimum as traverse(); only the order
// of visits differs (the warp enters first the child that is nearer for most
// of the lanes entering both), and a lane whose bound shrank after a node was
// pushed still visits it (testing a popped node's box again measured slower:
// 2,571 against 2,682 Mrays/s on the 1.31M sphere). Box tests run in FMA
// form (slab_fma). Only for warps whose valid lanes all use the culling
// copy.
template <bool kAny, bool kCount, int kStackN>
__device__ __forceinline__ int traverse_packet(const DevScene &s, const RayF &r, float eps, float d2, bool valid,
                                               float &best_t, uint32_t *stk, FetchCount *fc) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const GNode *nodes = s.nodes + s.n_nodes;
    const float nox = -(r.ox * r.ix), noy = -(r.oy * r.iy), noz = -(r.oz * r.iz);
    float limit = kAny ? sqrtf(d2) * kPruneRel : FLT_MAX;
    const float back = -s.tol;
    best_t = FLT_MAX;
    int best = -1;
    uint32_t best_key = 0xFFFFFFFFu;
    uint32_t a, b;
    unsigned mask;
    {
        float4 lo, hi;
        ldg_node(nodes, lo, hi);
        float tn, tf;
        mask = __ballot_sync(kFull, valid && slab_fma(lo, hi, r, nox, noy, noz, tn, tf));
        a = __float_as_uint(lo.w);
        b = __float_as_uint(hi.w);
    }
    int sp = 0;
    while (mask) {
        const bool in = (mask >> lane) & 1u;
        if (!(b & kLeafFlag)) {
            const GNode *c = nodes + a;
            float4 l0, h0, l1, h1;
            ldg_node(c, l0, h0);
            ldg_node(c + 1, l1, h1);
            if (kCount && in) fc->pairs++;
            float tn0, tf0, tn1, tf1;
            const bool v0 = in && slab_fma(l0, h0, r, nox, noy, noz, tn0, tf0) && tn0 <= limit && tf0 >= back;
            const bool v1 = in && slab_fma(l1, h1, r, nox, noy, noz, tn1, tf1) && tn1 <= limit && tf1 >= back;
            const unsigned m0 = __ballot_sync(kFull, v0), m1 = __ballot_sync(kFull, v1);
            if (m0 && m1) {
                const unsigned both = m0 & m1;
                const unsigned near0 = __ballot_sync(kFull, v0 && v1 && tn0 <= tn1);
                const bool go0 = both ? 2 * __popc(near0) >= __popc(both) : __popc(m0) >= __popc(m1);
                if (lane == 0) {
                    stk[sp] = __float_as_uint(go0 ? l1.w : l0.w);
                    stk[kStackN + sp] = __float_as_uint(go0 ? h1.w : h0.w);
                    stk[2 * kStackN + sp] = go0 ? m1 : m0;
                }
                sp++;
                a = __float_as_uint(go0 ? l0.w : l1.w);
                b = __float_as_uint(go0 ? h0.w : h1.w);
                mask = go0 ? m0 : m1;
                continue;
            }
            if (m0 | m1) {
                a = __float_as_uint(m0 ? l0.w : l1.w);
                b = __float_as_uint(m0 ? h0.w : h1.w);
                mask = m0 | m1;
                continue;
            }
        } else {
            // the lanes in the mask test the leaf's references
            bool open = in;
            const uint32_t end = a + (b & ~kLeafFlag);
            for (uint32_t i = a; i < end; i++) {
                const GTri *Tr = s.tris + i;
                const float4 v0 = ldg4(Tr->v0), e1 = ldg4(Tr->e1), e2 = ldg4(Tr->e2);
                if (open) {
                    if (kCount) fc->tris++;
                    float t;
                    if (intersect_tri(v0, e1, e2, r, eps, t) && t > 0) {
                        if (kAny) {
                            if (d2 > t * t) {
                                best = (int)i;
                                open = false;
                            }
                        } else {
                            const uint32_t key = __float_as_uint(e1.w);
                            if (t < best_t || (best >= 0 && t == best_t && key < best_key)) {
                                best_t = t;
                                best = (int)i;
                                best_key = key;
                                limit = t * kPruneRel;
                            }
                        }
                    }
                }
                if (kAny && !__any_sync(kFull, open)) break;
            }
        }
        // next node: the top of the stack, without the lanes already done
        const unsigned done = kAny ? __ballot_sync(kFull, best >= 0) : 0u;
        mask = 0;
        __syncwarp();
        while (sp > 0 && !mask) {
            sp--;
            a = stk[sp];
            b = stk[kStackN + sp];
            mask = stk[2 * kStackN + sp] & ~done;
        }
        __syncwarp();
    }
    return best;
}

// traverse_packet where every valid lane of the warp uses the culling copy
// (and has a finite o * inv on every axis), else traverse(); all lanes of
// the warp call it together.
template <bool kAny, bool kCount, int kStackN>
__device__ __forceinline__ int traverse_coherent(const DevScene &s, const RayF &r, float eps, float d2, bool valid,
                                                 float &best_t, uint32_t *stk, FetchCount *fc = nullptr) {
    // the packet's FMA slab test also needs o * inv finite
    const bool finite = isfinite(r.ix) && isfinite(r.iy) && isfinite(r.iz) && isfinite(r.ox * r.ix) &&
                        isfinite(r.oy * r.iy) && isfinite(r.oz * r.iz);
    const float cx = r.ox - s.cull_c[0], cy = r.oy - s.cull_c[1], cz = r.oz - s.cull_c[2];
    const bool cull = finite && cx * cx + cy * cy + cz * cz <= s.cull_r2;
    if (__all_sync(0xFFFFFFFFu, !valid || cull))
        return traverse_packet<kAny, kCount, kStackN>(s, r, eps, d2, valid, best_t, stk, fc);
    return traverse<kAny, kCount, kStackN>(s, r, eps, d2, valid, best_t, fc);
}

// Primary ray of pixel (px, py), src/scene_preprocessor.cpp:124-134.
__device__ __forceinline__ RayF primary_ray(const CameraConsts &c, uint32_t px, uint32_t py) {
    const float x = (2 * (((float)px + 0.5f) * c.inv_w) - 1) * c.angle;
    const float y = (1 - 2 * (((float)py + 0.5f) * c.inv_h)) * c.angle / c.aspect;
    const float dx = x * c.m[0][0] + y * c.m[1][0] + c.m[2][0];
    const float dy = x * c.m[0][1] + y * c.m[1][1] + c.m[2][1];
    const float dz = x * c.m[0][2] + y * c.m[1][2] + c.m[2][2];
    return make_ray(c.pos[0], c.pos[1], c.pos[2], dx, dy, dz);
}

// static_cast<uint8_t>(v * 255 + 0.5) on the reference's targets: truncate to
// int, keep the low byte.
__device__ __forceinline__ uint32_t quantise(float v) { return (uint32_t)(int32_t)(v * 255.f + 0.5f) & 0xFFu; }

// Pixel index of thread i: warps cover kWarpTileW x kWarpTileH pixel tiles,
// tiles row-major.
constexpr uint32_t kWarpTileW = 8, kWarpTileH = 4;
static_assert(kWarpTileW * kWarpTileH == 32, "a warp tile holds 32 pixels");

__host__ __device__ __forceinline__ uint64_t warp_tiles(uint32_t w, uint32_t h) {
    return (uint64_t)((w + kWarpTileW - 1) / kWarpTileW) * ((h + kWarpTileH - 1) / kWarpTileH);
}

__device__ __forceinline__ bool pixel_of(uint64_t i, uint32_t w, uint32_t h, uint32_t &px, uint32_t &py) {
    const uint32_t tiles_x = (w + kWarpTileW - 1) / kWarpTileW;
    const uint64_t tile = i >> 5;
    const uint32_t lane = (uint32_t)i & 31u;
    px = (uint32_t)(tile % tiles_x) * kWarpTileW + lane % kWarpTileW;
    py = (uint32_t)(tile / tiles_x) * kWarpTileH + lane / kWarpTileW;
    return px < w && py < h;
}

}  // namespace dev
}  // namespace pray_gpu
