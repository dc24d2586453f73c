// Per-pixel path tracing shared by the per-pixel kernel (pt.cu) and the
// batched persistent kernel (batch.cu): one lane per pixel, the pixel's
// samples in order, each an iterative bounce loop; all lanes of a warp call
// these functions together (the traversals are warp-collective).
//
// Mode 0 restates the reference's Kajiya path tracer
// (evaluatePathRecursive, src/pray.cpp:342-364; evaluatePath,
// src/pray.cpp:366-378): a miss returns the background, an emitter returns its
// colour, a hit at depth >= max_depth returns black, otherwise one cosine
// bounce whose result is multiplied by the albedo. The recursion multiplies
// the deepest value first, so the albedos of a path are kept on a small
// per-lane stack and applied in that order. Random numbers come from one
// PCG32 stream per (seed, pixel, sample) (include/nostrum_pray_sampling.h).
//
// Mode 1 (no reference counterpart) adds next-event estimation to the
// emitting triangles (area-weighted choice, uniform point, one occlusion ray)
// and Russian roulette from rr_depth; emitters seen by a bounce ray end the
// path without adding their emission (next-event estimation accounts for it).
//
// Mode 2 (pt_pixel_diffuse below) is the reference's branching variant.
#pragma once

#include <cfloat>
#include <cstdint>

#include "../../include/nostrum_pray_sampling.h"
#include "device_layout.h"
#include "trace_launch.h"
#include "traverse.cuh"

namespace pray_gpu {
namespace dev {

constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kShadowShrink = 0.999f;  // next-event occlusion ends short of the light point

__device__ __forceinline__ float4 shade_n(const DevScene &s, int id) {
    return __ldg(reinterpret_cast<const float4 *>(s.shade[id].n));
}
__device__ __forceinline__ float4 shade_c(const DevScene &s, int id) {
    return __ldg(reinterpret_cast<const float4 *>(s.shade[id].c));
}

// Emitter index for a uniform u: first j with cdf[j] > u * total.
__device__ __forceinline__ uint32_t pick_emitter(const DevScene &s, float u) {
    const float target = u * s.emit_area;
    uint32_t lo = 0, hi = s.n_emit - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(s.emit_cdf + mid) > target) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Pixels a lane takes one after another: a warp-collective source. All lanes
// call take() together; a lane that asks (want) may receive a pixel.
// OnePixel hands each lane one fixed pixel.
struct OnePixel {
    bool active;
    uint32_t px, py;
    bool given;
    __device__ __forceinline__ bool drained() const { return given; }
    __device__ __forceinline__ bool take(bool want, uint32_t &x, uint32_t &y) {
        const bool got = want && !given && active;
        given = true;
        x = px, y = py;
        return got;
    }
};

// Modes 0 and 1 bounce by bounce: all lanes of a warp call pt_sync together
// and run each bounce's extension rays, then its next-event occlusion rays,
// as two warp-collective traversals. Each lane works through its pixel's
// samples in order and starts its next sample as soon as its current path
// ends (path regeneration); a lane whose pixel is done takes the next one
// from `src`, so it does not wait for the warp's longest path. The per-pixel
// sums still add the samples in sample order, so the result is unchanged.
// pixels counts the pixels a lane finished. The per-pixel kernel runs it for
// modes 0 and 1, the batch kernel for mode 1 (next-event occlusion rays, all
// aimed at the emitters, keep the warp more coherent traced together than
// mixed with bounce rays).
template <int kStackN, class Src>
__device__ __forceinline__ void pt_sync(const DevScene &s, const PtLaunch &L, Src &src, uint32_t &segments,
                                        uint32_t &pixels) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    float alb_r[kMaxPtDepth], alb_g[kMaxPtDepth], alb_b[kMaxPtDepth];
    const bool any_geometry = s.n_refs > 0;
    // the lane's pixel
    bool have = false;
    uint32_t px = 0, py = 0;
    auto pixel = [&]() { return (uint64_t)py * L.cam.width + px; };
    float sr = 0.f, sg = 0.f, sb = 0.f;
    double ax = 0, ay = 0, az = 0;
    // its current path
    uint32_t smp = 0;
    pray_pcg32 rng;
    RayF r{};
    float lr = 0.f, lg = 0.f, lb = 0.f;
    float tr = 1.f, tg = 1.f, tb = 1.f;
    uint32_t depth = 0;
    bool alive = false;
    auto start = [&]() {
        rng = pray_pcg32_stream(L.seed, pixel(), L.sample_offset + smp);
        r = primary_ray(L.cam, px, py);
        lr = lg = lb = 0.f;
        tr = tg = tb = 1.f;
        depth = 0;
        alive = true;
    };
    auto finish_pixel = [&]() {
        const uint64_t pix = pixel();
        if (L.sum64) L.sum64[3 * pix] = ax, L.sum64[3 * pix + 1] = ay, L.sum64[3 * pix + 2] = az;
        const float ns = (float)L.num_samples;
        const float mr = sr / ns, mg = sg / ns, mb = sb / ns;
        if (L.radiance) {
            float *o = L.radiance + 3 * pix;
            o[0] = mr, o[1] = mg, o[2] = mb;
        }
        if (L.rgb) {
            uint8_t *o = L.rgb + 3 * pix;
            o[0] = (uint8_t)quantise(smax(0.f, smin(1.f, mr)));
            o[1] = (uint8_t)quantise(smax(0.f, smin(1.f, mg)));
            o[2] = (uint8_t)quantise(smax(0.f, smin(1.f, mb)));
        }
        pixels++;
        have = false;
    };
    while (true) {
        const unsigned idle = __ballot_sync(kFull, !have);
        if (idle && !src.drained()) {
            uint32_t x, y;
            if (src.take(!have, x, y)) {
                have = true;
                px = x, py = y;
                smp = 0;
                sr = sg = sb = 0.f;
                ax = ay = az = 0;
                if (L.sum64) {
                    const uint64_t pix = pixel();
                    ax = L.sum64[3 * pix], ay = L.sum64[3 * pix + 1], az = L.sum64[3 * pix + 2];
                }
                start();
            }
        }
        // (a source may hand out slots outside the image: go on until it is drained)
        if (!__any_sync(kFull, alive) && src.drained()) break;
        const bool was_alive = alive;
        float t;
        const int pos = traverse<false, false, kStackN>(s, r, L.eps, 0.f, alive && any_geometry, t);
        // next-event occlusion job of this bounce (mode 1)
        bool need = false;
        RayF sray = r;
        float sd2 = 0.f, cxr = 0.f, cxg = 0.f, cxb = 0.f;
        float4 nrm = make_float4(0.f, 0.f, 0.f, 0.f), col = nrm;
        float hx = 0.f, hy = 0.f, hz = 0.f;
        if (alive) {
            segments++;
            if (pos < 0) {
                if (L.mode == 0) lr = L.bg[0], lg = L.bg[1], lb = L.bg[2];
                else lr = lr + tr * L.bg[0], lg = lg + tg * L.bg[1], lb = lb + tb * L.bg[2];
                alive = false;
            } else {
                const int id = (int)__float_as_uint(__ldg(&s.tris[pos].v0[3]));
                nrm = shade_n(s, id), col = shade_c(s, id);
                if (nrm.w != 0.f) {
                    if (L.mode == 0) lr = col.x, lg = col.y, lb = col.z;
                    else if (depth == 0) lr = lr + tr * col.x, lg = lg + tg * col.y, lb = lb + tb * col.z;
                    alive = false;
                } else if (depth >= L.max_depth) {
                    if (L.mode == 0) lr = 0.f, lg = 0.f, lb = 0.f;
                    alive = false;
                } else {
                    hx = r.ox + r.dx * t, hy = r.oy + r.dy * t, hz = r.oz + r.dz * t;
                    if (L.mode != 0 && s.n_emit > 0) {
                        const float ue = pray_uniform(&rng), ua = pray_uniform(&rng), ub = pray_uniform(&rng);
                        const GTri *E = s.emit_tris + pick_emitter(s, ue);
                        const float4 ev0 = __ldg(reinterpret_cast<const float4 *>(E->v0));
                        const float4 ee1 = __ldg(reinterpret_cast<const float4 *>(E->e1));
                        const float4 ee2 = __ldg(reinterpret_cast<const float4 *>(E->e2));
                        const float su = sqrtf(ua);
                        const float b1 = su * (1.f - ub), b2 = su * ub;
                        const float yx = ev0.x + ee1.x * b1 + ee2.x * b2;
                        const float yy = ev0.y + ee1.y * b1 + ee2.y * b2;
                        const float yz = ev0.z + ee1.z * b1 + ee2.z * b2;
                        float wx = yx - hx, wy = yy - hy, wz = yz - hz;
                        const float d2 = wx * wx + wy * wy + wz * wz;
                        if (d2 > 0.f) {
                            const float inv = 1.0f / sqrtf(d2);
                            wx *= inv, wy *= inv, wz *= inv;
                            const int eid = (int)__float_as_uint(ev0.w);
                            const float4 en = shade_n(s, eid), ec = shade_c(s, eid);
                            const float cx = nrm.x * wx + nrm.y * wy + nrm.z * wz;
                            const float cy = -(en.x * wx + en.y * wy + en.z * wz);
                            if (cx > 0.f && cy > 0.f) {
                                need = true;
                                sray = make_ray(hx, hy, hz, wx, wy, wz);
                                sd2 = d2 * kShadowShrink;
                                const float g = ((cx * cy) * s.emit_area) * kInvPi / d2;
                                cxr = ((tr * col.x) * ec.x) * g;
                                cxg = ((tg * col.y) * ec.y) * g;
                                cxb = ((tb * col.z) * ec.z) * g;
                            }
                        }
                    }
                }
            }
        }
        float dummy;
        const bool occluded = traverse<true, false, kStackN>(s, sray, L.eps, sd2, need, dummy) >= 0;
        if (need) {
            segments++;
            if (!occluded) lr = lr + cxr, lg = lg + cxg, lb = lb + cxb;
        }
        if (alive) {
            // cosine bounce (and, in mode 1, Russian roulette)
            if (L.mode == 0) alb_r[depth] = col.x, alb_g[depth] = col.y, alb_b[depth] = col.z;
            const float u1 = pray_uniform(&rng), u2 = pray_uniform(&rng);
            const float n3[3] = {nrm.x, nrm.y, nrm.z};
            float d[3];
            pray_sample_hemisphere(n3, u1, u2, d);
            r = make_ray(hx, hy, hz, d[0], d[1], d[2]);
            if (L.mode != 0) {
                tr = tr * col.x, tg = tg * col.y, tb = tb * col.z;
                if (depth >= L.rr_depth) {
                    const float q = smin(smax(smax(tr, tg), tb), 0.95f);
                    if (!(pray_uniform(&rng) < q)) alive = false;
                    else tr = tr / q, tg = tg / q, tb = tb / q;
                }
            }
            depth++;
        }
        if (was_alive && !alive) {
            // the path ended: its value joins the pixel's sums in sample order
            if (L.mode == 0) {
                while (depth > 0) {
                    depth--;
                    lr = lr * alb_r[depth], lg = lg * alb_g[depth], lb = lb * alb_b[depth];
                }
            }
            sr = sr + lr, sg = sg + lg, sb = sb + lb;
            if (L.sum64) ax = ax + (double)lr, ay = ay + (double)lg, az = az + (double)lb;
            if (++smp < L.num_samples) start();
            else finish_pixel();
        }
    }
}

// One fixed pixel per lane (active lanes).
template <int kStackN>
__device__ __forceinline__ void pt_pixel_sync(const DevScene &s, const PtLaunch &L, bool active, uint32_t px,
                                         uint32_t py, uint32_t &segments) {
    OnePixel src{active, px, py, false};
    uint32_t pixels = 0;
    pt_sync<kStackN>(s, L, src, segments, pixels);
}

// Mode 0 as a per-lane state machine (the batch kernel's: 355 against 296
// Msamples/s on the 64-scene batch). All lanes of a warp call pt_lanes
// together. Each lane holds one ray at a time, its path's current bounce, and
// the warp advances every lane's ray by one traversal round (trav_round); a
// lane whose ray is done shades the hit and starts its next ray before the
// next round (the next bounce, the pixel's next sample, or a new pixel from
// `src`), so lanes do not idle until the warp's slowest ray is done. Per lane
// the operations and their order are those of the recursion, and the
// per-pixel sums add the samples in sample order. pixels counts the pixels a
// lane finished.
template <int kStackN, class Src>
__device__ __forceinline__ void pt_lanes(const DevScene &s, const PtLaunch &L, Src &src, uint32_t &segments,
                                         uint32_t &pixels) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const bool any_geometry = s.n_refs > 0;
    float alb_r[kMaxPtDepth], alb_g[kMaxPtDepth], alb_b[kMaxPtDepth];
    // the lane's pixel (its FP64 sums, when kept, are updated in place after
    // each path)
    bool have = false;
    uint32_t px = 0, py = 0, smp = 0;
    float sr = 0.f, sg = 0.f, sb = 0.f;
    auto pixel = [&]() { return (uint64_t)py * L.cam.width + px; };
    // its current path and ray
    pray_pcg32 rng;
    uint32_t depth = 0;
    bool job = false;
    RayF r{};
    Trav T;
    TravStack<kStackN> S;
    T.have_node = T.have_leaf = false;
    T.best = -1;

    auto extend = [&](const RayF &ray) {
        r = ray;
        job = true;
        trav_start<kClosest>(s, r, 0.f, any_geometry, T);
    };
    auto start_sample = [&]() {
        rng = pray_pcg32_stream(L.seed, pixel(), L.sample_offset + smp);
        depth = 0;
        extend(primary_ray(L.cam, px, py));
    };
    // the path ended with value l: the albedos of its bounces are applied
    // deepest first, and it joins the pixel's sums in sample order
    auto end_path = [&](float lr, float lg, float lb) {
        job = false;
        while (depth > 0) {
            depth--;
            lr = lr * alb_r[depth], lg = lg * alb_g[depth], lb = lb * alb_b[depth];
        }
        sr = sr + lr, sg = sg + lg, sb = sb + lb;
        if (L.sum64) {
            double *a = L.sum64 + 3 * pixel();
            a[0] = a[0] + (double)lr, a[1] = a[1] + (double)lg, a[2] = a[2] + (double)lb;
        }
        if (++smp < L.num_samples) {
            start_sample();
            return;
        }
        const float ns = (float)L.num_samples;
        const float mr = sr / ns, mg = sg / ns, mb = sb / ns;
        if (L.radiance) {
            float *o = L.radiance + 3 * pixel();
            o[0] = mr, o[1] = mg, o[2] = mb;
        }
        if (L.rgb) {
            uint8_t *o = L.rgb + 3 * pixel();
            o[0] = (uint8_t)quantise(smax(0.f, smin(1.f, mr)));
            o[1] = (uint8_t)quantise(smax(0.f, smin(1.f, mg)));
            o[2] = (uint8_t)quantise(smax(0.f, smin(1.f, mb)));
        }
        pixels++;
        have = false;
    };
    // the ray is done: a miss returns the background, an emitter its colour,
    // a hit at max_depth black; any other hit bounces
    auto shade = [&]() {
        const int pos = T.best;
        if (pos < 0) {
            end_path(L.bg[0], L.bg[1], L.bg[2]);
            return;
        }
        const int id = (int)__float_as_uint(__ldg(&s.tris[pos].v0[3]));
        const float4 nrm = shade_n(s, id), col = shade_c(s, id);
        if (nrm.w != 0.f) {
            end_path(col.x, col.y, col.z);
            return;
        }
        if (depth >= L.max_depth) {
            end_path(0.f, 0.f, 0.f);
            return;
        }
        const float t = T.best_t;
        const float hx = r.ox + r.dx * t, hy = r.oy + r.dy * t, hz = r.oz + r.dz * t;
        alb_r[depth] = col.x, alb_g[depth] = col.y, alb_b[depth] = col.z;
        const float u1 = pray_uniform(&rng), u2 = pray_uniform(&rng);
        const float n3[3] = {nrm.x, nrm.y, nrm.z};
        float d[3];
        pray_sample_hemisphere(n3, u1, u2, d);
        depth++;
        extend(make_ray(hx, hy, hz, d[0], d[1], d[2]));
    };

    while (true) {
        const unsigned idle = __ballot_sync(kFull, !have);
        if (idle && !src.drained()) {
            uint32_t x, y;
            if (src.take(!have, x, y)) {
                have = true;
                px = x, py = y;
                smp = 0;
                sr = sg = sb = 0.f;
                start_sample();
            }
        }
        // (a source may hand out slots outside the image: go on until it is drained)
        if (!__any_sync(kFull, job) && src.drained()) break;
        trav_round<kClosest, false>(s, r, L.eps, 0.f, T, S, nullptr);
        if (job && !T.active()) {
            segments++;
            shade();
        }
    }
}

// Mode 2 restates the reference's branching recursion
// (evaluatePathRecursiveDiffuse, src/pray.cpp:315-340; its GPU twin
// src/path_trace.cu:369-393): a miss returns the background, an emitter its
// colour, a hit at depth >= max_depth black; any other hit casts num_samples
// cosine bounce rays one after another and returns (sum * albedo) /
// num_samples. The recursion is unrolled into a per-lane stack of frames (one
// per ancestor hit: position, normal, albedo, running sum, children done); a
// finished ray's value is folded into its parent frame, and every frame whose
// children are all done is folded into its own parent in turn. One PCG32
// stream per pixel (sample index sample_offset) supplies the two uniforms of
// each bounce in depth-first order. As in pt_pixel_sync, every lane of a warp
// iterates until the warp's last tree ends, so the traversals line up.
template <int kStackN>
__device__ __forceinline__ void pt_pixel_diffuse(const DevScene &s, const PtLaunch &L, bool active, uint32_t px,
                                                 uint32_t py, uint32_t &segments) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint64_t pixel = active ? (uint64_t)py * L.cam.width + px : 0;
    RayF r = primary_ray(L.cam, active ? px : 0, active ? py : 0);
    pray_pcg32 rng = pray_pcg32_stream(L.seed, pixel, L.sample_offset);
    float fpos[kMaxDiffuseDepth][3], fnrm[kMaxDiffuseDepth][3], falb[kMaxDiffuseDepth][3],
        fsum[kMaxDiffuseDepth][3];
    uint32_t fdone[kMaxDiffuseDepth];
    uint32_t top = 0;  // frames on the stack = depth of the ray in flight
    float res0 = 0.f, res1 = 0.f, res2 = 0.f;
    bool alive = active;
    const bool any_geometry = s.n_refs > 0;
    const float nf = (float)L.num_samples;
    while (__any_sync(kFull, alive)) {
        float t;
        const int pos = traverse<false, false, kStackN>(s, r, L.eps, 0.f, alive && any_geometry, t);
        if (alive) {
            segments++;
            bool ends = true;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f;
            if (pos < 0) {
                v0 = L.bg[0], v1 = L.bg[1], v2 = L.bg[2];
            } else {
                const int id = (int)__float_as_uint(__ldg(&s.tris[pos].v0[3]));
                const float4 nrm = shade_n(s, id), col = shade_c(s, id);
                if (nrm.w != 0.f) {
                    v0 = col.x, v1 = col.y, v2 = col.z;
                } else if (top < L.max_depth) {
                    fpos[top][0] = r.ox + r.dx * t, fpos[top][1] = r.oy + r.dy * t, fpos[top][2] = r.oz + r.dz * t;
                    fnrm[top][0] = nrm.x, fnrm[top][1] = nrm.y, fnrm[top][2] = nrm.z;
                    falb[top][0] = col.x, falb[top][1] = col.y, falb[top][2] = col.z;
                    fsum[top][0] = 0.f, fsum[top][1] = 0.f, fsum[top][2] = 0.f;
                    fdone[top] = 0;
                    top++;
                    ends = false;
                }
            }
            while (ends) {
                if (top == 0) {
                    res0 = v0, res1 = v1, res2 = v2;
                    alive = false;
                    break;
                }
                const uint32_t k = top - 1;
                fsum[k][0] = fsum[k][0] + v0, fsum[k][1] = fsum[k][1] + v1, fsum[k][2] = fsum[k][2] + v2;
                if (++fdone[k] < L.num_samples) break;
                v0 = (fsum[k][0] * falb[k][0]) / nf;
                v1 = (fsum[k][1] * falb[k][1]) / nf;
                v2 = (fsum[k][2] * falb[k][2]) / nf;
                top = k;
            }
            if (alive) {
                const uint32_t k = top - 1;
                const float u1 = pray_uniform(&rng), u2 = pray_uniform(&rng);
                float d[3];
                pray_sample_hemisphere(fnrm[k], u1, u2, d);
                r = make_ray(fpos[k][0], fpos[k][1], fpos[k][2], d[0], d[1], d[2]);
            }
        }
    }
    if (active) {
        if (L.radiance) {
            float *o = L.radiance + 3 * pixel;
            o[0] = res0, o[1] = res1, o[2] = res2;
        }
        if (L.rgb) {
            uint8_t *o = L.rgb + 3 * pixel;
            o[0] = (uint8_t)quantise(smax(0.f, smin(1.f, res0)));
            o[1] = (uint8_t)quantise(smax(0.f, smin(1.f, res1)));
            o[2] = (uint8_t)quantise(smax(0.f, smin(1.f, res2)));
        }
    }
}

// Warp-aggregated [paths, segments] into counters (all lanes call).
__device__ __forceinline__ void count_paths(unsigned long long *counters, bool active, uint32_t num_samples,
                                            uint32_t segments) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t paths = __popc(__ballot_sync(kFull, active)) * num_samples;
    for (int o = 16; o > 0; o >>= 1) segments += __shfl_xor_sync(kFull, segments, o);
    if ((threadIdx.x & 31) == 0 && counters) {
        atomicAdd(counters + 0, (unsigned long long)paths);
        atomicAdd(counters + 1, (unsigned long long)segments);
    }
}

}  // namespace dev
}  // namespace pray_gpu
