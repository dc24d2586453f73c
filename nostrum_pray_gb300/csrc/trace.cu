// Closest-hit tracing of caller-given rays and the fused ray-traced render
// (primary ray, closest hit, Lambert shading with one occlusion ray per
// light, quantisation). Traversal and intersection: traverse.cuh.
#include <cfloat>
#include <cstdint>
#include <type_traits>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "device_layout.h"
#include "trace_launch.h"
#include "traverse.cuh"

namespace pray_gpu {

namespace {

using namespace dev;

// Occlusion of caller-given rays: 1 iff some triangle is hit at t > 0 with
// t^2 < dist2 (the any-hit walk stops at the first such triangle). The
// reference asks for the closest hit and tests lightDistSq > dst * dst
// (src/pray.cpp:39-43); the closest t satisfies it iff some t does.
template <int kStackN>
__global__ void __launch_bounds__(128) k_trace_occluded(DevScene s, const float *__restrict__ rays,
                                                        const float *__restrict__ dist2, uint64_t n, float eps,
                                                        uint8_t *__restrict__ occluded) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    RayF r{};
    float d2 = 0.f;
    if (valid) {
        const float *p = rays + 9 * i;
        r.ox = p[0], r.oy = p[1], r.oz = p[2];
        r.dx = p[3], r.dy = p[4], r.dz = p[5];
        r.ix = p[6], r.iy = p[7], r.iz = p[8];
        d2 = dist2[i];
    }
    float t;
    const int pos = traverse<true, false, kStackN>(s, r, eps, d2, valid && s.n_refs > 0 && d2 > 0.f, t);
    if (valid) occluded[i] = pos >= 0 ? 1 : 0;
}

template <int kStackN>
__global__ void __launch_bounds__(128) k_trace_closest(DevScene s, const float *__restrict__ rays, uint64_t n,
                                                       float eps, int32_t *__restrict__ ids,
                                                       float *__restrict__ ts) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    RayF r{};
    if (valid) {
        const float *p = rays + 9 * i;
        r.ox = p[0], r.oy = p[1], r.oz = p[2];
        r.dx = p[3], r.dy = p[4], r.dz = p[5];
        r.ix = p[6], r.iy = p[7], r.iz = p[8];
    }
    float t;
    const int pos = traverse<false, false, kStackN>(s, r, eps, 0.f, valid && s.n_refs > 0, t);
    if (valid) {
        ids[i] = pos >= 0 ? (int32_t)__float_as_uint(__ldg(&s.tris[pos].v0[3])) : -1;
        ts[i] = t;
    }
}

// Fused ray-tracing render: primary ray, closest hit, per-light Lambert with
// an occlusion ray, clamp and quantise (evaluateRay, src/pray.cpp:17-55, and
// the quantisation of src/pray.cpp:576-588). Every lane of a warp runs the
// same light loop so that the warp-collective traversals line up; a lane
// whose colour saturated stops casting (the reference's early break).
// kPrimPacket / kShadowPacket: the warp traverses its tile's primary /
// occlusion rays as a packet (traverse_coherent).
// Resident blocks per SM (the register cap): the all-packet walk (one
// shared-memory stack per warp) gains from more warps in flight despite
// some spills (1.31M sphere: 8 / 9 / 10 blocks 1.660 / 1.626 /
// 1.616 ms per frame); per-lane and primary-packet walks lose from them.
// Smaller blocks, so that a warp's slot frees without waiting for the
// block's other warps, measured slower: 64 x 20 1.68 ms, 32 x 32 1.63 ms,
// 64 x 16 1.74 ms against 1.61 ms for 128 x 10.
constexpr int kPacketBlocks = 10, kPacketThreads = 128;

template <bool kCount, int kStackN, bool kPrimPacket, bool kShadowPacket>
__global__ void __launch_bounds__(kShadowPacket ? kPacketThreads : 128, kShadowPacket ? kPacketBlocks : 8)
    k_render_rt(DevScene s, RtLaunch L) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t px, py;
    const bool active = pixel_of(i, L.cam.width, L.cam.height, px, py);
    uint32_t shadows = 0;
    FetchCount fc;
    // one traversal stack per warp (the tile's rays are coherent)
    __shared__ uint32_t stacks[4][3 * kStackN];
    uint32_t *stk = stacks[threadIdx.x >> 5];
    const RayF r = primary_ray(L.cam, active ? px : 0, active ? py : 0);
    float dist = FLT_MAX;
    const bool geo = active && s.n_refs > 0;
    const int pos = kPrimPacket ? traverse_coherent<false, kCount, kStackN>(s, r, L.eps, 0.f, geo, dist, stk, &fc)
                                : traverse<false, kCount, kStackN>(s, r, L.eps, 0.f, geo, dist, &fc);
    const bool hit = active && pos >= 0;
    float cr = L.bg[0], cg = L.bg[1], cb = L.bg[2];
    int32_t id = -1;
    float4 nrm = make_float4(0.f, 0.f, 0.f, 0.f), alb = nrm;
    float hx = 0.f, hy = 0.f, hz = 0.f;
    if (hit) {
        id = (int32_t)__float_as_uint(__ldg(&s.tris[pos].v0[3]));
        nrm = __ldg(reinterpret_cast<const float4 *>(s.shade[id].n));
        alb = __ldg(reinterpret_cast<const float4 *>(s.shade[id].c));
        hx = r.ox + r.dx * dist, hy = r.oy + r.dy * dist, hz = r.oz + r.dz * dist;
        cr = 0.f, cg = 0.f, cb = 0.f;
    }
    bool done = !hit;
    for (int l = 0; l < L.n_lights; l++) {
        float lx = 0.f, ly = 0.f, lz = 0.f, d2 = 0.f, lambert = 0.f;
        bool need = false;
        if (!done) {
            lx = L.lights[l][0] - hx, ly = L.lights[l][1] - hy, lz = L.lights[l][2] - hz;
            d2 = lx * lx + ly * ly + lz * lz;
            if (d2 > 0) {
                const float inv = 1.0f / sqrtf(d2);
                lx *= inv, ly *= inv, lz *= inv;
            }
            lambert = lx * nrm.x + ly * nrm.y + lz * nrm.z;
            need = !(lambert < 0.f);
        }
        const RayF sr = need ? make_ray(hx, hy, hz, lx, ly, lz) : r;
        shadows += need ? 1u : 0u;
        float dummy;
        const bool occluded =
            (kShadowPacket ? traverse_coherent<true, kCount, kStackN>(s, sr, L.eps, d2, need, dummy, stk, &fc)
                           : traverse<true, kCount, kStackN>(s, sr, L.eps, d2, need, dummy, &fc)) >= 0;
        if (need && !occluded) {
            const float w = 1.0f / d2;
            cr = cr + ((alb.x * L.lights[l][3]) * lambert) * w;
            cg = cg + ((alb.y * L.lights[l][4]) * lambert) * w;
            cb = cb + ((alb.z * L.lights[l][5]) * lambert) * w;
            if (cr >= 1.f && cg >= 1.f && cb >= 1.f) done = true;
        }
    }
    if (hit) {
        cr = smax(0.f, smin(1.f, cr));
        cg = smax(0.f, smin(1.f, cg));
        cb = smax(0.f, smin(1.f, cb));
    }
    if (active) {
        uint8_t *o = L.rgb + 3ull * ((uint64_t)py * L.cam.width + px);
        o[0] = (uint8_t)quantise(cr);
        o[1] = (uint8_t)quantise(cg);
        o[2] = (uint8_t)quantise(cb);
        if (L.ids) {
            const uint64_t pix = (uint64_t)py * L.cam.width + px;
            L.ids[pix] = id;
            L.ts[pix] = dist;
        }
    }
    if (L.counters) {
        // warp-aggregated ray counts: primary rays, occlusion rays
        const uint32_t prim = __popc(__ballot_sync(0xFFFFFFFFu, active));
        uint32_t sh = shadows;
        for (int o = 16; o > 0; o >>= 1) sh += __shfl_xor_sync(0xFFFFFFFFu, sh, o);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(L.counters + 0, (unsigned long long)prim);
            atomicAdd(L.counters + 1, (unsigned long long)sh);
        }
        if (kCount) {
            // node-pair fetches, triangle-reference fetches, shaded hits
            unsigned long long pairs = fc.pairs, tris = fc.tris;
            const uint32_t hits = __popc(__ballot_sync(0xFFFFFFFFu, hit));
            for (int o = 16; o > 0; o >>= 1) {
                pairs += __shfl_xor_sync(0xFFFFFFFFu, pairs, o);
                tris += __shfl_xor_sync(0xFFFFFFFFu, tris, o);
            }
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(L.counters + 2, pairs);
                atomicAdd(L.counters + 3, tris);
                atomicAdd(L.counters + 4, (unsigned long long)hits);
            }
        }
    }
}

// First-hit features of each pixel for the denoiser: albedo (or emitted
// colour) 3, geometric normal 3, hit distance 1, as FP16; zeros on a miss.
__global__ void __launch_bounds__(128) k_features(DevScene s, CameraConsts cam, float eps, __half *out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t px, py;
    const bool active = pixel_of(i, cam.width, cam.height, px, py);
    const RayF r = primary_ray(cam, active ? px : 0, active ? py : 0);
    float t = FLT_MAX;
    const int pos = traverse<false>(s, r, eps, 0.f, active && s.n_refs > 0, t);
    if (!active) return;
    float f[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (pos >= 0) {
        const int id = (int)__float_as_uint(__ldg(&s.tris[pos].v0[3]));
        const float4 nrm = __ldg(reinterpret_cast<const float4 *>(s.shade[id].n));
        const float4 col = __ldg(reinterpret_cast<const float4 *>(s.shade[id].c));
        f[0] = col.x, f[1] = col.y, f[2] = col.z, f[3] = nrm.x, f[4] = nrm.y, f[5] = nrm.z, f[6] = t;
    }
    __half *o = out + 7ull * ((uint64_t)py * cam.width + px);
    for (int k = 0; k < 7; k++) o[k] = __float2half(f[k]);
}

}  // namespace

cudaError_t launch_features(const DevScene &s, const CameraConsts &cam, float eps, __half *out, cudaStream_t stream) {
    const uint64_t threads = warp_tiles(cam.width, cam.height) * 32;
    k_features<<<(unsigned)((threads + 127) / 128), 128, 0, stream>>>(s, cam, eps, out);
    return cudaGetLastError();
}

cudaError_t launch_trace_occluded(const DevScene &s, const float *rays, const float *dist2, uint64_t n, float eps,
                                  uint8_t *occluded, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const unsigned threads = 128;
    const uint64_t blocks = (n + threads - 1) / threads;
    // a 32-entry stack (half the per-thread local memory) when the hierarchy is shallow enough
    if (s.depth < 32)
        k_trace_occluded<32><<<(unsigned)blocks, threads, 0, stream>>>(s, rays, dist2, n, eps, occluded);
    else
        k_trace_occluded<kStack><<<(unsigned)blocks, threads, 0, stream>>>(s, rays, dist2, n, eps, occluded);
    return cudaGetLastError();
}

cudaError_t launch_trace_closest(const DevScene &s, const float *rays, uint64_t n, float eps, int32_t *ids,
                                 float *ts, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const unsigned threads = 128;
    const uint64_t blocks = (n + threads - 1) / threads;
    if (s.depth < 32)
        k_trace_closest<32><<<(unsigned)blocks, threads, 0, stream>>>(s, rays, n, eps, ids, ts);
    else
        k_trace_closest<kStack><<<(unsigned)blocks, threads, 0, stream>>>(s, rays, n, eps, ids, ts);
    return cudaGetLastError();
}

cudaError_t launch_render_rt(const DevScene &s, const RtLaunch &L, cudaStream_t stream) {
    const uint64_t tiles = warp_tiles(L.cam.width, L.cam.height);
    const uint64_t threads = tiles * 32;
    if (threads == 0) return cudaSuccess;
    const unsigned bs = L.packets == 1 ? kPacketThreads : 128, grid = (unsigned)((threads + bs - 1) / bs);
    // a 32-entry stack (half the per-thread local memory) when the hierarchy is shallow enough
    const bool small = s.depth < 32;
    auto go = [&](auto kernel) { kernel<<<grid, bs, 0, stream>>>(s, L); };
    // L.packets: 0 per lane, 1 primary and occlusion rays as packets, 2
    // primary rays only
    auto pick = [&](auto count) {
        constexpr bool kC = decltype(count)::value;
        if (L.packets == 1) small ? go(k_render_rt<kC, 32, true, true>) : go(k_render_rt<kC, kStack, true, true>);
        else if (L.packets == 2)
            small ? go(k_render_rt<kC, 32, true, false>) : go(k_render_rt<kC, kStack, true, false>);
        else small ? go(k_render_rt<kC, 32, false, false>) : go(k_render_rt<kC, kStack, false, false>);
    };
    if (L.count_fetches) pick(std::true_type{});
    else pick(std::false_type{});
    return cudaGetLastError();
}

}  // namespace pray_gpu
