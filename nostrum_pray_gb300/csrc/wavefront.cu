// Wavefront path tracer (next-event estimation + Russian roulette mode).
//
// A frame is processed in rounds of S samples per pixel. Each round runs
//   init     one path per (pixel, sample): primary ray, PCG32 stream
//   repeat max_depth + 1 times:
//     extend   closest hit for every queued path
//     shade    miss / emitter / depth termination, next-event sample (an
//              occlusion job), cosine bounce and Russian roulette; surviving
//              paths are appended to the next queue
//     occlude  any-hit test of the occlusion jobs; unoccluded contributions
//              are added to their path's radiance
//   accumulate  per pixel, the round's samples in sample order
// and a final pass writes the mean radiance and the 8-bit image.
//
// Queues are compacted with one atomic per warp (ballot + popc + shfl). Every
// path keeps its own slot, and each pixel sums its samples in sample order,
// so the result does not depend on queue order: it equals the per-pixel
// kernel (pt.cu, mode 1) and the oracle bit for bit. Kernels read their work
// counts from device memory and loop over them with a fixed grid, so a whole
// frame is a fixed launch sequence that the host captures once into a CUDA
// graph and replays.
//
// Built with --fmad=false like the rest of the tracing code.
#include <cfloat>
#include <algorithm>
#include <atomic>
#include <cstdint>

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "../../include/nostrum_pray_sampling.h"
#include "device_layout.h"
#include "trace_launch.h"
#include "traverse.cuh"

namespace cg = cooperative_groups;

namespace pray_gpu {

namespace {

using namespace dev;

constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kShadowShrink = 0.999f;
constexpr int kThreads = 256;
constexpr int kRefillIdle = 8;  // dynamic fetch: refill a warp's idle lanes once this many are idle
constexpr int kTraceBlocksPerSm = 5;  // resident blocks per SM of the extend and occlusion passes (register cap)

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Appends for every lane with `pred`; returns the lane's slot (valid where
// pred). Called by all lanes of a converged warp.
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool pred) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, pred);
    uint32_t base = 0;
    if (m) {
        const int leader = __ffs(m) - 1;
        if ((int)lane_id() == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
    }
    return base + (uint32_t)__popc(m & ((1u << lane_id()) - 1u));
}

__device__ __forceinline__ void warp_count(unsigned long long *c, uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if (lane_id() == 0 && c) atomicAdd(c, (unsigned long long)v);
}

// Warp-converged grid-stride loop bounds: every lane of a warp runs the same
// number of iterations; `i` may be >= n on the last one.
__device__ __forceinline__ uint64_t first_index() { return (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ uint64_t grid_stride() { return (uint64_t)gridDim.x * blockDim.x; }
__device__ __forceinline__ uint64_t rounded(uint64_t n) { return (n + 31) & ~31ull; }

__device__ __forceinline__ uint64_t pcg_inc(uint64_t pixel, uint32_t sample) {
    return (((pixel << 32) ^ (uint64_t)sample) << 1u) | 1u;
}

__global__ void __launch_bounds__(kThreads) k_wf_init(PtLaunch L, WavefrontScratch w, uint32_t round_base,
                                                      uint32_t S, uint64_t P) {
    const uint64_t n = P * S;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counts[0] = (uint32_t)n;
        w.counts[1] = 0;
        w.counts[2] = 0;
        w.counts[3] = 0;
        w.counts[4] = 0;
        w.counts[5] = 0;
    }
    for (uint64_t i = first_index(); i < n; i += grid_stride()) {
        const uint64_t pixel = i % P;
        const uint32_t sample = L.sample_offset + round_base + (uint32_t)(i / P);
        const uint32_t px = (uint32_t)(pixel % L.cam.width), py = (uint32_t)(pixel / L.cam.width);
        const RayF r = primary_ray(L.cam, px, py);
        w.org[i] = make_float4(r.ox, r.oy, r.oz, 0.f);
        w.dir[i] = make_float4(r.dx, r.dy, r.dz, 0.f);
        w.thr[i] = make_float4(1.f, 1.f, 1.f, 0.f);
        w.rad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        w.rng[i] = pray_pcg32_stream(L.seed, pixel, sample).state;
        w.depth[i] = 0;
        w.queue[0][i] = (uint32_t)i;
    }
}

// Hands the warp's idle lanes (mask `idle`) the next entries of a work list
// of n items through the counter; returns the lane's item index (>= n: none)
// and sets `drained` (warp-uniform) once every item has been handed out.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t *counter, unsigned idle, uint32_t n, bool &drained) {
    uint32_t base = 0;
    if (lane_id() == 0) base = atomicAdd(counter, (uint32_t)__popc(idle));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if ((uint64_t)base + (uint32_t)__popc(idle) >= n) drained = true;
    return base + (uint32_t)__popc(idle & ((1u << lane_id()) - 1u));
}

// Closest hit of every queued path, with dynamic fetch (after Aila & Laine
// 2009): each warp runs the traversal round by round and, whenever at least
// kRefillIdle of its lanes have finished their ray, gives those lanes the next
// queue entries (one atomic per warp), so lanes do not idle until the
// slowest ray of the warp is done. Work is handed out through counts[3]
// (reset by the shade pass). It also empties the next shade pass's output
// queue and its occlusion-job count (counts[jobs]; the occlusion pass of the
// previous bounce, which may run beside this one, reads the other slot).
template <int kStackN>
__global__ void __launch_bounds__(kThreads, kTraceBlocksPerSm) k_wf_extend(DevScene s, PtLaunch L, WavefrontScratch w,
                                                                         int in, int out, int jobs) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t n = w.counts[in];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counts[out] = 0;
        w.counts[jobs] = 0;
    }
    uint32_t seg = 0;
    Trav T;
    TravStack<kStackN> S;
    T.have_node = T.have_leaf = false;
    RayF r{};
    uint32_t p = 0;
    bool has = false, drained = false;
    while (true) {
        const unsigned idle = __ballot_sync(kFull, !has);
        if (!drained && (__popc(idle) >= kRefillIdle || idle == kFull)) {
            const uint32_t idx = warp_fetch(w.counts + 3, idle, n, drained);
            if (!has && idx < n) {
                p = w.queue[in][idx];
                const float4 o = w.org[p], d = w.dir[p];
                r.ox = o.x, r.oy = o.y, r.oz = o.z;
                r.dx = d.x, r.dy = d.y, r.dz = d.z;
                r.ix = 1.0f / d.x, r.iy = 1.0f / d.y, r.iz = 1.0f / d.z;
                has = true;
                trav_start<kClosest>(s, r, 0.f, s.n_refs > 0, T);
            }
        }
        if (!__any_sync(kFull, has)) break;
        trav_round<kClosest, false>(s, r, L.eps, 0.f, T, S, nullptr);
        if (has && !T.active()) {
            w.hit_t[p] = T.best_t;
            w.hit_ref[p] = T.best;
            seg++;
            has = false;
        }
    }
    if (L.counters) warp_count(L.counters + 1, seg);
}

// Shading of every queued path: background or emitter, next-event job
// (appended to counts[jobs]), cosine bounce and Russian roulette into the
// queue `out`. Resets the fetch counters of the occlusion pass that follows
// and of the next extend pass (counts[4], counts[3]).
__global__ void __launch_bounds__(kThreads) k_wf_shade(DevScene s, PtLaunch L, WavefrontScratch w, int in, int out,
                                                       int jobs, uint32_t round_base, uint64_t P) {
    const uint32_t n = w.counts[in];
    if (blockIdx.x == 0 && threadIdx.x == 0) w.counts[3] = w.counts[4] = 0;
    for (uint64_t i = first_index(); i < rounded(n); i += grid_stride()) {
        bool cont = false, job = false;
        uint32_t p = 0;
        float4 jo, jd, jc;
        if (i < n) {
            p = w.queue[in][i];
            const int pos = w.hit_ref[p];
            float4 T = w.thr[p], R = w.rad[p];
            const uint32_t depth = w.depth[p];
            if (pos < 0) {
                R.x = R.x + T.x * L.bg[0], R.y = R.y + T.y * L.bg[1], R.z = R.z + T.z * L.bg[2];
            } else {
                const int id = (int)__float_as_uint(__ldg(&s.tris[pos].v0[3]));
                const float4 nrm = __ldg(reinterpret_cast<const float4 *>(s.shade[id].n));
                const float4 col = __ldg(reinterpret_cast<const float4 *>(s.shade[id].c));
                if (nrm.w != 0.f) {
                    if (depth == 0) R.x = R.x + T.x * col.x, R.y = R.y + T.y * col.y, R.z = R.z + T.z * col.z;
                } else if (depth < L.max_depth) {
                    const float4 o = w.org[p], d = w.dir[p];
                    const float t = w.hit_t[p];
                    const float hx = o.x + d.x * t, hy = o.y + d.y * t, hz = o.z + d.z * t;
                    const uint64_t pixel = p % P;
                    const uint32_t sample = L.sample_offset + round_base + (uint32_t)(p / P);
                    pray_pcg32 rng;
                    rng.state = w.rng[p];
                    rng.inc = pcg_inc(pixel, sample);
                    if (s.n_emit > 0) {
                        const float ue = pray_uniform(&rng), ua = pray_uniform(&rng), ub = pray_uniform(&rng);
                        const float target = ue * s.emit_area;
                        uint32_t lo = 0, hi = s.n_emit - 1;
                        while (lo < hi) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (__ldg(s.emit_cdf + mid) > target) hi = mid;
                            else lo = mid + 1;
                        }
                        const GTri *E = s.emit_tris + lo;
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
                            const float4 en = __ldg(reinterpret_cast<const float4 *>(s.shade[eid].n));
                            const float4 ec = __ldg(reinterpret_cast<const float4 *>(s.shade[eid].c));
                            const float cx = nrm.x * wx + nrm.y * wy + nrm.z * wz;
                            const float cy = -(en.x * wx + en.y * wy + en.z * wz);
                            if (cx > 0.f && cy > 0.f) {
                                const float g = ((cx * cy) * s.emit_area) * kInvPi / d2;
                                job = true;
                                jo = make_float4(hx, hy, hz, __uint_as_float(p));
                                jd = make_float4(wx, wy, wz, d2 * kShadowShrink);
                                jc = make_float4(((T.x * col.x) * ec.x) * g, ((T.y * col.y) * ec.y) * g,
                                                 ((T.z * col.z) * ec.z) * g, 0.f);
                            }
                        }
                    }
                    const float u1 = pray_uniform(&rng), u2 = pray_uniform(&rng);
                    const float n3[3] = {nrm.x, nrm.y, nrm.z};
                    float dd[3];
                    pray_sample_hemisphere(n3, u1, u2, dd);
                    const RayF nr = make_ray(hx, hy, hz, dd[0], dd[1], dd[2]);
                    T.x = T.x * col.x, T.y = T.y * col.y, T.z = T.z * col.z;
                    cont = true;
                    if (depth >= L.rr_depth) {
                        const float q = smin(smax(smax(T.x, T.y), T.z), 0.95f);
                        if (!(pray_uniform(&rng) < q)) cont = false;
                        else T.x = T.x / q, T.y = T.y / q, T.z = T.z / q;
                    }
                    w.org[p] = make_float4(hx, hy, hz, 0.f);
                    w.dir[p] = make_float4(nr.dx, nr.dy, nr.dz, 0.f);
                    w.thr[p] = T;
                    w.rng[p] = rng.state;
                    w.depth[p] = depth + 1;
                }
            }
            w.rad[p] = R;
        }
        const uint32_t js = warp_append(w.counts + jobs, job);
        if (job) {
            float4 *j = w.shadow + 3ull * js;
            j[0] = jo;
            j[1] = jd;
            j[2] = jc;
        }
        const uint32_t qs = warp_append(w.counts + out, cont);
        if (cont) w.queue[out][qs] = p;
    }
}

// Any-hit test of every occlusion job (counts[jobs] of them), with the same
// dynamic fetch (counts[4]); an unoccluded job adds its contribution to its
// path.
template <int kStackN>
__global__ void __launch_bounds__(kThreads, kTraceBlocksPerSm) k_wf_occlude(DevScene s, PtLaunch L,
                                                                          WavefrontScratch w, int jobs) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t n = w.counts[jobs];
    uint32_t seg = 0;
    Trav T;
    TravStack<kStackN> S;
    T.have_node = T.have_leaf = false;
    RayF r{};
    float d2 = 0.f;
    float4 jo = make_float4(0.f, 0.f, 0.f, 0.f), jc = jo;
    bool has = false, drained = false;
    while (true) {
        const unsigned idle = __ballot_sync(kFull, !has);
        if (!drained && (__popc(idle) >= kRefillIdle || idle == kFull)) {
            const uint32_t idx = warp_fetch(w.counts + 4, idle, n, drained);
            if (!has && idx < n) {
                const float4 *j = w.shadow + 3ull * idx;
                jo = j[0];
                const float4 jd = j[1];
                jc = j[2];
                r = make_ray(jo.x, jo.y, jo.z, jd.x, jd.y, jd.z);
                d2 = jd.w;
                has = true;
                trav_start<kAnyHit>(s, r, d2, s.n_refs > 0, T);
            }
        }
        if (!__any_sync(kFull, has)) break;
        trav_round<kAnyHit, false>(s, r, L.eps, d2, T, S, nullptr);
        if (has && !T.active()) {
            seg++;
            if (T.best < 0) {
                const uint32_t p = __float_as_uint(jo.w);
                float4 R = w.rad[p];
                R.x = R.x + jc.x, R.y = R.y + jc.y, R.z = R.z + jc.z;
                w.rad[p] = R;
            }
            has = false;
        }
    }
    if (L.counters) warp_count(L.counters + 1, seg);
}

__global__ void __launch_bounds__(kThreads) k_wf_accumulate(PtLaunch L, WavefrontScratch w, uint32_t S, uint64_t P,
                                                            int first) {
    for (uint64_t p = first_index(); p < P; p += grid_stride()) {
        float sx = first ? 0.f : w.pixel_sum[3 * p], sy = first ? 0.f : w.pixel_sum[3 * p + 1],
              sz = first ? 0.f : w.pixel_sum[3 * p + 2];
        double ax = 0, ay = 0, az = 0;
        if (L.sum64) ax = L.sum64[3 * p], ay = L.sum64[3 * p + 1], az = L.sum64[3 * p + 2];
        for (uint32_t k = 0; k < S; k++) {
            const float4 r = w.rad[(uint64_t)k * P + p];
            sx = sx + r.x, sy = sy + r.y, sz = sz + r.z;
            if (L.sum64) ax = ax + (double)r.x, ay = ay + (double)r.y, az = az + (double)r.z;
        }
        w.pixel_sum[3 * p] = sx, w.pixel_sum[3 * p + 1] = sy, w.pixel_sum[3 * p + 2] = sz;
        if (L.sum64) L.sum64[3 * p] = ax, L.sum64[3 * p + 1] = ay, L.sum64[3 * p + 2] = az;
    }
    if (L.counters && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(L.counters, (unsigned long long)(P * S));
}

__global__ void __launch_bounds__(kThreads) k_wf_finish(PtLaunch L, WavefrontScratch w, uint64_t P) {
    const float ns = (float)L.num_samples;
    for (uint64_t p = first_index(); p < P; p += grid_stride()) {
        const float mr = w.pixel_sum[3 * p] / ns, mg = w.pixel_sum[3 * p + 1] / ns, mb = w.pixel_sum[3 * p + 2] / ns;
        if (L.radiance) L.radiance[3 * p] = mr, L.radiance[3 * p + 1] = mg, L.radiance[3 * p + 2] = mb;
        if (L.rgb) {
            L.rgb[3 * p] = (uint8_t)quantise(smax(0.f, smin(1.f, mr)));
            L.rgb[3 * p + 1] = (uint8_t)quantise(smax(0.f, smin(1.f, mg)));
            L.rgb[3 * p + 2] = (uint8_t)quantise(smax(0.f, smin(1.f, mb)));
        }
    }
}

// FP64 relative MSE over one cluster of CTAs, the whole grid (distributed
// shared memory, no global scratch, one launch). The FP64 divide is many
// instructions on this part's narrow FP64 pipe, so one SM would take
// milliseconds for a 512^2 frame; 16 SMs share it (8 where a 16-CTA cluster
// cannot be placed). Deterministic for a given cluster size: each CTA sums a
// fixed stride of the values, reduces its threads' sums by a fixed tree, and
// CTA 0 adds the CTAs' sums in rank order.
constexpr int kRelmseThreads = 1024;

__global__ void __launch_bounds__(kRelmseThreads) k_relmse(const double *img, double a, const double *ref, double b,
                                                           uint64_t n, double *out) {
    __shared__ double sm[kRelmseThreads];
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank(), ctas = cluster.num_blocks();
    double acc = 0.0;
    for (uint64_t i = (uint64_t)rank * kRelmseThreads + threadIdx.x; i < n; i += (uint64_t)kRelmseThreads * ctas) {
        const double x = img[i] * a, r = ref[i] * b;
        const double d = x - r;
        acc += d * d / (r * r + 0.01);
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kRelmseThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    cluster.sync();  // every CTA's sum in its sm[0]
    if (rank == 0 && threadIdx.x == 0) {
        double total = 0.0;
        for (unsigned c = 0; c < ctas; c++) total += *cluster.map_shared_rank(&sm[0], c);
        out[0] = n ? total / (double)n : 0.0;
    }
    cluster.sync();  // the other CTAs' shared memory stays until CTA 0 has read it
}

}  // namespace

uint64_t wavefront_scratch_bytes(uint64_t capacity, uint64_t pixels) {
    auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
    return 4 * al(16 * capacity) + al(8 * capacity) + al(4 * capacity) * 3 + 2 * al(4 * capacity) +
           al(48 * capacity) + al(32) + al(12 * pixels);
}

WavefrontScratch wavefront_carve(void *base, uint64_t capacity, uint64_t pixels) {
    auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
    char *p = static_cast<char *>(base);
    WavefrontScratch w;
    auto take = [&](uint64_t bytes) {
        char *r = p;
        p += al(bytes);
        return r;
    };
    w.org = reinterpret_cast<float4 *>(take(16 * capacity));
    w.dir = reinterpret_cast<float4 *>(take(16 * capacity));
    w.thr = reinterpret_cast<float4 *>(take(16 * capacity));
    w.rad = reinterpret_cast<float4 *>(take(16 * capacity));
    w.rng = reinterpret_cast<uint64_t *>(take(8 * capacity));
    w.depth = reinterpret_cast<uint32_t *>(take(4 * capacity));
    w.hit_t = reinterpret_cast<float *>(take(4 * capacity));
    w.hit_ref = reinterpret_cast<int32_t *>(take(4 * capacity));
    w.queue[0] = reinterpret_cast<uint32_t *>(take(4 * capacity));
    w.queue[1] = reinterpret_cast<uint32_t *>(take(4 * capacity));
    w.shadow = reinterpret_cast<float4 *>(take(48 * capacity));
    w.counts = reinterpret_cast<uint32_t *>(take(32));
    w.pixel_sum = reinterpret_cast<float *>(take(12 * pixels));
    w.capacity = capacity;
    return w;
}

cudaError_t wavefront_preload_kernels() {
    cudaFuncAttributes a;
    const void *kernels[] = {
        reinterpret_cast<const void *>(k_wf_init),         reinterpret_cast<const void *>(k_wf_extend<32>),
        reinterpret_cast<const void *>(k_wf_extend<kStack>), reinterpret_cast<const void *>(k_wf_shade),
        reinterpret_cast<const void *>(k_wf_occlude<32>),  reinterpret_cast<const void *>(k_wf_occlude<kStack>),
        reinterpret_cast<const void *>(k_wf_accumulate),   reinterpret_cast<const void *>(k_wf_finish)};
    for (const void *k : kernels) {
        cudaError_t e = cudaFuncGetAttributes(&a, k);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t record_wavefront_frame(const DevScene &s, const PtLaunch &L, const WavefrontScratch &w, int sm_count,
                                   cudaStream_t stream, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
    const uint64_t P = (uint64_t)L.cam.width * L.cam.height;
    if (P == 0 || L.num_samples == 0) return cudaSuccess;
    const uint32_t S = (uint32_t)std::min<uint64_t>(L.num_samples, std::max<uint64_t>(1, w.capacity / P));
    const unsigned grid = (unsigned)std::max(1, sm_count) * kTraceBlocksPerSm;
    const bool small_stack = s.depth < 32;  // a 32-entry traversal stack suffices
    // With a side stream, bounce b's occlusion pass runs there, beside bounce
    // b + 1's extend pass (they touch different fields and counters: the
    // two alternate occlusion-job counts, counts[2] and counts[5]), so each
    // fills the other's ramp and tail; shade b + 1 waits for both.
    const bool overlap = side && fork && join;
    cudaError_t e = cudaSuccess;
    for (uint32_t base = 0; base < L.num_samples && e == cudaSuccess; base += S) {
        const uint32_t Sr = std::min(S, L.num_samples - base);
        k_wf_init<<<grid, kThreads, 0, stream>>>(L, w, base, Sr, P);
        for (uint32_t it = 0; it <= L.max_depth && e == cudaSuccess; it++) {
            const int in = (int)(it & 1), out = 1 - in, jobs = (it & 1) ? 5 : 2;
            if (small_stack) k_wf_extend<32><<<grid, kThreads, 0, stream>>>(s, L, w, in, out, jobs);
            else k_wf_extend<kStack><<<grid, kThreads, 0, stream>>>(s, L, w, in, out, jobs);
            if (overlap && it > 0) e = cudaStreamWaitEvent(stream, join, 0);
            k_wf_shade<<<grid, kThreads, 0, stream>>>(s, L, w, in, out, jobs, base, P);
            cudaStream_t occ = stream;
            if (overlap) {
                if (e == cudaSuccess) e = cudaEventRecord(fork, stream);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork, 0);
                occ = side;
            }
            if (small_stack) k_wf_occlude<32><<<grid, kThreads, 0, occ>>>(s, L, w, jobs);
            else k_wf_occlude<kStack><<<grid, kThreads, 0, occ>>>(s, L, w, jobs);
            if (overlap && e == cudaSuccess) e = cudaEventRecord(join, side);
        }
        if (overlap && e == cudaSuccess) e = cudaStreamWaitEvent(stream, join, 0);
        k_wf_accumulate<<<grid, kThreads, 0, stream>>>(L, w, Sr, P, base == 0 ? 1 : 0);
    }
    k_wf_finish<<<grid, kThreads, 0, stream>>>(L, w, P);
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_relmse(const double *img, double a, const double *ref, double b, uint64_t n, double *out,
                          cudaStream_t stream) {
    // the cluster size, once per device: 16 (a non-portable size) when the
    // occupancy query can place such a cluster, else 8
    static std::atomic<int> sizes[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1, attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kRelmseThreads), cfg.stream = stream;
    cfg.attrs = attr, cfg.numAttrs = 1;
    int ctas = sizes[dev].load();
    if (ctas == 0) {
        ctas = 8;
        if (cudaFuncSetAttribute(k_relmse, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            int clusters = 0;
            attr[0].val.clusterDim.x = 16;
            cfg.gridDim = dim3(16);
            if (cudaOccupancyMaxActiveClusters(&clusters, k_relmse, &cfg) == cudaSuccess && clusters >= 1) ctas = 16;
        }
        cudaGetLastError();  // a refused query leaves the 8-CTA cluster
        sizes[dev].store(ctas);
    }
    attr[0].val.clusterDim.x = (unsigned)ctas;
    cfg.gridDim = dim3((unsigned)ctas);
    e = cudaLaunchKernelEx(&cfg, k_relmse, img, a, ref, b, n, out);
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace pray_gpu
