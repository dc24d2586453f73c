// Host-side launchers of the tracing kernels (trace.cu). Called by the C-ABI
// layer with device pointers; they return the launch status and do not
// synchronise.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "device_layout.h"
#include "host/camera.h"

namespace pray_gpu {

constexpr int kMaxLights = 64;

struct RtLaunch {
    CameraConsts cam;
    float lights[kMaxLights][6];  // position, colour
    int n_lights;
    float bg[3];
    float eps;                       // det threshold of the intersector
    uint8_t *rgb;                    // out: height x width x 3
    int32_t *ids;                    // optional out: primary hit triangle id per pixel (-1: miss)
    float *ts;                       // optional out: primary hit distance per pixel (FLT_MAX: miss)
    unsigned long long *counters;    // optional out (accumulated): [0] primary rays, [1] occlusion rays
    int count_fetches;               // also accumulate [2] node-pair fetches, [3] triangle fetches, [4] shaded hits
    int packets;                     // pray_traversal: warp packets (traverse_packet) for primary and occlusion
                                     // rays (1), primary rays only (2), none (0)
};

constexpr int kMaxPtDepth = 64;  // bounce limit of the path tracer (per-thread albedo stack)
constexpr int kMaxDiffuseDepth = 8;  // depth limit of the branching mode (per-thread frame stack)

struct PtLaunch {
    CameraConsts cam;
    float bg[3];
    uint32_t max_depth, num_samples, rr_depth;
    int32_t mode;                    // 0: reference recursion, 1: NEE + Russian roulette, 2: branching
    uint64_t seed;
    float eps;
    uint32_t sample_offset;          // first sample index (PCG stream selector)
    uint8_t *rgb;                    // optional out: height x width x 3
    float *radiance;                 // optional out: height x width x 3 mean radiance
    double *sum64;                   // optional in/out: height x width x 3 FP64 sums, samples added in order
    unsigned long long *counters;    // optional out (accumulated): [0] paths, [1] ray segments
    unsigned long long *next_pixel;  // per-pixel kernel: work counter of the frame (zero at launch)
};

// Per-pixel kernel on `sm_count` SMs; mode 1 needs L.next_pixel (zeroed on
// the stream before the launch; one frame at a time per counter).
cudaError_t launch_render_pt(const DevScene &s, const PtLaunch &L, int sm_count, cudaStream_t stream);

// Wavefront path tracer (wavefront.cu): path pool and queues in `scratch`.
struct WavefrontScratch {
    float4 *org, *dir, *thr, *rad;   // per path: origin, direction, throughput, radiance
    uint64_t *rng;                   // per path: PCG32 state
    uint32_t *depth;                 // per path
    float *hit_t;                    // per path: closest-hit distance
    int32_t *hit_ref;                // per path: closest-hit reference (-1: miss)
    uint32_t *queue[2];              // path ids, ping-pong
    float4 *shadow;                  // occlusion jobs: 3 float4 each (origin+path, dir+dist2, contribution)
    uint32_t *counts;                // [0], [1]: queue lengths, [2]: occlusion jobs, [3], [4]: fetch counters
    float *pixel_sum;                // per pixel x 3: running float sum over samples
    uint64_t capacity;               // paths per round
};

// Bytes of scratch for `capacity` paths and `pixels` pixels.
uint64_t wavefront_scratch_bytes(uint64_t capacity, uint64_t pixels);
// Carves a scratch block of wavefront_scratch_bytes() bytes (256-byte aligned base).
WavefrontScratch wavefront_carve(void *base, uint64_t capacity, uint64_t pixels);
// Loads every kernel a wavefront frame may launch (both traversal-stack
// variants) on the current device, so that no later frame triggers a lazy
// module load.
cudaError_t wavefront_preload_kernels();
// Enqueues one whole frame (all rounds) on `stream`; capturable in a graph.
// With `side`, `fork` and `join` (a second stream and two events), each
// bounce's occlusion pass runs on `side` beside the next bounce's extend
// pass; without them every pass runs on `stream` in order. The same image.
cudaError_t record_wavefront_frame(const DevScene &s, const PtLaunch &L, const WavefrontScratch &w, int sm_count,
                                   cudaStream_t stream, cudaStream_t side = nullptr, cudaEvent_t fork = nullptr,
                                   cudaEvent_t join = nullptr);

// Allocation-free wavefront frame on the static scratch of
// wavefront_noalloc.cu (why receives a message on a size or set-up error).
cudaError_t launch_wavefront_noalloc(const DevScene &s, const PtLaunch &L, uint64_t max_paths, cudaStream_t stream,
                                     std::string &why);
// Largest frame (pixels) the allocation-free path accepts.
uint64_t noalloc_max_pixels();

cudaError_t launch_relmse(const double *img, double img_scale, const double *ref, double ref_scale, uint64_t n,
                          double *out, cudaStream_t stream);

cudaError_t launch_features(const DevScene &s, const CameraConsts &cam, float eps, __half *out, cudaStream_t stream);

cudaError_t launch_trace_occluded(const DevScene &s, const float *rays, const float *dist2, uint64_t n, float eps,
                                  uint8_t *occluded, cudaStream_t stream);
cudaError_t launch_trace_closest(const DevScene &s, const float *rays, uint64_t n, float eps, int32_t *ids,
                                 float *ts, cudaStream_t stream);

cudaError_t launch_render_rt(const DevScene &s, const RtLaunch &L, cudaStream_t stream);

}  // namespace pray_gpu
