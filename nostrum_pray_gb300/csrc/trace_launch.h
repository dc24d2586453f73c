// Host-side launchers of the tracing kernels (trace.cu). Called by the C-ABI
// layer with device pointers; they return the launch status and do not
// synchronise.
#pragma once

#include <cstdint>

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
};

constexpr int kMaxPtDepth = 64;  // bounce limit of the path tracer (per-thread albedo stack)

struct PtLaunch {
    CameraConsts cam;
    float bg[3];
    uint32_t max_depth, num_samples, rr_depth;
    int32_t mode;                    // 0: reference recursion, 1: NEE + Russian roulette
    uint64_t seed;
    float eps;
    uint8_t *rgb;                    // out: height x width x 3
    float *radiance;                 // optional out: height x width x 3 mean radiance
    unsigned long long *counters;    // optional out (accumulated): [0] paths, [1] ray segments
};

cudaError_t launch_render_pt(const DevScene &s, const PtLaunch &L, cudaStream_t stream);

cudaError_t launch_trace_closest(const DevScene &s, const float *rays, uint64_t n, float eps, int32_t *ids,
                                 float *ts, cudaStream_t stream);

cudaError_t launch_render_rt(const DevScene &s, const RtLaunch &L, cudaStream_t stream);

}  // namespace pray_gpu
