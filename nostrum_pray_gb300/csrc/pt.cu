// Per-pixel path-tracing kernels: one lane per pixel (pt_pixel.cuh), warps
// over 8x4 pixel tiles; the branching mode has a kernel of its own so that its
// frame stack does not weigh on the other modes. Built with --fmad=false like the rest of the
// tracing code.
#include <cstdint>

#include <cuda_runtime.h>

#include "pt_pixel.cuh"

namespace pray_gpu {

namespace {

using namespace dev;

// Modes 0 and 1 bounce by bounce (pt_pixel_sync). The per-lane state machine
// that the batch kernel runs for mode 0 measured slower here: 176.6 against
// 194.7 Msamples/s on the closed room, 653 against 863 on a 20k-triangle
// sphere (at 8 blocks of 128 threads per SM, 64 registers).
__global__ void __launch_bounds__(128, 10) k_render_pt(DevScene s, PtLaunch L) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t px, py;
    const bool active = pixel_of(i, L.cam.width, L.cam.height, px, py);
    uint32_t segments = 0;
    pt_pixel_sync<kStack>(s, L, active, px, py, segments);
    if (L.counters) count_paths(L.counters, active, L.num_samples, segments);
}

__global__ void __launch_bounds__(128) k_render_pt_diffuse(DevScene s, PtLaunch L) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t px, py;
    const bool active = pixel_of(i, L.cam.width, L.cam.height, px, py);
    uint32_t segments = 0;
    pt_pixel_diffuse<kStack>(s, L, active, px, py, segments);
    if (L.counters) count_paths(L.counters, active, 1, segments);
}

}  // namespace

cudaError_t launch_render_pt(const DevScene &s, const PtLaunch &L, cudaStream_t stream) {
    const uint64_t tiles = warp_tiles(L.cam.width, L.cam.height);
    const uint64_t threads = tiles * 32;
    if (threads == 0) return cudaSuccess;
    const unsigned bs = 128;
    if (L.mode == 2)
        k_render_pt_diffuse<<<(unsigned)((threads + bs - 1) / bs), bs, 0, stream>>>(s, L);
    else
        k_render_pt<<<(unsigned)((threads + bs - 1) / bs), bs, 0, stream>>>(s, L);
    return cudaGetLastError();
}

}  // namespace pray_gpu
