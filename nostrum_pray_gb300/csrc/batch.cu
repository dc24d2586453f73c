// Many scenes path-traced in one persistent launch.
//
// Each scene of a batch is cut into tiles of 32 pixels (tile_w x tile_h, one
// warp per tile); the tiles of all scenes are numbered consecutively. A fixed
// grid of warps pulls tile numbers from one device counter (lane 0 does the
// atomic, the warp shares it), finds the tile's scene by binary search over
// the per-scene first-tile table and runs the per-pixel path tracer
// (pt_pixel.cuh) on it with that scene's tree and frame parameters. Uneven
// scenes (a 1k-triangle soup next to a 500k-triangle sphere, 256^2 next to
// 1024^2) thus share the GPU without a launch per scene. The counter is reset
// by a memset in the same stream, so the pair is captured into one CUDA graph.
// Tile shape, block size, grid size and the traversal stack depth are launch
// parameters picked by the host autotuner.
#include <algorithm>
#include <cstdint>

#include <cuda_runtime.h>

#include "batch_launch.h"
#include "pt_pixel.cuh"

namespace pray_gpu {

namespace {

using namespace dev;

// kLanes: every item runs mode 0, on the per-lane state machine; otherwise
// each tile runs pt_pixel_sync (modes 0 and 1).
template <int kStackN, bool kLanes>
__global__ void __launch_bounds__(256, 4) k_batch_pt(BatchLaunch B) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    while (true) {
        uint64_t tile = 0;
        if (lane == 0) tile = atomicAdd(B.next_tile, 1ull);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= B.total_tiles) break;
        // scene owning the tile: last item with first_tile <= tile
        int lo = 0, hi = B.n_items - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (B.items[mid].first_tile <= tile) lo = mid;
            else hi = mid - 1;
        }
        const BatchItem &it = B.items[lo];
        const uint64_t local = tile - it.first_tile;
        const uint32_t tiles_x = (it.L.cam.width + B.tile_w - 1) / B.tile_w;
        const uint32_t px = (uint32_t)(local % tiles_x) * B.tile_w + lane % B.tile_w;
        const uint32_t py = (uint32_t)(local / tiles_x) * B.tile_h + lane / B.tile_w;
        const bool active = px < it.L.cam.width && py < it.L.cam.height;
        uint32_t segments = 0;
        if (kLanes) {
            OnePixel src{active, px, py, false};
            uint32_t pixels = 0;
            pt_lanes<kStackN>(it.s, it.L, src, segments, pixels);
        } else {
            pt_pixel_sync<kStackN>(it.s, it.L, active, px, py, segments);
        }
        count_paths(B.counters, active, it.L.num_samples, segments);
    }
}

}  // namespace

cudaError_t launch_batch_pt(const BatchLaunch &B, int block_threads, int blocks, int stack_entries,
                            cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(B.next_tile, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    if (stack_entries <= 32) {
        if (B.kajiya) k_batch_pt<32, true><<<blocks, block_threads, 0, stream>>>(B);
        else k_batch_pt<32, false><<<blocks, block_threads, 0, stream>>>(B);
    } else {
        if (B.kajiya) k_batch_pt<kStack, true><<<blocks, block_threads, 0, stream>>>(B);
        else k_batch_pt<kStack, false><<<blocks, block_threads, 0, stream>>>(B);
    }
    return cudaGetLastError();
}

cudaError_t batch_max_blocks_per_sm(int block_threads, int stack_entries, bool kajiya, int *blocks) {
    if (stack_entries <= 32)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            blocks, kajiya ? k_batch_pt<32, true> : k_batch_pt<32, false>, block_threads, 0);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        blocks, kajiya ? k_batch_pt<kStack, true> : k_batch_pt<kStack, false>, block_threads, 0);
}

}  // namespace pray_gpu
