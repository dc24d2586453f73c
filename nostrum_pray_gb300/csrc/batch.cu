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

// Scene owning a tile: the last item with first_tile <= tile.
__device__ __forceinline__ int item_of(const BatchLaunch &B, uint64_t tile) {
    int lo = 0, hi = B.n_items - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B.items[mid].first_tile <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ uint64_t next_tile(const BatchLaunch &B) {
    uint64_t tile = 0;
    if ((threadIdx.x & 31u) == 0) tile = atomicAdd(B.next_tile, 1ull);
    return __shfl_sync(0xFFFFFFFFu, tile, 0);
}

// Pixels for the per-lane state machine (pt_lanes) from consecutive tiles of
// one scene: a lane whose pixel is done takes the next pixel of the warp's
// current tile, and once that tile is handed out the warp pulls the next
// tile from the counter, so lanes of a tile's short paths (background
// pixels) do not idle while its long ones finish. A tile of another scene
// ends the refills and is kept in `pending` for the warp's next scene.
// Warp-uniform state.
struct TileSrc {
    const BatchLaunch &B;
    int item;
    uint32_t tiles_x, width, height;
    uint64_t tile;
    uint32_t slot;     // next pixel slot of `tile` (32: handed out)
    uint64_t pending;  // fetched tile of another scene (>= total_tiles: none)
    bool done;
    __device__ __forceinline__ bool drained() const { return done && slot >= 32; }
    __device__ __forceinline__ bool take(bool want, uint32_t &x, uint32_t &y) {
        const unsigned ask = __ballot_sync(0xFFFFFFFFu, want);
        const uint32_t rank = __popc(ask & ((1u << (threadIdx.x & 31u)) - 1u));
        if (slot >= 32 && !done) {
            const uint64_t t = next_tile(B);
            if (t >= B.total_tiles) {
                done = true;
            } else if (item_of(B, t) != item) {
                pending = t;
                done = true;
            } else {
                tile = t;
                slot = 0;
            }
        }
        if (slot >= 32) return false;
        const uint32_t s = slot + rank;
        slot = min(32u, slot + (uint32_t)__popc(ask));
        if (!want || s >= 32) return false;
        const uint64_t local = tile - B.items[item].first_tile;
        x = (uint32_t)(local % tiles_x) * B.tile_w + s % B.tile_w;
        y = (uint32_t)(local / tiles_x) * B.tile_h + s / B.tile_w;
        return x < width && y < height;
    }
};

// kLanes: every item runs mode 0, on the per-lane state machine with lanes
// refilled across the scene's tiles; otherwise each tile runs pt_pixel_sync
// (modes 0 and 1).
template <int kStackN, bool kLanes>
__global__ void __launch_bounds__(256, 4) k_batch_pt(BatchLaunch B) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    if (kLanes) {
        uint64_t tile = next_tile(B);
        while (tile < B.total_tiles) {
            const int item = item_of(B, tile);
            const BatchItem &it = B.items[item];
            TileSrc src{B, item, (it.L.cam.width + B.tile_w - 1) / B.tile_w, it.L.cam.width, it.L.cam.height,
                        tile, 0, B.total_tiles, false};
            uint32_t segments = 0, pixels = 0;
            pt_lanes<kStackN>(it.s, it.L, src, segments, pixels);
            // [paths, segments] of this scene's pixels
            unsigned long long paths = (unsigned long long)pixels * it.L.num_samples, segs = segments;
            for (int o = 16; o > 0; o >>= 1) {
                paths += __shfl_xor_sync(kFull, paths, o);
                segs += __shfl_xor_sync(kFull, segs, o);
            }
            if (lane == 0 && B.counters) {
                atomicAdd(B.counters + 0, paths);
                atomicAdd(B.counters + 1, segs);
            }
            tile = src.pending < B.total_tiles ? src.pending : next_tile(B);
        }
        return;
    }
    while (true) {
        const uint64_t tile = next_tile(B);
        if (tile >= B.total_tiles) break;
        const BatchItem &it = B.items[item_of(B, tile)];
        const uint64_t local = tile - it.first_tile;
        const uint32_t tiles_x = (it.L.cam.width + B.tile_w - 1) / B.tile_w;
        const uint32_t px = (uint32_t)(local % tiles_x) * B.tile_w + lane % B.tile_w;
        const uint32_t py = (uint32_t)(local / tiles_x) * B.tile_h + lane / B.tile_w;
        const bool active = px < it.L.cam.width && py < it.L.cam.height;
        uint32_t segments = 0;
        pt_pixel_sync<kStackN>(it.s, it.L, active, px, py, segments);
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
