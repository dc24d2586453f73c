// Batched path tracing (batch.cu): per-scene launch records in device memory
// and the persistent launch over all of them.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "device_layout.h"
#include "trace_launch.h"

namespace pray_gpu {

struct BatchItem {
    DevScene s;           // the scene's device tree and shading data
    PtLaunch L;           // its frame: camera, samples, depth, mode, outputs
    uint64_t first_tile;  // number of the scene's first 32-pixel tile in the batch
};

struct BatchLaunch {
    const BatchItem *items;        // device array, n_items long
    int n_items;
    uint64_t total_tiles;
    unsigned long long *next_tile; // device work counter (reset by launch_batch_pt)
    uint32_t tile_w, tile_h;       // tile_w * tile_h == 32
    unsigned long long *counters;  // optional: [paths, segments] accumulated
    bool kajiya;                   // every item runs mode 0 (the per-lane state machine serves them)
};

// Memset of the work counter + the persistent kernel (both on `stream`).
cudaError_t launch_batch_pt(const BatchLaunch &B, int block_threads, int blocks, int stack_entries,
                            cudaStream_t stream);
// Resident blocks per SM of the batch kernel for a block size, stack depth
// and kernel (kajiya: the mode-0 kernel).
cudaError_t batch_max_blocks_per_sm(int block_threads, int stack_entries, bool kajiya, int *blocks);

}  // namespace pray_gpu
