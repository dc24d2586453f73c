// Allocation-free variant of the wavefront path tracer.
//
// Some host applications cannot let this library allocate device memory while
// they render a frame: engines that reserve all GPU memory up front for their
// own pool allocator (a cudaMalloc then fails or fragments their pool), and
// frame loops with hard latency budgets, where cudaMalloc / cudaFree may
// synchronise the device. For them this file keeps the wavefront scheduler's
// scratch (path pool, queues, per-pixel running sums) in one statically
// sized device array instead of memory allocated on first use.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds its kNoAllocScratchBytes (160 MiB) until the process exits.
// Host code cannot use the array's name as a device address; the first call on
// each device looks the address up with cudaGetSymbolAddress (with that device
// current) and caches it, and every launch gets the address as a parameter.
// The same first call also loads every kernel a frame may launch (both
// traversal-stack depths), so module loading happens there and nowhere later;
// make that first call before any stream capture.
//
// All calls share the one array and it keeps the last call's contents. Nothing
// in it needs to start at zero: the init pass of every round writes all path
// state and the queue counters, and the first round overwrites the per-pixel
// sums. Calls whose work overlaps on the GPU (different streams, or different
// host threads without ordering) race on the array; callers must order them.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "device_layout.h"
#include "trace_launch.h"

namespace pray_gpu {

namespace {

constexpr uint64_t kNoAllocScratchBytes = 160ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

}  // namespace

uint64_t noalloc_max_pixels() {
    // smallest pool: one path per pixel
    uint64_t lo = 0, hi = kNoAllocScratchBytes / 64;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) / 2;
        if (wavefront_scratch_bytes(mid, mid) <= kNoAllocScratchBytes) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

cudaError_t launch_wavefront_noalloc(const DevScene &s, const PtLaunch &L, uint64_t max_paths, cudaStream_t stream,
                                     std::string &why) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) {
        why = "device index beyond the allocation-free path's table";
        return cudaErrorInvalidDevice;
    }
    void *base = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                why = "cudaGetSymbolAddress of the static scratch failed";
                return e;
            }
            int n = 0;
            e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            e = wavefront_preload_kernels();
            if (e != cudaSuccess) {
                why = "loading the wavefront kernels failed";
                return e;
            }
            g_scratch_addr[dev] = p;
            g_sm_count[dev] = n;
        }
        base = g_scratch_addr[dev];
        sms = g_sm_count[dev];
    }
    const uint64_t P = (uint64_t)L.cam.width * L.cam.height;
    if (wavefront_scratch_bytes(P, P) > kNoAllocScratchBytes) {
        why = "frame of " + std::to_string(P) + " pixels exceeds the allocation-free path's limit of " +
              std::to_string(noalloc_max_pixels()) + " pixels (160 MiB of static scratch)";
        return cudaErrorInvalidValue;
    }
    // largest pool that fits, capped by the request and by what one frame needs
    uint64_t want = P * (uint64_t)L.num_samples;
    if (max_paths && max_paths < want) want = max_paths;
    if (want < P) want = P;
    uint64_t lo = P, hi = want;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) / 2;
        if (wavefront_scratch_bytes(mid, P) <= kNoAllocScratchBytes) lo = mid;
        else hi = mid - 1;
    }
    const WavefrontScratch w = wavefront_carve(base, lo, P);
    return record_wavefront_frame(s, L, w, sms, stream);
}

}  // namespace pray_gpu
