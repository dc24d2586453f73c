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

// Modes 0 and 1 bounce by bounce (pt_sync). The per-lane state machine
// that the batch kernel runs for mode 0 measured slower here: 176.6 against
// 194.7 Msamples/s on the closed room, 653 against 863 on a 20k-triangle
// sphere (at 8 blocks of 128 threads per SM, 64 registers).
// Pixels of the frame in warp-tile order (pixel_of) from a counter: the lanes
// of a warp whose pixel is done take the next slots together (one atomic), so
// they do not wait for the warp's longest path. Warp-uniform state.
struct FrameSrc {
    unsigned long long *next;
    uint64_t slots;
    uint32_t width, height;
    bool done;
    __device__ __forceinline__ bool drained() const { return done; }
    __device__ __forceinline__ bool take(bool want, uint32_t &x, uint32_t &y) {
        constexpr unsigned kFull = 0xFFFFFFFFu;
        const unsigned ask = __ballot_sync(kFull, want);
        unsigned long long base = 0;
        if ((threadIdx.x & 31u) == 0) base = atomicAdd(next, (unsigned long long)__popc(ask));
        base = __shfl_sync(kFull, base, 0);
        if (base + __popc(ask) >= slots) done = true;
        const uint64_t slot = base + __popc(ask & ((1u << (threadIdx.x & 31u)) - 1u));
        if (!want || slot >= slots) return false;
        return pixel_of(slot, width, height, x, y);
    }
};

// kRefill (mode 1): a persistent grid whose lanes take pixels from the
// frame's counter (512^2 at 1 spp: 1.68 -> 1.49 ms; room 1024^2 at 64 spp
// unchanged). Mode 0 keeps one pixel per lane: refilled, it measured 6 %
// slower on the room. kBlocks: resident blocks per SM (the register cap).
// Long frames run 10 (48 registers); a frame of fewer paths than two rounds
// of those lanes is bound by its last paths, which run faster with more
// registers and fewer spills: 8 blocks (64 registers) take 512^2 at 1 spp
// from 1.231 to 1.186 ms, where the 1024^2 x 64-spp room drops from 200.2
// to 191.0 Msamples/s.
template <bool kRefill, int kBlocks>
__global__ void __launch_bounds__(128, kBlocks) k_render_pt(DevScene s, PtLaunch L) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    uint32_t segments = 0, pixels = 0;
    if (kRefill) {
        FrameSrc src{L.next_pixel, warp_tiles(L.cam.width, L.cam.height) * 32, L.cam.width, L.cam.height, false};
        pt_sync<kStack>(s, L, src, segments, pixels);
    } else {
        const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        uint32_t px, py;
        const bool active = pixel_of(i, L.cam.width, L.cam.height, px, py);
        OnePixel src{active, px, py, false};
        pt_sync<kStack>(s, L, src, segments, pixels);
    }
    if (L.counters) {
        unsigned long long paths = (unsigned long long)pixels * L.num_samples, segs = segments;
        for (int o = 16; o > 0; o >>= 1) {
            paths += __shfl_xor_sync(kFull, paths, o);
            segs += __shfl_xor_sync(kFull, segs, o);
        }
        if ((threadIdx.x & 31u) == 0) {
            atomicAdd(L.counters + 0, paths);
            atomicAdd(L.counters + 1, segs);
        }
    }
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

cudaError_t launch_render_pt(const DevScene &s, const PtLaunch &L, int sm_count, cudaStream_t stream) {
    const uint64_t tiles = warp_tiles(L.cam.width, L.cam.height);
    const uint64_t threads = tiles * 32;
    if (threads == 0) return cudaSuccess;
    const unsigned bs = 128;
    const uint64_t blocks = (threads + bs - 1) / bs;
    if (L.mode == 2) {
        k_render_pt_diffuse<<<(unsigned)blocks, bs, 0, stream>>>(s, L);
    } else if (L.mode == 1) {
        if (!L.next_pixel) return cudaErrorInvalidValue;
        // persistent: as many blocks as stay resident, or fewer
        const uint64_t sms = (uint64_t)(sm_count > 0 ? sm_count : 1);
        const uint64_t paths = (uint64_t)L.cam.width * L.cam.height * L.num_samples;
        if (paths < 2 * sms * 10 * bs) {
            const uint64_t resident = sms * 8;
            k_render_pt<true, 8><<<(unsigned)(blocks < resident ? blocks : resident), bs, 0, stream>>>(s, L);
        } else {
            const uint64_t resident = sms * 10;
            k_render_pt<true, 10><<<(unsigned)(blocks < resident ? blocks : resident), bs, 0, stream>>>(s, L);
        }
    } else {
        k_render_pt<false, 10><<<(unsigned)blocks, bs, 0, stream>>>(s, L);
    }
    return cudaGetLastError();
}

}  // namespace pray_gpu
