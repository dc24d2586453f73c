// 3x3 convolution forward on the 5th-generation tensor cores (tcgen05), BF16
// operands, FP32 accumulation in tensor memory (TMEM).
//
// Implicit GEMM without an im2col copy. One CTA (4 warps) computes a tile of
// 16 x 8 output pixels (M = 128) x all output channels (N = Cout rounded up
// to 16). The input halo of the tile, 18 x 10 pixels x Cin, is loaded once
// by TMA (one 4-D tiled copy per 8-channel chunk; out-of-image pixels arrive
// as zeros, which is the convolution's padding) into planes of
// [y][x][8 channels] (16 bytes per pixel). In that layout the A operand of
// tap (dy, dx) for 16 channels is the halo itself seen through a shared-memory
// matrix descriptor: the tile's 8-pixel rows are the 8-row core-matrix
// groups (stride 160 bytes = one halo row), the two 8-channel chunks are the
// K-direction core matrices (stride = one plane), and the start address moves
// by (dy * 10 + dx) * 16 bytes. So all nine taps read the same halo and the
// threads gather nothing. The weights are packed once (tc_pack_weights) as
// [tap][8-channel chunk][row][8] BF16 — exactly the no-swizzle K-major
// core-matrix layout — and copied with plain bulk copies, all taps at once
// when they fit or through a ring of per-tap stages. One thread issues the
// kind::f16 MMAs (M 128, N Npad, K 16) and commits them to mbarriers.
//
// The deep, small levels have too few tiles for 152 SMs: there each tile's
// output channels are split over CTAs (each loads its slice of the weights
// with one 3-D TMA box), or, for a single 16-channel chunk, the nine taps over
// 3 or 9 CTAs, each writing FP32 partial sums that a second kernel adds in
// split order (deterministic) with the bias and ReLU.
//
// The epilogue also performs the network's glue (TcFuse): 2 x 2 average
// pooling, nearest 2x upsampling into a concatenation, the residual add and
// the output transform, as extra stores of the values it holds.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error,
// stops issuing, waits (bounded) for the copies and MMAs it issued, and frees
// its TMEM.
#include <atomic>
#include <cstdint>
#include <cstring>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "denoise_ops.h"

namespace pray_gpu {
namespace dn {

static_assert(sizeof(CUtensorMap) == sizeof(TcConvPlan::tmap), "tensor map size");

namespace {

constexpr int kTileW = 8, kTileH = 16;
constexpr int kHaloW = kTileW + 2, kHaloH = kTileH + 2;
constexpr uint32_t kChunkBytes = kHaloW * kHaloH * 16;  // one 8-channel halo plane (2880)
constexpr uint32_t kPlaneBytes = 2944;                  // plane stride, 128-byte aligned
constexpr uint32_t kRowBytes = kHaloW * 16;             // one halo row of one plane (160)
constexpr uint32_t kWaitLimit = 1u << 24;
constexpr size_t kSmemBudget = 110 * 1024;              // target per CTA (two or more CTAs per SM)
constexpr size_t kSmemPersistent = 200 * 1024;          // persistent kernel: up to one CTA per SM
constexpr size_t kSmemMax = 227 * 1024;
constexpr size_t kSmemPerSm = 228 * 1024;

struct TcArgs {
    const __nv_bfloat16 *w;  // packed weights [tap][chunk][npad][8]
    const float *bias;
    __nv_bfloat16 *y;
    float *y32;
    float *partial;          // [split][M][npad] when splits > 1
    int n, h, wd, cin, cout, npad, relu;
    int tiles_x, tiles_y;
    int taps_per_split, taps_per_stage, stages;
    int nsplit;               // > 1: blockIdx.y picks output channels [y * npad, (y + 1) * npad), all taps,
                              // the weight slice by TMA (wmap) from the packing of npad_full rows
    int npad_full;
    int tmem_cols;
    uint32_t w_off, bar_off;  // shared-memory offsets (the halo is at 0)
    uint32_t halo_stride;     // persistent kernel: distance between the halo ring's slots
    int *err;
    TcFuse f;                 // extra stores of the epilogue
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Programmatic dependent launch. A convolution launched with programmatic
// stream serialisation may start while the previous kernel of the stream
// still runs: its prologue (barriers, tensor memory, weight copies) overlaps
// that kernel's tail, and the thread that loads the input waits here for the
// previous kernel to complete (and its writes to be visible) before the first
// input copy. Every global store of the kernel follows that wait (the
// epilogue runs after the MMAs, which follow the input copies). Once past it,
// the CTA lets the next kernel launch. Launched without the attribute, both
// instructions return at once.
__device__ __forceinline__ void grid_dependency_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Shared-memory matrix descriptor: start, leading (K-direction) and stride
// (8-row group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M.
__host__ __device__ constexpr uint32_t inst_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One 8-channel chunk of the halo: box (8 channels, 10 x, 18 y, 1 image) at
// (c, x, y, img); x and y may be -1 (zero fill).
__device__ __forceinline__ void tma_halo(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c, int x, int y,
                                         int img) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, "
        "%6}], [%2];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c), "r"(x), "r"(y), "r"(img)
        : "memory");
}

// A slice of packed weights: box (8 channels, npad rows, taps x chunks) of the
// 3-D map (8, npad_full, 9 x cin / 8) at rows from n, (tap, chunk) from k.
__device__ __forceinline__ void tma_w(uint32_t dst, const CUtensorMap *map, uint32_t bar, int n, int k) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(0), "r"(n), "r"(k)
        : "memory");
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// Epilogue of one tile: the calling warp reads TMEM lanes 32q..32q+31 (q =
// quad, the warp's lane quadrant: its warp index mod 4; tile rows m = pixel
// (m / 8, m % 8)) from column `tmem` on, 16 columns at a time, and stores
// bias + ReLU + BF16 (16-byte stores), FP32, or raw FP32 partials, plus the
// extra stores of P.f. A warp holds four whole tile rows, so the 2 x 2 blocks
// of the pooling are lanes (l, l + 1, l + 8, l + 9) for l with even row and
// column, summed in the order of k_avgpool (row-major).
__device__ __forceinline__ void epilogue(const TcArgs &P, uint32_t tmem, int img, int y0, int x0, int split,
                                         int quad, int n0 = 0) {
    const int lane = (int)(threadIdx.x & 31);
    const int m = quad * 32 + lane;
    const int yy = y0 + (m >> 3), xx = x0 + (m & 7);
    const bool valid = yy < P.h && xx < P.wd;
    const size_t M = (size_t)P.n * P.h * P.wd;
    const size_t pix = ((size_t)img * P.h + yy) * P.wd + xx;
    const bool vec = (P.y || P.f.pool || P.f.cat) && (P.cout & 15) == 0;
    for (int c0 = 0; c0 < P.npad; c0 += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // the pooling's shuffles need every lane of the warp
        if (!valid && !(vec && P.f.pool)) continue;
        if (P.partial) {
            float4 *o = reinterpret_cast<float4 *>(P.partial + ((size_t)split * M + pix) * P.npad + c0);
#pragma unroll
            for (int k = 0; k < 4; k++)
                o[k] = make_float4(__uint_as_float(r[4 * k]), __uint_as_float(r[4 * k + 1]),
                                   __uint_as_float(r[4 * k + 2]), __uint_as_float(r[4 * k + 3]));
        } else if (vec) {
            float v[16];
#pragma unroll
            for (int k = 0; k < 16; k++) {
                v[k] = __uint_as_float(r[k]) + __ldg(P.bias + n0 + c0 + k);
                if (P.relu) v[k] = fmaxf(v[k], 0.f);
            }
            const uint4 lo = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
            const uint4 hi =
                make_uint4(pack2(v[8], v[9]), pack2(v[10], v[11]), pack2(v[12], v[13]), pack2(v[14], v[15]));
            if (valid && P.y) {
                uint4 *o = reinterpret_cast<uint4 *>(P.y + pix * P.cout + n0 + c0);
                o[0] = lo, o[1] = hi;
            }
            if (valid && P.f.cat) {
                const int ch = P.f.cat_off + n0 + c0;
                if (P.f.cat_up) {
                    const size_t W2 = 2 * (size_t)P.wd;
                    const size_t b = (((size_t)img * 2 * P.h + 2 * yy) * W2 + 2 * xx) * P.f.cat_c + ch;
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        uint4 *o = reinterpret_cast<uint4 *>(P.f.cat + b + ((q >> 1) * W2 + (q & 1)) * P.f.cat_c);
                        o[0] = lo, o[1] = hi;
                    }
                } else {
                    uint4 *o = reinterpret_cast<uint4 *>(P.f.cat + pix * P.f.cat_c + ch);
                    o[0] = lo, o[1] = hi;
                }
            }
            if (P.f.pool) {
                const uint32_t wd[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
                uint32_t po[8];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const __nv_bfloat162 a2 = *reinterpret_cast<const __nv_bfloat162 *>(&wd[k]);
                    const float a0 = __low2float(a2), a1 = __high2float(a2);
                    const float b0 = __shfl_down_sync(0xFFFFFFFFu, a0, 1), b1 = __shfl_down_sync(0xFFFFFFFFu, a1, 1);
                    const float c0v = __shfl_down_sync(0xFFFFFFFFu, a0, 8);
                    const float c1v = __shfl_down_sync(0xFFFFFFFFu, a1, 8);
                    const float d0 = __shfl_down_sync(0xFFFFFFFFu, a0, 9), d1 = __shfl_down_sync(0xFFFFFFFFu, a1, 9);
                    po[k] = pack2(0.25f * (a0 + b0 + c0v + d0), 0.25f * (a1 + b1 + c1v + d1));
                }
                const int ho = P.h >> 1, wo = P.wd >> 1, yo = yy >> 1, xo = xx >> 1;
                if (((lane >> 3) & 1) == 0 && (lane & 1) == 0 && yo < ho && xo < wo) {
                    uint4 *o = reinterpret_cast<uint4 *>(P.f.pool + (((size_t)img * ho + yo) * wo + xo) * P.cout +
                                                         n0 + c0);
                    o[0] = make_uint4(po[0], po[1], po[2], po[3]);
                    o[1] = make_uint4(po[4], po[5], po[6], po[7]);
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < 16; k++) {
                const int co = n0 + c0 + k;
                if (co >= P.cout) break;
                float v = __uint_as_float(r[k]) + __ldg(P.bias + co);
                if (P.relu) v = fmaxf(v, 0.f);
                if (P.y) P.y[pix * P.cout + co] = __float2bfloat16(v);
                if (P.f.res) v += __bfloat162float(P.f.res[pix * P.f.res_c + co]);
                if (P.y32) P.y32[pix * P.cout + co] = v;
                if (P.f.rad)
                    P.f.rad[pix * 3 + co] =
                        expm1f(v) * (fmaxf(__half2float(P.f.feat[7 * pix + co]), 0.f) + kDemodFloor);
            }
        }
    }
}

__global__ void __launch_bounds__(128) k_conv_tc(const __grid_constant__ CUtensorMap xmap,
                                                 const __grid_constant__ CUtensorMap wmap, TcArgs P) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int nchunk = P.cin >> 3;
    const uint32_t halo = smem_u32(smem), wbase = halo + P.w_off;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + P.bar_off);
    // bars[0] halo loaded, bars[1] all MMAs done, bars[2 + s] stage s loaded,
    // bars[2 + stages + s] stage s consumed by its MMAs
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 + 2 * P.stages);
    int *okflag = reinterpret_cast<int *>(tmem_slot + 1);
    auto bar = [&](int i) { return smem_u32(&bars[i]); };

    const int per_img = P.tiles_x * P.tiles_y;
    const int img = blockIdx.x / per_img, rem = blockIdx.x - img * per_img;
    const int y0 = (rem / P.tiles_x) * kTileH, x0 = (rem % P.tiles_x) * kTileW;
    // tap split (nsplit 1): blockIdx.y picks a group of taps; output-channel
    // split: all taps, channels from n0
    const int split = P.nsplit > 1 ? 0 : blockIdx.y;
    const int n0 = P.nsplit > 1 ? (int)blockIdx.y * P.npad : 0;
    const int t0 = split * P.taps_per_split;
    const int nloads = P.taps_per_split / P.taps_per_stage;
    const int kchunks = P.cin >> 3;  // 8-channel chunks per tap (the weight map's third coordinate)
    const uint32_t wtap_bytes = (uint32_t)P.cin * P.npad * 2;
    const uint32_t stage_bytes = wtap_bytes * P.taps_per_stage;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 2 + 2 * P.stages; i++) mbar_init(bar(i));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (tid == 0) {
        bool ok = true;
        // weights: the first `stages` loads; with the output-channel split, one
        // TMA box per load: rows n0..n0+npad of every (tap, chunk) of the stage
        int issued = 0;
        const __nv_bfloat16 *wsrc = P.w + (size_t)t0 * P.cin * P.npad;
        auto load_weights = [&](int stage, int load) {
            mbar_expect_tx(bar(2 + stage), stage_bytes);
            if (P.nsplit > 1)
                tma_w(wbase + stage * stage_bytes, &wmap, bar(2 + stage), n0,
                      (t0 + load * P.taps_per_stage) * kchunks);
            else
                bulk_copy(wbase + stage * stage_bytes, wsrc + (size_t)load * P.taps_per_stage * P.cin * P.npad,
                          stage_bytes, bar(2 + stage));
        };
        for (; issued < nloads && issued < P.stages; issued++) load_weights(issued, issued);
        // the weights do not depend on the previous kernel; the input does
        grid_dependency_wait();
        // halo: one copy per 8-channel chunk, all completing on bars[0]
        mbar_expect_tx(bar(0), (uint32_t)nchunk * kChunkBytes);
        for (int c = 0; c < nchunk; c++) tma_halo(halo + c * kPlaneBytes, &xmap, bar(0), 8 * c, x0 - 1, y0 - 1, img);
        const bool halo_done = mbar_wait(bar(0), 0);
        ok = halo_done;
        const uint32_t idesc = inst_desc(128, P.npad);
        int consumed = 0;
        for (int j = 0; j < nloads && ok; j++) {
            const int s = j % P.stages;
            if (!mbar_wait(bar(2 + s), (uint32_t)(j / P.stages) & 1)) {
                ok = false;
                break;
            }
            consumed = j + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int q = 0; q < P.taps_per_stage; q++) {
                const int tap = t0 + j * P.taps_per_stage + q;
                const int dy = tap / 3, dx = tap - 3 * (tap / 3);
                const uint32_t a0 = halo + (uint32_t)(dy * kHaloW + dx) * 16;
                const uint32_t b0 = wbase + s * stage_bytes + q * wtap_bytes;
                for (int p = 0; p < nchunk / 2; p++) {
                    const uint64_t ad = smem_desc(a0 + 2 * p * kPlaneBytes, kPlaneBytes, kRowBytes);
                    const uint64_t bd = smem_desc(b0 + 2 * p * P.npad * 16, P.npad * 16, 128);
                    mma(tmem, ad, bd, idesc, (j | q | p) != 0 ? 1u : 0u);
                }
            }
            commit(bar(2 + P.stages + s));
            // refill the stage of the previous load once its MMAs are done
            // (this load's MMAs are queued behind them)
            if (j >= 1 && issued < nloads) {
                const int jp = j - 1, sp = jp % P.stages;
                if (!mbar_wait(bar(2 + P.stages + sp), (uint32_t)(jp / P.stages) & 1)) {
                    ok = false;
                    break;
                }
                load_weights(sp, issued);
                issued++;
            }
        }
        // all MMAs issued so far complete on bars[1]
        commit(bar(1));
        if (!ok) {
            // drain copies still in flight (bounded) before the shared memory goes away
            if (!halo_done) mbar_wait(bar(0), 0);
            for (int j = consumed; j < issued; j++) mbar_wait(bar(2 + j % P.stages), (uint32_t)(j / P.stages) & 1);
        }
        *okflag = ok ? 1 : 0;
    }
    __syncthreads();
    const bool ok = mbar_wait(bar(1), 0) && *okflag;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (!ok && tid == 0) atomicExch(P.err, 1);
    if (ok) epilogue(P, tmem, img, y0, x0, split, warp, n0);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P.tmem_cols)
                     : "memory");
    }
}

__device__ __forceinline__ void mbar_init_count(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

constexpr int kWsThreads = 192;  // warp 0 loads, warp 1 issues MMAs, warps 2-5 drain accumulators

// Persistent, warp-specialised variant for levels that need no tap split and
// whose weights fit in shared memory beside a ring of halos. Each CTA loads
// the weights once and walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...:
//   warp 0 (one thread) loads tile i's halo into ring slot i % H once the
//     MMAs of tile i - H have released it;
//   warp 1 (one thread) waits for the halo and for accumulator i % 2 to be
//     drained, issues the tile's MMAs into it and commits them to the slot's
//     "released" and the accumulator's "full" barriers;
//   warps 2-5 (one TMEM lane quadrant each) drain accumulator i % 2 to
//     global memory and release it.
// So halo loads, MMAs and epilogues of consecutive tiles overlap. Every wait
// is bounded; a timeout sets a shared abort flag that ends every role's
// loop, and the copies and MMAs in flight are waited for (bounded) before
// the shared memory and TMEM are released.
__global__ void __launch_bounds__(kWsThreads) k_conv_tc_persistent(const __grid_constant__ CUtensorMap xmap,
                                                                   TcArgs P) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int H = P.stages;  // halo ring slots
    const int nchunk = P.cin >> 3;
    const uint32_t halo0 = smem_u32(smem), wbase = halo0 + P.w_off;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + P.bar_off);
    // bars: [0, H) halo loaded, [H, 2H) halo released, 2H + a accumulator
    // full, 2H + 2 + a accumulator drained, 2H + 4 weights loaded, 2H + 5
    // final drain of the MMAs
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * H + 6);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    volatile int *issued = reinterpret_cast<volatile int *>(tmem_slot + 2);    // halos loaded so far
    volatile int *consumed = reinterpret_cast<volatile int *>(tmem_slot + 3);  // halos the MMA warp waited for
    volatile int *w_waited = reinterpret_cast<volatile int *>(tmem_slot + 4);
    auto bar = [&](int i) { return smem_u32(&bars[i]); };
    const int full0 = 0, empty0 = H, accf0 = 2 * H, acce0 = 2 * H + 2, wbar = 2 * H + 4, dbar = 2 * H + 5;
    const int per_img = P.tiles_x * P.tiles_y;
    const int tiles = P.n * per_img;
    const int items = tiles > (int)blockIdx.x ? (tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile_of = [&](int i, int &img, int &y0, int &x0) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        img = t / per_img;
        const int rem = t - img * per_img;
        y0 = (rem / P.tiles_x) * kTileH;
        x0 = (rem % P.tiles_x) * kTileW;
    };
    const uint32_t wbytes = (uint32_t)P.cin * P.npad * 2 * 9;
    const int acc_stride = (P.npad + 31) & ~31;  // TMEM columns between the two accumulators

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 2 * H; i++) mbar_init(bar(i));
        mbar_init(bar(accf0)), mbar_init(bar(accf0 + 1));
        mbar_init_count(bar(acce0), 128), mbar_init_count(bar(acce0 + 1), 128);
        mbar_init(bar(wbar)), mbar_init(bar(dbar));
        *abort_flag = 0, *issued = 0, *consumed = 0, *w_waited = 0;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0 && items > 0) {
            mbar_expect_tx(bar(wbar), wbytes);
            bulk_copy(wbase, P.w, wbytes, bar(wbar));
            grid_dependency_wait();
            for (int i = 0; i < items && !*abort_flag; i++) {
                const int h = i % H;
                if (i >= H && !mbar_wait(bar(empty0 + h), (uint32_t)((i / H) - 1) & 1)) {
                    *abort_flag = 1;
                    break;
                }
                int img, y0, x0;
                tile_of(i, img, y0, x0);
                const uint32_t dst = halo0 + (uint32_t)h * P.halo_stride;
                mbar_expect_tx(bar(full0 + h), (uint32_t)nchunk * kChunkBytes);
                for (int c = 0; c < nchunk; c++)
                    tma_halo(dst + c * kPlaneBytes, &xmap, bar(full0 + h), 8 * c, x0 - 1, y0 - 1, img);
                *issued = i + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && items > 0) {
            bool ok = mbar_wait(bar(wbar), 0);
            *w_waited = 1;
            if (!ok) *abort_flag = 1;
            const uint32_t idesc = inst_desc(128, P.npad);
            for (int i = 0; i < items && ok && !*abort_flag; i++) {
                const int h = i % H, a = i & 1;
                if (!mbar_wait(bar(full0 + h), (uint32_t)(i / H) & 1)) {
                    *abort_flag = 1;
                    break;
                }
                *consumed = i + 1;
                if (i >= 2 && !mbar_wait(bar(acce0 + a), (uint32_t)((i >> 1) - 1) & 1)) {
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(a * acc_stride);
                const uint32_t hb = halo0 + (uint32_t)h * P.halo_stride;
                for (int tap = 0; tap < 9; tap++) {
                    const int dy = tap / 3, dx = tap - 3 * (tap / 3);
                    const uint32_t a0 = hb + (uint32_t)(dy * kHaloW + dx) * 16;
                    const uint32_t b0 = wbase + (uint32_t)tap * P.cin * P.npad * 2;
                    for (int p = 0; p < nchunk / 2; p++) {
                        const uint64_t ad = smem_desc(a0 + 2 * p * kPlaneBytes, kPlaneBytes, kRowBytes);
                        const uint64_t bd = smem_desc(b0 + 2 * p * P.npad * 16, P.npad * 16, 128);
                        mma(acc, ad, bd, idesc, (tap | p) != 0 ? 1u : 0u);
                    }
                }
                commit(bar(empty0 + h));
                commit(bar(accf0 + a));
            }
            // everything this thread issued completes before TMEM is freed
            commit(bar(dbar));
            mbar_wait(bar(dbar), 0);
        }
    } else {
        const int quad = warp & 3;  // warps 2, 3, 4, 5 -> TMEM lane quadrants 2, 3, 0, 1
        // every decision warp-uniform: the TMEM loads below are warp-collective
        for (int i = 0; i < items; i++) {
            if (__any_sync(0xFFFFFFFFu, *abort_flag != 0)) break;
            const int a = i & 1;
            if (!__all_sync(0xFFFFFFFFu, mbar_wait(bar(accf0 + a), (uint32_t)(i >> 1) & 1))) {
                if (lane == 0) *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            int img, y0, x0;
            tile_of(i, img, y0, x0);
            epilogue(P, tmem + (uint32_t)(a * acc_stride), img, y0, x0, 0, quad);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(bar(acce0 + a));
        }
    }
    __syncthreads();
    if (tid == 0 && *abort_flag) {
        atomicExch(P.err, 1);
        // copies still in flight (bounded) before the shared memory goes away
        if (items > 0 && !*w_waited) mbar_wait(bar(wbar), 0);
        for (int j = *consumed; j < *issued; j++) mbar_wait(bar(full0 + j % H), (uint32_t)(j / H) & 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P.tmem_cols)
                     : "memory");
    }
}

// Sum of the split partials in split order, plus bias, ReLU, store; four
// channels per thread when cout is a multiple of 4, else one.
// ---- weight gradient ---------------------------------------------------------
//
// dw[co][tap][ci] = sum_p g[p][co] x[p + offset(tap)][ci]: per tap a GEMM with
// M = co (128 rows: the output-gradient channels, zero rows above cout),
// N = ci (cin_pad), K = pixels. Both operands come straight from the
// channel-planar tiles TMA writes ([8-channel plane][pixel][8 channels], 16
// bytes per pixel), read as MN-major matrices (the 8 channels of a pixel
// contiguous, pixels along K):
//   A: the tile's output gradient, one 2,048-byte plane per 8 channels
//      (16 x 8 pixels); core matrices 128 bytes apart along K (8 pixels = one
//      tile row) and one plane apart along M;
//   B: the input halo (18 x 10 pixels per plane, as in the forward pass);
//      for tap (dy, dx) the K-step covering tile rows 2k and 2k + 1 starts at
//      halo pixel (2k + dy, dx), core matrices one halo row (160 bytes) apart
//      along K and one plane apart along N.
// So every tap reads the same halo, shifted by whole 16-byte pixels, as in
// the forward pass. Each CTA owns a group of tiles and a group of taps
// (tensor memory holds taps_per_pass x cin_pad FP32 columns). One thread
// loads the tiles into two shared-memory stages, the next tile's planes
// while the tensor cores work on this one's (one stage where two do not
// fit), and issues the MMAs. The accumulators of the output channels below
// cout go to partial[group][tap][co][ci]; k_wgrad_finalize adds the groups in
// order into dw. Every wait is bounded (error flag, drain, TMEM freed).
constexpr uint32_t kGradPlaneBytes = kTileW * kTileH * 16;  // 2,048
constexpr int kGradPlanes = 16;                             // 128 rows of A

struct WgArgs {
    float *partial;  // [group][9][cout][cin_pad]
    int n, h, wd, cin_pad, cout, cout_pad;
    int tiles_x, tiles_y, tiles, tiles_per_cta, taps_per_pass, tmem_cols, stages;
    uint32_t b_off, stage_bytes, bar_off;
    int *err;
};

// MN-major A and B: transpose bits of the kind::f16 instruction descriptor
__host__ __device__ constexpr uint32_t inst_desc_mn(int m, int n) { return inst_desc(m, n) | (1u << 15) | (1u << 16); }

// One plane (8 channels) of a tile of the output gradient: box (8, 8, 16, 1).
__device__ __forceinline__ void tma_tile(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c, int x, int y,
                                         int img) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, "
        "%6}], [%2];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c), "r"(x), "r"(y), "r"(img)
        : "memory");
}

__global__ void __launch_bounds__(128) k_wgrad_tc(const __grid_constant__ CUtensorMap gmap,
                                                  const __grid_constant__ CUtensorMap xmap, WgArgs P) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int S = P.stages;
    const uint32_t base = smem_u32(smem);
    // bars[s] stage s loaded, bars[2 + s] MMAs reading stage s done, bars[4] drain
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + P.bar_off);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 5);
    int *okflag = reinterpret_cast<int *>(tmem_slot + 1);
    const int gplanes = P.cout_pad >> 3, xplanes = P.cin_pad >> 3;
    const int group = blockIdx.x, pass = blockIdx.y;
    const int tap0 = pass * P.taps_per_pass, ntaps = min(9 - tap0, P.taps_per_pass);
    const int t_begin = group * P.tiles_per_cta, t_end = min(P.tiles, t_begin + P.tiles_per_cta);
    auto abase = [&](int st) { return base + (uint32_t)st * P.stage_bytes; };
    auto bar = [&](int i) { return smem_u32(&bars[i]); };

    // the rows of A above cout_pad stay zero, in every stage
    for (int st = 0; st < S; st++)
        for (uint32_t i = (uint32_t)gplanes * kGradPlaneBytes / 16 + tid; i < kGradPlanes * kGradPlaneBytes / 16;
             i += 128)
            reinterpret_cast<uint4 *>(smem + (size_t)st * P.stage_bytes)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 5; i++) mbar_init(bar(i));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the zero rows, for the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (tid == 0) {
        bool ok = true;
        const uint32_t idesc = inst_desc_mn(128, P.cin_pad);
        const uint32_t bytes = (uint32_t)gplanes * kGradPlaneBytes + (uint32_t)xplanes * kChunkBytes;
        const int per_img = P.tiles_x * P.tiles_y;
        const int n = t_end > t_begin ? t_end - t_begin : 0;
        // tile i of the group goes to stage i % S; issue() starts its loads
        auto issue = [&](int i) {
            const int t = t_begin + i, st = i % S;
            const int img = t / per_img, rem = t - img * per_img;
            const int y0 = (rem / P.tiles_x) * kTileH, x0 = (rem % P.tiles_x) * kTileW;
            const uint32_t a = abase(st), b = a + P.b_off;
            mbar_expect_tx(bar(st), bytes);
            for (int c = 0; c < gplanes; c++) tma_tile(a + c * kGradPlaneBytes, &gmap, bar(st), 8 * c, x0, y0, img);
            for (int c = 0; c < xplanes; c++)
                tma_halo(b + c * kPlaneBytes, &xmap, bar(st), 8 * c, x0 - 1, y0 - 1, img);
        };
        int issued = 0, consumed = 0, committed = 0;
        if (n > 0) issue(issued++);
        for (int i = 0; i < n && ok; i++) {
            const int st = i % S;
            // with two stages, load tile i + 1 into the other stage as soon as
            // the MMAs of tile i - 1, which read it, are done
            if (S == 2 && i + 1 < n) {
                if (i >= 1 && !mbar_wait(bar(2 + (st ^ 1)), (uint32_t)((i - 1) / 2) & 1u)) {
                    ok = false;
                    break;
                }
                issue(issued++);
            }
            if (!mbar_wait(bar(st), (uint32_t)(i / S) & 1u)) {
                ok = false;
                break;
            }
            consumed = i + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = abase(st), b = a + P.b_off;
            for (int q = 0; q < ntaps; q++) {
                const int tap = tap0 + q, dy = tap / 3, dx = tap - 3 * (tap / 3);
                const uint32_t d = tmem + (uint32_t)(q * P.cin_pad);
                for (int k = 0; k < kTileH / 2; k++) {
                    const uint64_t ad = smem_desc(a + (uint32_t)k * 256u, 128u, kGradPlaneBytes);
                    const uint64_t bd =
                        smem_desc(b + (uint32_t)((2 * k + dy) * kHaloW + dx) * 16u, kRowBytes, kPlaneBytes);
                    mma(d, ad, bd, idesc, (i == 0 && k == 0) ? 0u : 1u);
                }
            }
            commit(bar(2 + st));
            committed = i + 1;
            if (S == 1) {
                // one stage: the next load waits for this tile's MMAs
                if (!mbar_wait(bar(2), (uint32_t)i & 1u)) {
                    ok = false;
                    break;
                }
                if (i + 1 < n) issue(issued++);
            }
        }
        if (ok && n > 0 && S == 2 && !mbar_wait(bar(2 + (n - 1) % 2), (uint32_t)((n - 1) / 2) & 1u)) ok = false;
        *okflag = !ok ? 0 : (n == 0 ? 2 : 1);  // 2: no tile in this group
        if (!ok) {
            // bounded drain: copies still in flight, then every MMA issued
            for (int j = consumed; j < issued; j++) mbar_wait(bar(j % S), (uint32_t)(j / S) & 1u);
            if (committed > 0) {
                commit(bar(4));
                mbar_wait(bar(4), 0);
            }
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int flag = *okflag;
    if (flag == 0 && tid == 0) atomicExch(P.err, 1);
    // epilogue: warp q reads TMEM lanes 32q..32q+31 (rows co), all columns;
    // rows from cout on are zero padding and are not stored
    const int co = warp * 32 + (tid & 31);
    for (int q = 0; q < ntaps && warp * 32 < P.cout; q++) {
        float *dst = P.partial + (((size_t)group * 9 + tap0 + q) * P.cout + co) * P.cin_pad;
        for (int c0 = 0; c0 < P.cin_pad; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(q * P.cin_pad + c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (co >= P.cout) continue;
            float4 *o = reinterpret_cast<float4 *>(dst + c0);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float v0 = flag == 1 ? __uint_as_float(r[4 * k]) : 0.f;
                const float v1 = flag == 1 ? __uint_as_float(r[4 * k + 1]) : 0.f;
                const float v2 = flag == 1 ? __uint_as_float(r[4 * k + 2]) : 0.f;
                const float v3 = flag == 1 ? __uint_as_float(r[4 * k + 3]) : 0.f;
                o[k] = make_float4(v0, v1, v2, v3);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P.tmem_cols)
                     : "memory");
    }
}

// dw[co][tap][ci] += sum over groups (in order) of partial[group][tap][co][ci]
// Block of 256 threads: 32 consecutive gradient elements x 8 slices; slice
// s adds groups s, s + 8, ..., and the 8 slice sums are added in slice order
// (the same order on every run).
constexpr int kFinSlices = 8;
__global__ void k_wgrad_finalize(const float *partial, float *dw, int groups, int cout, int cin, int cin_pad) {
    __shared__ float sm[kFinSlices][32];
    const size_t total = (size_t)cout * 9 * cin;
    const int lane = (int)threadIdx.x & 31, slice = (int)threadIdx.x >> 5;
    const size_t i = (size_t)blockIdx.x * 32 + lane;
    float v = 0.f;
    if (i < total) {
        const int ci = (int)(i % cin);
        const size_t rest = i / cin;
        const int tap = (int)(rest % 9), co = (int)(rest / 9);
        for (int g = slice; g < groups; g += kFinSlices)
            v += partial[(((size_t)g * 9 + tap) * cout + co) * cin_pad + ci];
    }
    sm[slice][lane] = v;
    __syncthreads();
    if (slice == 0 && i < total) {
        float s = sm[0][lane];
        for (int k = 1; k < kFinSlices; k++) s += sm[k][lane];
        dw[i] += s;
    }
}

template <int kVec>
__global__ void k_conv_finalize(const float *partial, const float *bias, __nv_bfloat16 *y, float *y32, size_t M,
                                int npad, int cout, int splits, int relu) {
    const int groups = cout / kVec;
    const size_t total = M * (size_t)groups;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t pix = i / groups;
        const int co = kVec * (int)(i - pix * groups);
        float v[kVec];
#pragma unroll
        for (int k = 0; k < kVec; k++) v[k] = partial[pix * npad + co + k];
        for (int s = 1; s < splits; s++) {
            const float *q = partial + ((size_t)s * M + pix) * npad + co;
#pragma unroll
            for (int k = 0; k < kVec; k++) v[k] = v[k] + q[k];
        }
#pragma unroll
        for (int k = 0; k < kVec; k++) {
            v[k] = v[k] + bias[co + k];
            if (relu) v[k] = fmaxf(v[k], 0.f);
        }
        if (kVec == 4) {
            if (y) {
                uint2 o;
                o.x = pack2(v[0], v[1 % kVec]);
                o.y = pack2(v[2 % kVec], v[3 % kVec]);
                *reinterpret_cast<uint2 *>(y + pix * cout + co) = o;
            }
            if (y32)
                *reinterpret_cast<float4 *>(y32 + pix * cout + co) =
                    make_float4(v[0], v[1 % kVec], v[2 % kVec], v[3 % kVec]);
        } else {
            if (y) y[pix * cout + co] = __float2bfloat16(v[0]);
            if (y32) y32[pix * cout + co] = v[0];
        }
    }
}

// out[tap][chunk][row][8] from w[cout][9][cin] (zero rows and channels pad).
__global__ void k_pack_weights(const float *w, __nv_bfloat16 *out, int cin, int cin_pad, int cout, int npad) {
    const int nchunk = cin_pad >> 3;
    const size_t total = (size_t)9 * cin_pad * npad;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(i & 7);
        const size_t rowi = i >> 3;
        const int r = (int)(rowi % npad);
        const size_t ct = rowi / npad;
        const int chunk = (int)(ct % nchunk), tap = (int)(ct / nchunk);
        const int ci = chunk * 8 + e;
        const float v = (r < cout && ci < cin) ? w[((size_t)r * 9 + tap) * cin + ci] : 0.f;
        out[i] = __float2bfloat16(v);
    }
}

// The backward-data convolution's weights, packed like k_pack_weights: the
// input gradient of a 3x3 convolution is a 3x3 convolution of the output
// gradient (cout_f channels, padded to cin_pad) with the weights transposed
// (output channel ci, input channel co) and the taps mirrored (tap 8 - t):
// out[tap][chunk][ci][8] = w[co][8 - tap][ci], w[cout_f][9][cin_f].
__global__ void k_pack_weights_bwd(const float *w, __nv_bfloat16 *out, int cin_f, int cout_f, int cin_pad,
                                   int npad) {
    const int nchunk = cin_pad >> 3;
    const size_t total = (size_t)9 * cin_pad * npad;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(i & 7);
        const size_t rowi = i >> 3;
        const int r = (int)(rowi % npad);  // ci
        const size_t ct = rowi / npad;
        const int chunk = (int)(ct % nchunk), tap = (int)(ct / nchunk);
        const int co = chunk * 8 + e;
        const float v = (r < cin_f && co < cout_f) ? w[((size_t)co * 9 + (8 - tap)) * cin_f + r] : 0.f;
        out[i] = __float2bfloat16(v);
    }
}

__global__ void k_pack_all(const TcPackJob *jobs, int njobs, size_t total) {
    __shared__ TcPackJob sj[64];
    for (int i = (int)threadIdx.x; i < njobs; i += (int)blockDim.x) sj[i] = jobs[i];
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        int j = 0;
        while (j + 1 < njobs && sj[j + 1].begin <= i) j++;
        const TcPackJob &J = sj[j];
        const size_t li = i - J.begin;
        const int e = (int)(li & 7);
        const size_t rowi = li >> 3;
        const int r = (int)(rowi % J.npad);
        const size_t ct = rowi / J.npad;
        const int nchunk = J.cin_pad >> 3;
        const int chunk = (int)(ct % nchunk), tap = (int)(ct / nchunk);
        const int c = chunk * 8 + e;
        float v;
        if (!J.bwd)  // row r = output channel, c = input channel
            v = (r < J.cout_f && c < J.cin_f) ? J.w[((size_t)r * 9 + tap) * J.cin_f + c] : 0.f;
        else  // transposed, taps mirrored: row r = input channel, c = output channel
            v = (r < J.cin_f && c < J.cout_f) ? J.w[((size_t)c * 9 + (8 - tap)) * J.cin_f + r] : 0.f;
        J.out[li] = __float2bfloat16(v);
    }
}

unsigned grid_for(size_t n) {
    const size_t b = (n + 255) / 256;
    return (unsigned)(b < 4096 ? (b ? b : 1) : 4096);
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

}  // namespace

size_t tc_packed_weight_elems(int cin_pad, int cout) { return (size_t)9 * cin_pad * ((cout + 15) / 16 * 16); }

cudaError_t tc_pack_weights(const float *w, __nv_bfloat16 *packed, int cin, int cin_pad, int cout, cudaStream_t st) {
    const int npad = (cout + 15) / 16 * 16;
    k_pack_weights<<<grid_for(tc_packed_weight_elems(cin_pad, cout)), 256, 0, st>>>(w, packed, cin, cin_pad, cout,
                                                                                   npad);
    return cudaGetLastError();
}

cudaError_t tc_pack_all(const TcPackJob *jobs_dev, int njobs, size_t total, cudaStream_t st) {
    if (njobs <= 0 || njobs > 64) return cudaErrorInvalidValue;
    k_pack_all<<<grid_for(total), 256, 0, st>>>(jobs_dev, njobs, total);
    return cudaGetLastError();
}

cudaError_t tc_pack_weights_bwd(const float *w, __nv_bfloat16 *packed, int cin_f, int cout_f, cudaStream_t st) {
    const int cin_pad = (cout_f + 15) / 16 * 16, npad = (cin_f + 15) / 16 * 16;
    k_pack_weights_bwd<<<grid_for(tc_packed_weight_elems(cin_pad, cin_f)), 256, 0, st>>>(w, packed, cin_f, cout_f,
                                                                                        cin_pad, npad);
    return cudaGetLastError();
}

cudaError_t tc_wgrad_plan(TcWgradPlan &p, const __nv_bfloat16 *g, int n, int h, int w, int cin, int cin_pad, int cout,
                          int sm_count) {
    std::memset(&p, 0, sizeof(p));
    if (n <= 0 || h <= 0 || w <= 0 || cin <= 0 || cin > cin_pad || (cin_pad & 15) || cin_pad > 256 || cout <= 0 ||
        cout > 128)
        return cudaErrorInvalidValue;
    p.g = g, p.n = n, p.h = h, p.w = w, p.cin = cin, p.cin_pad = cin_pad, p.cout = cout;
    p.cout_pad = (cout + 15) / 16 * 16;
    p.tiles_x = (w + kTileW - 1) / kTileW;
    p.tiles_y = (h + kTileH - 1) / kTileH;
    const long long tiles = (long long)n * p.tiles_x * p.tiles_y;
    if (tiles > 0x7FFFFFFFLL) return cudaErrorInvalidValue;
    p.tiles = (int)tiles;
    // taps per pass: as many accumulators of cin_pad columns as 512 TMEM columns hold
    p.taps_per_pass = 512 / cin_pad < 9 ? 512 / cin_pad : 9;
    p.passes = (9 + p.taps_per_pass - 1) / p.taps_per_pass;
    int cols = 32;
    while (cols < p.taps_per_pass * cin_pad) cols <<= 1;
    p.tmem_cols = cols;
    // about one CTA per SM over all groups and passes (a CTA overlaps its
    // loads with its MMAs; fewer groups also mean fewer partial sums)
    const long long want = sm_count;
    long long per = (tiles * p.passes + want - 1) / want;
    if (per < 1) per = 1;
    p.tiles_per_cta = (int)per;
    p.groups = (int)((tiles + per - 1) / per);
    // a stage: 128 rows of A (16 planes), then the halo planes of B; two
    // stages (loads of the next tile beside the MMAs of this one) where they fit
    p.b_off = kGradPlanes * kGradPlaneBytes;
    p.stage_bytes = (p.b_off + (uint32_t)(cin_pad / 8) * kPlaneBytes + 1023) & ~1023u;
    p.stages = 2 * (size_t)p.stage_bytes + 64 <= kSmemMax ? 2 : 1;
    p.bar_off = (uint32_t)p.stages * p.stage_bytes;
    p.smem = p.bar_off + 5 * 8 + 16;
    if (p.smem > kSmemMax) return cudaErrorInvalidValue;
    // no more CTAs per SM than TMEM has columns for (tcgen05.alloc would wait):
    // ask for enough shared memory to keep the others off the SM
    const size_t max_ctas = 512 / cols;
    if (kSmemPerSm / (p.smem + 1024) > max_ctas) {
        p.smem = kSmemPerSm / max_ctas - 1024 + 16;
        if (p.smem > kSmemMax) p.smem = kSmemMax;
    }
    p.partial_floats = (size_t)p.groups * 9 * cout * cin_pad;
    EncodeTiled enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[4] = {(cuuint64_t)p.cout_pad, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)p.cout_pad * 2, (cuuint64_t)w * p.cout_pad * 2,
                                   (cuuint64_t)h * w * p.cout_pad * 2};
    const cuuint32_t box[4] = {8, kTileW, kTileH, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUtensorMap *map = reinterpret_cast<CUtensorMap *>(p.gmap);
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16 *>(g), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t conv3x3_wgrad_tc(const TcWgradPlan &p, const TcConvPlan &fwd, float *dw, float *partial, int *err,
                             cudaStream_t st) {
    if (!partial || !dw || fwd.cin != p.cin_pad || fwd.n != p.n || fwd.h != p.h || fwd.w != p.w)
        return cudaErrorInvalidValue;
    static std::atomic<uint64_t> attr_set{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (!bit || !(attr_set.load() & bit)) {
        e = cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    WgArgs a;
    a.partial = partial;
    a.n = p.n, a.h = p.h, a.wd = p.w, a.cin_pad = p.cin_pad, a.cout = p.cout, a.cout_pad = p.cout_pad;
    a.tiles_x = p.tiles_x, a.tiles_y = p.tiles_y, a.tiles = p.tiles, a.tiles_per_cta = p.tiles_per_cta;
    a.taps_per_pass = p.taps_per_pass, a.tmem_cols = p.tmem_cols, a.stages = p.stages;
    a.b_off = p.b_off, a.stage_bytes = p.stage_bytes, a.bar_off = p.bar_off;
    a.err = err;
    CUtensorMap gm, xm;
    std::memcpy(&gm, p.gmap, sizeof(gm));
    std::memcpy(&xm, fwd.tmap, sizeof(xm));
    k_wgrad_tc<<<dim3((unsigned)p.groups, (unsigned)p.passes), 128, p.smem, st>>>(gm, xm, a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const size_t elems = (size_t)p.cout * 9 * p.cin;
    k_wgrad_finalize<<<(unsigned)((elems + 31) / 32), 32 * kFinSlices, 0, st>>>(partial, dw, p.groups, p.cout, p.cin,
                                                                             p.cin_pad);
    return cudaGetLastError();
}

cudaError_t tc_conv_plan(TcConvPlan &p, const __nv_bfloat16 *x, int n, int h, int w, int cin, int cout, bool relu,
                         int sm_count) {
    std::memset(&p, 0, sizeof(p));
    if (n <= 0 || h <= 0 || w <= 0 || cin <= 0 || (cin & 15) || cin > 2040 || cout <= 0) return cudaErrorInvalidValue;
    p.x = x, p.n = n, p.h = h, p.w = w, p.cin = cin, p.cout = cout, p.relu = relu ? 1 : 0;
    p.npad = (cout + 15) / 16 * 16;
    if (p.npad > 256) return cudaErrorInvalidValue;
    p.tiles_x = (w + kTileW - 1) / kTileW;
    p.tiles_y = (h + kTileH - 1) / kTileH;
    const long long tiles = (long long)n * p.tiles_x * p.tiles_y;
    if (tiles > 0x7FFFFFFFLL) return cudaErrorInvalidValue;
    p.tiles = (int)tiles;
    // too few tiles to fill the GPU twice: split the output channels into
    // chunks of a multiple of 16 (each CTA all nine taps for its chunk, so no
    // partial sums), the widest chunk that still gives one CTA per SM (every
    // chunk's CTA loads the whole input halo, so narrower chunks cost loads);
    // with a single 16-channel chunk, split the taps instead (partial sums and
    // a finalize pass)
    p.splits = 1;
    p.nsplit = 1;
    p.npad_full = p.npad;
    if (tiles < 2LL * sm_count) {
        if (p.npad >= 32) {
            int cw = 16;
            for (int c = p.npad / 2 / 16 * 16; c >= 16; c -= 16)
                if (p.npad % c == 0 && tiles * (p.npad / c) >= (long long)sm_count) {
                    cw = c;
                    break;
                }
            p.nsplit = p.npad / cw;
            p.npad = cw;
        } else {
            p.splits = (tiles * 3 >= 2LL * sm_count) ? 3 : 9;
        }
    }
    p.taps_per_split = 9 / p.splits;
    const size_t halo = (size_t)(cin / 8) * kPlaneBytes;
    const size_t wtap = (size_t)cin * p.npad * 2;
    // a TMA box of the weight slice spans at most 256 (tap, chunk) rows
    const bool box_ok = p.nsplit == 1 || (size_t)p.taps_per_split * (cin / 8) <= 256;
    if (halo + p.taps_per_split * wtap <= kSmemBudget && box_ok) {
        p.taps_per_stage = p.taps_per_split;
        p.stages = 1;
    } else {
        p.taps_per_stage = 1;
        size_t fit = halo < kSmemBudget ? (kSmemBudget - halo) / wtap : 0;
        if (fit < 2) fit = 2;
        p.stages = (int)(fit < (size_t)p.taps_per_split ? fit : (size_t)p.taps_per_split);
    }
    if (p.nsplit > 1 && (size_t)p.taps_per_stage * (cin / 8) > 256) return cudaErrorInvalidValue;
    // persistent pipelined kernel: no split, two halos and all weights resident
    p.persistent = p.splits == 1 && p.nsplit == 1 && 2 * halo + 9 * wtap + 64 <= kSmemPersistent;
    size_t smem;
    int cols = 32;
    if (p.persistent) {
        while (cols < 2 * ((p.npad + 31) & ~31)) cols <<= 1;
        // a ring of three halos unless two keep more CTAs resident per SM
        auto ring_smem = [&](int ring) {
            const size_t bar = (ring * halo + 9 * wtap + 15) & ~(size_t)15;
            return bar + 8 * (2 * (size_t)ring + 6) + 32;
        };
        auto resident = [&](int ring) {
            const size_t by_smem = kSmemPerSm / (ring_smem(ring) + 1024), by_tmem = 512 / (size_t)cols;
            return by_smem < by_tmem ? by_smem : by_tmem;
        };
        const int ring = ring_smem(3) <= kSmemPersistent && resident(3) >= resident(2) ? 3 : 2;
        p.stages = ring;
        p.halo_stride = (uint32_t)halo;
        p.w_off = (uint32_t)(ring * halo);
        p.bar_off = (uint32_t)((ring * halo + 9 * wtap + 15) & ~(size_t)15);
        smem = ring_smem(ring);
    } else {
        p.halo_stride = 0;
        p.w_off = (uint32_t)halo;
        p.bar_off = (uint32_t)(halo + (size_t)p.stages * p.taps_per_stage * wtap);
        p.bar_off = (p.bar_off + 15) & ~15u;
        smem = p.bar_off + 8 * (2 + 2 * (size_t)p.stages) + 16;
        while (cols < p.npad) cols <<= 1;
    }
    p.tmem_cols = cols;
    // no more CTAs per SM than TMEM has columns for (tcgen05.alloc would wait)
    const size_t max_ctas = 512 / cols;
    if (smem > kSmemMax) return cudaErrorInvalidValue;
    if (kSmemPerSm / (smem + 1024) > max_ctas) {
        smem = kSmemPerSm / max_ctas - 1024 + 16;
        if (smem > kSmemMax) smem = kSmemMax;  // one CTA per SM
    }
    p.smem = smem;
    if (p.persistent) {
        size_t per_sm = kSmemPerSm / (smem + 1024);
        if (per_sm > max_ctas) per_sm = max_ctas;
        if (per_sm < 1) per_sm = 1;
        const long long slots = (long long)sm_count * (long long)per_sm;
        p.grid = (int)(tiles < slots ? tiles : slots);
    } else {
        p.grid = p.tiles;
    }
    p.partial_floats = p.splits > 1 ? (size_t)p.splits * n * h * w * p.npad : 0;

    EncodeTiled enc = encode_fn();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)w * cin * 2, (cuuint64_t)h * w * cin * 2};
    const cuuint32_t box[4] = {8, kHaloW, kHaloH, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUtensorMap *map = reinterpret_cast<CUtensorMap *>(p.tmap);
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16 *>(x), dims, strides,
                           box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t conv3x3_forward_tc(const TcConvPlan &p, const __nv_bfloat16 *wpacked, const float *bias,
                               __nv_bfloat16 *y, float *y32, float *partial, int *err, cudaStream_t st,
                               const TcFuse *fuse, bool overlap_prologue) {
    if (p.splits > 1 && !partial) return cudaErrorInvalidValue;
    if (fuse) {
        if (p.splits > 1) return cudaErrorInvalidValue;
        if ((fuse->pool || fuse->cat) && (p.cout & 15)) return cudaErrorInvalidValue;
        if (fuse->cat && (fuse->cat_c & 7 || fuse->cat_off & 7 || fuse->cat_off + p.cout > fuse->cat_c))
            return cudaErrorInvalidValue;
        if ((fuse->res || fuse->rad) && !y32) return cudaErrorInvalidValue;
        if (fuse->rad && (p.cout != 3 || !fuse->feat)) return cudaErrorInvalidValue;
    }
    // the shared-memory opt-in is a per-device setting of each kernel: once per device
    static std::atomic<uint64_t> attr_set{0};
    int dev = 0;
    cudaError_t e0 = cudaGetDevice(&dev);
    if (e0 != cudaSuccess) return e0;
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (!bit || !(attr_set.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_conv_tc_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    TcArgs a;
    a.w = wpacked, a.bias = bias;
    a.y = p.splits > 1 ? nullptr : y;
    a.y32 = p.splits > 1 ? nullptr : y32;
    a.partial = p.splits > 1 ? partial : nullptr;
    a.n = p.n, a.h = p.h, a.wd = p.w, a.cin = p.cin, a.cout = p.cout, a.npad = p.npad, a.relu = p.relu;
    a.tiles_x = p.tiles_x, a.tiles_y = p.tiles_y;
    a.taps_per_split = p.taps_per_split, a.taps_per_stage = p.taps_per_stage, a.stages = p.stages;
    a.nsplit = p.nsplit, a.npad_full = p.npad_full;
    a.tmem_cols = p.tmem_cols;
    a.w_off = p.w_off, a.bar_off = p.bar_off, a.halo_stride = p.halo_stride;
    a.err = err;
    if (fuse) a.f = *fuse;
    CUtensorMap map, wmap;
    std::memcpy(&map, p.tmap, sizeof(map));
    std::memset(&wmap, 0, sizeof(wmap));
    if (p.nsplit > 1) {
        // the packed weights [tap][chunk][npad_full rows][8] as a 3-D map:
        // (8 channels, rows, tap x chunk); each CTA loads rows n0..n0+npad
        EncodeTiled enc = encode_fn();
        if (!enc) return cudaErrorNotSupported;
        const cuuint64_t dims[3] = {8, (cuuint64_t)p.npad_full, (cuuint64_t)9 * (p.cin / 8)};
        const cuuint64_t strides[2] = {16, (cuuint64_t)p.npad_full * 16};
        const cuuint32_t box[3] = {8, (cuuint32_t)p.npad, (cuuint32_t)(p.taps_per_stage * (p.cin / 8))};
        const cuuint32_t estr[3] = {1, 1, 1};
        const CUresult r = enc(&wmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(wpacked), dims,
                               strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.dynamicSmemBytes = p.smem;
    cfg.stream = st;
    cfg.attrs = overlap_prologue ? attr : nullptr;
    cfg.numAttrs = overlap_prologue ? 1 : 0;
    cudaError_t e;
    if (p.persistent) {
        cfg.gridDim = dim3((unsigned)p.grid), cfg.blockDim = dim3(kWsThreads);
        e = cudaLaunchKernelEx(&cfg, k_conv_tc_persistent, map, a);
    } else {
        cfg.gridDim = dim3((unsigned)p.tiles, (unsigned)(p.nsplit > 1 ? p.nsplit : p.splits)), cfg.blockDim = dim3(128);
        e = cudaLaunchKernelEx(&cfg, k_conv_tc, map, wmap, a);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess || p.splits == 1) return e;
    const size_t M = (size_t)p.n * p.h * p.w;
    if ((p.cout & 3) == 0)
        k_conv_finalize<4><<<grid_for(M * p.cout / 4), 256, 0, st>>>(partial, bias, y, y32, M, p.npad, p.cout,
                                                                      p.splits, p.relu);
    else
        k_conv_finalize<1><<<grid_for(M * p.cout), 256, 0, st>>>(partial, bias, y, y32, M, p.npad, p.cout, p.splits,
                                                                  p.relu);
    return cudaGetLastError();
}

}  // namespace dn
}  // namespace pray_gpu
