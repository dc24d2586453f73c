// 3x3 convolution forward on the 5th-generation tensor cores (tcgen05).
//
// Implicit GEMM: D[pixel][cout] = sum_k A[pixel][k] B[cout][k], k = tap * Cin
// + ci, A gathered from the NHWC activations with zero padding (im2col, never
// materialised), B the [Cout][3][3][Cin] weights; BF16 operands, FP32
// accumulation in tensor memory (TMEM).
//
// One CTA (4 warps) computes a 128-pixel x Npad tile (Npad = Cout rounded up
// to 16, one TMEM column per output channel). Each stage gathers a 64-deep K
// slice of A and B into shared memory in the no-swizzle K-major canonical
// layout (8-row x 16-byte core matrices; neighbours along K 128 B apart,
// along rows 256 B apart), fences it for the async proxy, and one thread
// issues four kind::f16 MMAs (M 128, N Npad, K 16 each) and commits them to
// an mbarrier. Two shared-memory stages alternate, so the gather of stage s+1
// overlaps the MMAs of stage s. The epilogue reads the accumulator back with
// tcgen05.ld (each warp its 32 TMEM lanes), adds the bias, applies ReLU and
// stores BF16 (or FP32). Every mbarrier wait is bounded: on timeout the
// kernel records an error, stops issuing, drains what it issued (again
// bounded) and frees its TMEM.
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "denoise_ops.h"

namespace pray_gpu {
namespace dn {

namespace {

constexpr int kTM = 128;         // pixels per tile (MMA M)
constexpr int kKStage = 64;      // K per stage (4 MMAs of K 16)
constexpr int kSubBytesA = kTM * 16 * 2;  // one 128 x 16 BF16 sub-tile
constexpr uint32_t kWaitLimit = 1u << 24;

struct TcArgs {
    const __nv_bfloat16 *x;
    const __nv_bfloat16 *w;
    const float *bias;
    __nv_bfloat16 *y;
    float *y32;
    int n, h, wd, cin, cout, relu;
    int K, Kpad, Npad, tmem_cols;
    int *err;  // set to 1 if an mbarrier wait timed out
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading (K) and stride (row-group)
// byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M.
__host__ __device__ constexpr uint32_t inst_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(addr), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Byte offset of element (row, k) of a stage tile in the core-matrix layout:
// sub-tile k / 16 (rows x 16), core matrix (row / 8, (k % 16) / 8), row % 8
// at 16 B, k % 8 at 2 B.
__device__ __forceinline__ uint32_t tile_off(int row, int k, int sub_bytes) {
    return (uint32_t)((k >> 4) * sub_bytes + (row >> 3) * 256 + ((k >> 3) & 1) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ float bfv(__nv_bfloat16 v) { return __bfloat162float(v); }

// Gathers 8 consecutive k (one 16-byte core-matrix row) of A for `pix`.
__device__ __forceinline__ uint4 gather_a8(const TcArgs &P, int pix, int k0) {
    alignas(16) __nv_bfloat16 v[8];
    const int M = P.n * P.h * P.wd;
    if (pix < M && (P.cin & 7) == 0 && k0 < P.K) {
        const int tap = k0 / P.cin, ci = k0 - tap * P.cin;
        const int xw = pix % P.wd, yh = (pix / P.wd) % P.h, img = pix / (P.wd * P.h);
        const int sx = xw + tap % 3 - 1, sy = yh + tap / 3 - 1;
        if (sx < 0 || sy < 0 || sx >= P.wd || sy >= P.h) return make_uint4(0, 0, 0, 0);
        return *reinterpret_cast<const uint4 *>(P.x + (((size_t)img * P.h + sy) * P.wd + sx) * P.cin + ci);
    }
    for (int e = 0; e < 8; e++) {
        const int k = k0 + e;
        float val = 0.f;
        if (pix < M && k < P.K) {
            const int tap = k / P.cin, ci = k - tap * P.cin;
            const int xw = pix % P.wd, yh = (pix / P.wd) % P.h, img = pix / (P.wd * P.h);
            const int sx = xw + tap % 3 - 1, sy = yh + tap / 3 - 1;
            if (sx >= 0 && sy >= 0 && sx < P.wd && sy < P.h)
                val = bfv(P.x[(((size_t)img * P.h + sy) * P.wd + sx) * P.cin + ci]);
        }
        v[e] = __float2bfloat16(val);
    }
    return *reinterpret_cast<const uint4 *>(v);
}

// 8 consecutive k of B (weights) for output channel co.
__device__ __forceinline__ uint4 gather_b8(const TcArgs &P, int co, int k0) {
    alignas(16) __nv_bfloat16 v[8];
    if (co < P.cout && (P.K & 7) == 0 && k0 < P.K)
        return *reinterpret_cast<const uint4 *>(P.w + (size_t)co * P.K + k0);
    for (int e = 0; e < 8; e++) {
        const int k = k0 + e;
        v[e] = (co < P.cout && k < P.K) ? P.w[(size_t)co * P.K + k] : __float2bfloat16(0.f);
    }
    return *reinterpret_cast<const uint4 *>(v);
}

__global__ void __launch_bounds__(128) k_conv_tc(TcArgs P) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int sub_b = P.Npad * 32;                       // one Npad x 16 BF16 sub-tile of B
    const int stage_bytes = 4 * kSubBytesA + 4 * sub_b;  // A then B
    uint8_t *stage0 = smem;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + 2 * stage_bytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * kTM;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = inst_desc(kTM, P.Npad);
    const int stages = P.Kpad / kKStage + ((P.Kpad % kKStage) ? 1 : 0);
    uint32_t phase[2] = {0, 0};
    bool issued[2] = {false, false};
    bool ok = true;

    for (int s = 0; s < stages && ok; s++) {
        const int buf = s & 1;
        uint8_t *A = stage0 + buf * stage_bytes;
        uint8_t *B = A + 4 * kSubBytesA;
        // the MMAs that last read this buffer must be done
        if (issued[buf]) {
            ok = mbar_wait(smem_u32(&mbar[buf]), phase[buf]);
            phase[buf] ^= 1;
            issued[buf] = false;
            if (!ok) break;
        }
        const int k0 = s * kKStage;
        // A: 128 rows x 8 chunks of 8 k; B: Npad rows x 8 chunks
        for (int i = tid; i < kTM * 8; i += 128) {
            const int row = i >> 3, c = i & 7;
            *reinterpret_cast<uint4 *>(A + tile_off(row, c * 8, kSubBytesA)) = gather_a8(P, m0 + row, k0 + c * 8);
        }
        for (int i = tid; i < P.Npad * 8; i += 128) {
            const int row = i >> 3, c = i & 7;
            *reinterpret_cast<uint4 *>(B + tile_off(row, c * 8, sub_b)) = gather_b8(P, row, k0 + c * 8);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int sub = 0; sub < 4; sub++) {
                const int kk = k0 + sub * 16;
                if (kk >= P.Kpad) break;
                const uint64_t ad = smem_desc(smem_u32(A + sub * kSubBytesA), 128, 256);
                const uint64_t bd = smem_desc(smem_u32(B + sub * sub_b), 128, 256);
                const uint32_t acc = kk > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[buf]))
                         : "memory");
        }
        issued[buf] = true;
    }
    // drain: wait for every committed group (bounded)
    for (int b = 0; b < 2; b++)
        if (issued[b]) {
            if (!mbar_wait(smem_u32(&mbar[b]), phase[b])) ok = false;
            phase[b] ^= 1;
        }
    if (!ok && tid == 0) atomicExch(P.err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (ok) {
        // epilogue: warp w holds TMEM lanes 32w..32w+31 = tile rows
        const int row = warp * 32 + (tid & 31);
        const int pix = m0 + row;
        const int M = P.n * P.h * P.wd;
        for (int c0 = 0; c0 < P.Npad; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (pix < M) {
                for (int j = 0; j < 16; j++) {
                    const int co = c0 + j;
                    if (co >= P.cout) break;
                    float v = __uint_as_float(r[j]) + P.bias[co];
                    if (P.relu) v = fmaxf(v, 0.f);
                    if (P.y) P.y[(size_t)pix * P.cout + co] = __float2bfloat16(v);
                    if (P.y32) P.y32[(size_t)pix * P.cout + co] = v;
                }
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

}  // namespace

cudaError_t conv3x3_forward_tc(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *b, __nv_bfloat16 *y,
                               float *y32, int n, int h, int wd, int cin, int cout, bool relu, int *err,
                               cudaStream_t st) {
    TcArgs P;
    P.x = x, P.w = w, P.bias = b, P.y = y, P.y32 = y32;
    P.n = n, P.h = h, P.wd = wd, P.cin = cin, P.cout = cout, P.relu = relu ? 1 : 0;
    P.K = 9 * cin;
    P.Kpad = (P.K + 15) / 16 * 16;
    P.Npad = (cout + 15) / 16 * 16;
    if (P.Npad > 256) return cudaErrorInvalidValue;
    int cols = 32;
    while (cols < P.Npad) cols <<= 1;
    P.tmem_cols = cols;
    P.err = err;
    const int M = n * h * wd;
    if (M <= 0) return cudaSuccess;
    const size_t smem = 2 * (size_t)(4 * kSubBytesA + 4 * P.Npad * 32) + 64;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    k_conv_tc<<<(M + kTM - 1) / kTM, 128, smem, st>>>(P);
    return cudaGetLastError();
}

}  // namespace dn
}  // namespace pray_gpu
