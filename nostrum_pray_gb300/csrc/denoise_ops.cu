// Denoiser layers (sm_103a): 3x3 convolutions as implicit GEMMs, 2x2 average
// pooling, nearest 2x upsampling, channel concatenation, ReLU masks, L1 loss
// and Adam. Activations are BF16 NHWC tensors, weights [Cout][3][3][Cin]
// with FP32 master copies, gradients FP32; every product accumulates in
// FP32.
//
// Convolution GEMMs (p = pixel, t = tap of the 3x3 stencil):
//   forward      Y[p][co]      = b[co] + sum_{t,ci} X[p+t][ci] W[co][t][ci]    (M=pixels, N=Cout, K=9Cin)
//   grad input   dX[p][ci]     = sum_{t,co} G[p-t][co] W[co][t][ci]            (M=pixels, N=Cin,  K=9Cout)
//   grad weights dW[co][t][ci] = sum_p G[p][co] X[p+t][ci]                     (M=Cout, N=9Cin, K=pixels)
// with zero padding outside the image and G the output gradient after the
// ReLU mask. One tiled kernel (64x64 tile, 16-deep K steps staged in shared
// memory, 4x4 outputs per thread) serves all three through gather functors;
// the weight gradient splits K over blocks and adds with FP32 atomics.
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "denoise_ops.h"

namespace pray_gpu {
namespace dn {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, kThreads = 256;

struct Geom {
    int n, h, w;  // images, height, width
};

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// X[p + tap][ci] with zero padding; k = tap * Cin + ci.
struct GatherIm2col {
    const __nv_bfloat16 *x;
    Geom g;
    int cin;
    __device__ __forceinline__ float operator()(int p, int k) const {
        const int tap = k / cin, ci = k - tap * cin;
        const int xw = p % g.w, yh = (p / g.w) % g.h, img = p / (g.w * g.h);
        const int sx = xw + tap % 3 - 1, sy = yh + tap / 3 - 1;
        if (sx < 0 || sy < 0 || sx >= g.w || sy >= g.h) return 0.f;
        return bf(x[(((size_t)img * g.h + sy) * g.w + sx) * cin + ci]);
    }
};

// W[co][tap][ci] as B[k = tap*Cin + ci][co].
struct GatherWeightsFwd {
    const __nv_bfloat16 *wt;
    int cin;
    __device__ __forceinline__ float operator()(int k, int co) const { return bf(wt[(size_t)co * 9 * cin + k]); }
};

// G[p - tap][co] with zero padding; k = tap * Cout + co.
struct GatherGradShift {
    const float *g;
    Geom geo;
    int cout;
    __device__ __forceinline__ float operator()(int p, int k) const {
        const int tap = k / cout, co = k - tap * cout;
        const int xw = p % geo.w, yh = (p / geo.w) % geo.h, img = p / (geo.w * geo.h);
        const int sx = xw - (tap % 3 - 1), sy = yh - (tap / 3 - 1);
        if (sx < 0 || sy < 0 || sx >= geo.w || sy >= geo.h) return 0.f;
        return g[(((size_t)img * geo.h + sy) * geo.w + sx) * cout + co];
    }
};

// W[co][tap][ci] as B[k = tap*Cout + co][ci].
struct GatherWeightsBwd {
    const __nv_bfloat16 *wt;
    int cin, cout;
    __device__ __forceinline__ float operator()(int k, int ci) const {
        const int tap = k / cout, co = k - tap * cout;
        return bf(wt[((size_t)co * 9 + tap) * cin + ci]);
    }
};

// A[co][p] = G[p][co] for the weight gradient.
struct GatherGradT {
    const float *g;
    int cout;
    __device__ __forceinline__ float operator()(int co, int p) const { return g[(size_t)p * cout + co]; }
};

// B[p][k = tap*Cin + ci] = X[p + tap][ci].
struct GatherIm2colT {
    GatherIm2col inner;
    __device__ __forceinline__ float operator()(int p, int k) const { return inner(p, k); }
};

struct StoreFwd {
    __nv_bfloat16 *y;
    float *y32;
    const float *bias;
    int cout;
    bool relu;
    __device__ __forceinline__ void operator()(int p, int co, float acc) const {
        float v = acc + bias[co];
        if (relu) v = fmaxf(v, 0.f);
        if (y) y[(size_t)p * cout + co] = __float2bfloat16(v);
        if (y32) y32[(size_t)p * cout + co] = v;
    }
};

struct StoreGradIn {
    float *dx;
    int cin;
    __device__ __forceinline__ void operator()(int p, int ci, float acc) const { dx[(size_t)p * cin + ci] = acc; }
};

struct StoreGradW {
    float *dw;
    int n9cin;
    __device__ __forceinline__ void operator()(int co, int k, float acc) const {
        atomicAdd(dw + (size_t)co * n9cin + k, acc);
    }
};

// C[M x N] = A[M x K] B[K x N]; blockIdx.z splits K into chunks of k_chunk.
template <class AL, class BL, class EP>
__global__ void __launch_bounds__(kThreads) k_gemm(int M, int N, int K, int k_chunk, AL A, BL B, EP E) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int k_begin = blockIdx.z * k_chunk, k_end = min(K, k_begin + k_chunk);
    float acc[4][4] = {};
    for (int k0 = k_begin; k0 < k_end; k0 += BK) {
        for (int i = threadIdx.x; i < BK * BM; i += kThreads) {
            const int kk = i / BM, mm = i % BM;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < k_end) ? A(m, k) : 0.f;
        }
        for (int i = threadIdx.x; i < BK * BN; i += kThreads) {
            const int kk = i / BN, nn = i % BN;
            const int nidx = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (nidx < N && k < k_end) ? B(k, nidx) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; r++) a[r] = As[kk][ty * 4 + r], b[r] = Bs[kk][tx * 4 + r];
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int m = m0 + ty * 4 + r, nidx = n0 + tx * 4 + c;
            if (m < M && nidx < N) E(m, nidx, acc[r][c]);
        }
}

template <class AL, class BL, class EP>
cudaError_t gemm(int M, int N, int K, int splits, AL A, BL B, EP E, cudaStream_t st) {
    if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
    splits = max(1, splits);
    int chunk = (K + splits - 1) / splits;
    chunk = (chunk + BK - 1) / BK * BK;
    splits = (K + chunk - 1) / chunk;
    dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, splits);
    k_gemm<<<grid, kThreads, 0, st>>>(M, N, K, chunk, A, B, E);
    return cudaGetLastError();
}

__device__ __forceinline__ size_t gtid() { return (size_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ size_t gstride() { return (size_t)gridDim.x * blockDim.x; }

__global__ void k_relu_mask(const __nv_bfloat16 *y, const float *g, float *out, size_t n) {
    for (size_t i = gtid(); i < n; i += gstride()) out[i] = bf(y[i]) > 0.f ? g[i] : 0.f;
}

__global__ void k_grad_bf16(const float *g, __nv_bfloat16 *out, size_t pixels, int c, int c_pad) {
    const size_t n = pixels * (size_t)c_pad;
    for (size_t i = gtid(); i < n; i += gstride()) {
        const size_t p = i / (size_t)c_pad;
        const int k = (int)(i - p * c_pad);
        out[i] = __float2bfloat16(k < c ? g[p * c + k] : 0.f);
    }
}

// Threads (r, k), r < rows, k < c_pad: channel k of pixels p0 + r, p0 + r +
// rows, ... of the block's range; reads and writes are row-contiguous.
__global__ void k_grad_prep(const __nv_bfloat16 *y, const float *g, __nv_bfloat16 *out, float *part, size_t pixels,
                            size_t chunk, int c, int c_pad, int rows) {
    __shared__ float sm[256];
    const int k = (int)threadIdx.x % c_pad, r = (int)threadIdx.x / c_pad;
    const size_t p0 = (size_t)blockIdx.x * chunk, p1 = p0 + chunk < pixels ? p0 + chunk : pixels;
    float acc = 0.f;
    for (size_t p = p0 + r; p < p1; p += rows) {
        float v = 0.f;
        if (k < c) {
            v = g[p * c + k];
            if (y && !(bf(y[p * c + k]) > 0.f)) v = 0.f;
        }
        out[p * c_pad + k] = __float2bfloat16(v);
        acc += v;
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    if (r == 0 && k < c) {
        float s = 0.f;
        for (int i = 0; i < rows; i++) s += sm[i * c_pad + k];
        part[(size_t)blockIdx.x * c + k] = s;
    }
}

// One block (256 threads) per channel: thread t adds the partials of blocks
// t, t + 256, ..., then a fixed tree adds the 256 sums (the same order on
// every run).
__global__ void k_bias_finalize(const float *part, float *db, int blocks, int c) {
    // a backward-data convolution launched next may start its prologue now
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ float sm[256];
    const int k = (int)blockIdx.x, t = (int)threadIdx.x;
    float s = 0.f;
    for (int b = t; b < blocks; b += 256) s += part[(size_t)b * c + k];
    sm[t] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) sm[t] += sm[t + o];
        __syncthreads();
    }
    if (t == 0) db[k] += sm[0];
}

__global__ void k_bias_grad(const float *g, float *db, size_t pixels, int c) {
    // one block per channel
    __shared__ float sm[256];
    const int co = blockIdx.x;
    float acc = 0.f;
    for (size_t p = threadIdx.x; p < pixels; p += blockDim.x) acc += g[p * c + co];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[co] += sm[0];
}

__global__ void k_avgpool(const __nv_bfloat16 *x, __nv_bfloat16 *y, int n, int h, int w, int c) {
    const int ho = h / 2, wo = w / 2;
    const size_t total = (size_t)n * ho * wo * c;
    for (size_t i = gtid(); i < total; i += gstride()) {
        const int ch = (int)(i % c);
        size_t r = i / c;
        const int xo = (int)(r % wo);
        r /= wo;
        const int yo = (int)(r % ho);
        const int img = (int)(r / ho);
        const size_t b = (((size_t)img * h + 2 * yo) * w + 2 * xo) * c + ch;
        const float s = bf(x[b]) + bf(x[b + c]) + bf(x[b + (size_t)w * c]) + bf(x[b + (size_t)w * c + c]);
        y[i] = __float2bfloat16(0.25f * s);
    }
}

__global__ void k_avgpool_bwd(const float *gy, float *gx, int n, int h, int w, int c) {
    const size_t total = (size_t)n * h * w * c;
    const int wo = w / 2, ho = h / 2;
    for (size_t i = gtid(); i < total; i += gstride()) {
        const int ch = (int)(i % c);
        size_t r = i / c;
        const int xx = (int)(r % w);
        r /= w;
        const int yy = (int)(r % h);
        const int img = (int)(r / h);
        gx[i] += 0.25f * gy[(((size_t)img * ho + yy / 2) * wo + xx / 2) * c + ch];
    }
}

// nearest 2x upsampling of x (c channels) into channels [0, c) of y (cy channels)
// gradient of the nearest 2x upsampling: gx[h,w] = sum of the 4 children (channels [0,c) of gy)
__global__ void k_upsample_bwd(const float *gy, float *gx, int n, int h, int w, int c, int cy) {
    const int W = 2 * w;
    const size_t total = (size_t)n * h * w * c;
    for (size_t i = gtid(); i < total; i += gstride()) {
        const int ch = (int)(i % c);
        size_t r = i / c;
        const int xx = (int)(r % w);
        r /= w;
        const int yy = (int)(r % h);
        const int img = (int)(r / h);
        const size_t b = (((size_t)img * 2 * h + 2 * yy) * W + 2 * xx) * cy + ch;
        gx[i] = gy[b] + gy[b + cy] + gy[b + (size_t)W * cy] + gy[b + (size_t)W * cy + cy];
    }
}

// gx (c channels) += channels [off, off+c) of gy (cy channels)
__global__ void k_split_add(const float *gy, float *gx, size_t pixels, int c, int cy, int off) {
    const size_t total = pixels * c;
    for (size_t i = gtid(); i < total; i += gstride()) gx[i] += gy[(i / c) * cy + off + i % c];
}

// Demodulation divisor of value i (pixel i / 3): first-hit albedo of its
// channel, clamped at 0, plus 0.05.
__device__ __forceinline__ float demod(const __half *feat, size_t i) {
    return fmaxf(__half2float(feat[7 * (i / 3) + i % 3]), 0.f) + kDemodFloor;
}

// network input: log1p(radiance / demodulation) 3, albedo 3, normal 3, depth
// 1 from FP16 feature buffers (radiance n x 3 floats, features n x 7 halves);
// x16 (optional) receives the same 10 channels padded to 16 with zeros
__global__ void k_pack_input(const float *rad, const __half *feat, __nv_bfloat16 *x, __nv_bfloat16 *x16,
                             size_t pixels) {
    // the first convolution may launch now (its prologue overlaps this
    // kernel; it waits for this kernel's completion before reading x16)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    for (size_t p = gtid(); p < pixels; p += gstride()) {
        __nv_bfloat16 v[16];
        for (int k = 0; k < 3; k++) v[k] = __float2bfloat16(log1pf(fmaxf(rad[3 * p + k], 0.f) / demod(feat, 3 * p + k)));
        for (int k = 0; k < 7; k++) v[3 + k] = __float2bfloat16(__half2float(feat[7 * p + k]));
        for (int k = 10; k < 16; k++) v[k] = __float2bfloat16(0.f);
        if (x)
            for (int k = 0; k < 10; k++) x[p * 10 + k] = v[k];
        if (x16) {
            uint4 *o = reinterpret_cast<uint4 *>(x16 + p * 16);
            o[0] = *reinterpret_cast<const uint4 *>(v);
            o[1] = *reinterpret_cast<const uint4 *>(v + 8);
        }
    }
}

// L1 loss on log1p(radiance / demodulation): out = network output (log
// space), target in linear radiance; gradient into g (scaled by 1/n), each
// block's sum of |d| into part[block] by a fixed tree; k_l1_finalize adds the
// blocks' sums in a fixed order, so the loss is the same bits on every run
__global__ void k_l1(const float *out, const float *target, const __half *feat, float *g, float *part, size_t n) {
    __shared__ float sm[256];
    float acc = 0.f;
    const float inv = 1.f / (float)n;
    for (size_t i = gtid(); i < n; i += gstride()) {
        const float d = out[i] - log1pf(fmaxf(target[i], 0.f) / demod(feat, i));
        acc += fabsf(d);
        g[i] = (d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f)) * inv;
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_l1_finalize(const float *part, int blocks, float *loss, float inv) {
    __shared__ float sm[256];
    float s = 0.f;
    for (int b = (int)threadIdx.x; b < blocks; b += 256) s += part[b];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[0] = sm[0] * inv;
}

// residual output: out (log space) += the input's log(1 + radiance) channels
__global__ void k_add_input(float *out, const __nv_bfloat16 *x0, int x0_c, size_t pixels) {
    for (size_t i = gtid(); i < pixels * 3; i += gstride()) out[i] += bf(x0[(i / 3) * x0_c + i % 3]);
}

__global__ void k_expm1(const float *out, const __half *feat, float *rad, size_t n) {
    for (size_t i = gtid(); i < n; i += gstride()) rad[i] = expm1f(out[i]) * demod(feat, i);
}

// cat (c + cs channels, 2h x 2w) = [nearest 2x upsampling of low (c
// channels, h x w), skip (cs channels, 2h x 2w)], 8 channels (16 bytes) per
// thread; c and cs multiples of 8
__global__ void k_upsample_concat(const __nv_bfloat16 *low, const __nv_bfloat16 *skip, __nv_bfloat16 *cat, int n,
                                  int h, int w, int c, int cs) {
    const int H = 2 * h, W = 2 * w, cy = c + cs, chunks = cy / 8;
    const size_t total = (size_t)n * H * W * chunks;
    for (size_t i = gtid(); i < total; i += gstride()) {
        const int k = (int)(i % chunks);
        const size_t pix = i / chunks;
        const int xx = (int)(pix % W);
        const size_t r = pix / W;
        const int yy = (int)(r % H);
        const int img = (int)(r / H);
        uint4 v;
        if (8 * k < c)
            v = *reinterpret_cast<const uint4 *>(low + (((size_t)img * h + yy / 2) * w + xx / 2) * c + 8 * k);
        else
            v = *reinterpret_cast<const uint4 *>(skip + pix * cs + (8 * k - c));
        *reinterpret_cast<uint4 *>(cat + pix * cy + 8 * k) = v;
    }
}

__global__ void k_adam(float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (size_t i = gtid(); i < n; i += gstride()) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16(wi);
    }
}

__global__ void k_to_bf16(const float *a, __nv_bfloat16 *b, size_t n) {
    for (size_t i = gtid(); i < n; i += gstride()) b[i] = __float2bfloat16(a[i]);
}

constexpr size_t kMaxBlocks = 152 * 32;  // grid-stride kernels: at most this many blocks of 256
static_assert(kL1Parts >= (int)kMaxBlocks, "l1_loss scratch holds one sum per block");
unsigned blocks_for(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, kMaxBlocks); }

}  // namespace

cudaError_t conv3x3_forward(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *b, __nv_bfloat16 *y,
                            float *y32, int n, int h, int wd, int cin, int cout, bool relu, cudaStream_t st) {
    const Geom g{n, h, wd};
    const int M = n * h * wd;
    return gemm(M, cout, 9 * cin, 1, GatherIm2col{x, g, cin}, GatherWeightsFwd{w, cin},
                StoreFwd{y, y32, b, cout, relu}, st);
}

cudaError_t conv3x3_backward(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *gpre, float *dx, float *dw,
                             float *db, int n, int h, int wd, int cin, int cout, cudaStream_t st) {
    const Geom g{n, h, wd};
    const int P = n * h * wd;
    cudaError_t e;
    if (dx) {
        e = gemm(P, cin, 9 * cout, 1, GatherGradShift{gpre, g, cout}, GatherWeightsBwd{w, cin, cout},
                 StoreGradIn{dx, cin}, st);
        if (e != cudaSuccess) return e;
    }
    const int splits = std::max(1, std::min(256, P / 1024));
    e = gemm(cout, 9 * cin, P, splits, GatherGradT{gpre, cout}, GatherIm2colT{GatherIm2col{x, g, cin}},
             StoreGradW{dw, 9 * cin}, st);
    if (e != cudaSuccess) return e;
    k_bias_grad<<<cout, 256, 0, st>>>(gpre, db, (size_t)P, cout);
    return cudaGetLastError();
}

cudaError_t relu_mask(const __nv_bfloat16 *y, const float *g, float *out, size_t n, cudaStream_t st) {
    k_relu_mask<<<blocks_for(n), 256, 0, st>>>(y, g, out, n);
    return cudaGetLastError();
}
cudaError_t bias_grad(const float *g, float *db, size_t pixels, int c, cudaStream_t st) {
    k_bias_grad<<<c, 256, 0, st>>>(g, db, pixels, c);
    return cudaGetLastError();
}
cudaError_t grad_prep(const __nv_bfloat16 *y, const float *g, __nv_bfloat16 *out, float *part, float *db,
                      size_t pixels, int c, int c_pad, cudaStream_t st) {
    if (c_pad < c || c_pad > 256 || (c_pad & 15) || pixels == 0) return cudaErrorInvalidValue;
    const int rows = 256 / c_pad;
    const size_t chunk = (pixels + kGradPrepBlocks - 1) / kGradPrepBlocks;
    const int blocks = (int)((pixels + chunk - 1) / chunk);
    k_grad_prep<<<blocks, rows * c_pad, 0, st>>>(y, g, out, part, pixels, chunk, c, c_pad, rows);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_bias_finalize<<<c, 256, 0, st>>>(part, db, blocks, c);
    return cudaGetLastError();
}
cudaError_t grad_bf16(const float *g, __nv_bfloat16 *out, size_t pixels, int c, int c_pad, cudaStream_t st) {
    if (c_pad < c) return cudaErrorInvalidValue;
    k_grad_bf16<<<blocks_for(pixels * (size_t)c_pad), 256, 0, st>>>(g, out, pixels, c, c_pad);
    return cudaGetLastError();
}
cudaError_t avgpool(const __nv_bfloat16 *x, __nv_bfloat16 *y, int n, int h, int w, int c, cudaStream_t st) {
    k_avgpool<<<blocks_for((size_t)n * h * w * c / 4), 256, 0, st>>>(x, y, n, h, w, c);
    return cudaGetLastError();
}
cudaError_t avgpool_backward(const float *gy, float *gx, int n, int h, int w, int c, cudaStream_t st) {
    k_avgpool_bwd<<<blocks_for((size_t)n * h * w * c), 256, 0, st>>>(gy, gx, n, h, w, c);
    return cudaGetLastError();
}
cudaError_t upsample_backward(const float *gy, float *gx, int n, int h, int w, int c, int cy, cudaStream_t st) {
    k_upsample_bwd<<<blocks_for((size_t)n * h * w * c), 256, 0, st>>>(gy, gx, n, h, w, c, cy);
    return cudaGetLastError();
}
cudaError_t split_add(const float *gy, float *gx, size_t pixels, int c, int cy, int off, cudaStream_t st) {
    k_split_add<<<blocks_for(pixels * c), 256, 0, st>>>(gy, gx, pixels, c, cy, off);
    return cudaGetLastError();
}
cudaError_t upsample_concat(const __nv_bfloat16 *low, const __nv_bfloat16 *skip, __nv_bfloat16 *cat, int n, int h,
                            int w, int c, int cs, cudaStream_t st) {
    if ((c & 7) || (cs & 7)) return cudaErrorInvalidValue;
    k_upsample_concat<<<blocks_for((size_t)n * 4 * h * w * ((c + cs) / 8)), 256, 0, st>>>(low, skip, cat, n, h, w, c,
                                                                                         cs);
    return cudaGetLastError();
}
cudaError_t pack_input(const float *rad, const __half *feat, __nv_bfloat16 *x, __nv_bfloat16 *x16, size_t pixels,
                       cudaStream_t st) {
    k_pack_input<<<blocks_for(pixels), 256, 0, st>>>(rad, feat, x, x16, pixels);
    return cudaGetLastError();
}
cudaError_t l1_loss(const float *out, const float *target, const __half *feat, float *g, float *loss, float *part,
                    size_t n, cudaStream_t st) {
    const unsigned blocks = blocks_for(n);
    k_l1<<<blocks, 256, 0, st>>>(out, target, feat, g, part, n);
    k_l1_finalize<<<1, 256, 0, st>>>(part, (int)blocks, loss, 1.f / (float)n);
    return cudaGetLastError();
}
cudaError_t add_input(float *out, const __nv_bfloat16 *x0, int x0_c, size_t pixels, cudaStream_t st) {
    k_add_input<<<blocks_for(pixels * 3), 256, 0, st>>>(out, x0, x0_c, pixels);
    return cudaGetLastError();
}
cudaError_t expm1_out(const float *out, const __half *feat, float *rad, size_t n, cudaStream_t st) {
    k_expm1<<<blocks_for(n), 256, 0, st>>>(out, feat, rad, n);
    return cudaGetLastError();
}
cudaError_t adam(float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, size_t n, float lr, float b1,
                 float b2, float eps, int step, cudaStream_t st) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<blocks_for(n), 256, 0, st>>>(w, g, m, v, wb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}
cudaError_t to_bf16(const float *a, __nv_bfloat16 *b, size_t n, cudaStream_t st) {
    k_to_bf16<<<blocks_for(n), 256, 0, st>>>(a, b, n);
    return cudaGetLastError();
}

}  // namespace dn
}  // namespace pray_gpu
