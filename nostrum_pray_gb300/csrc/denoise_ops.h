// Denoiser layer launchers (denoise_ops.cu). NHWC tensors; n images of
// h x w pixels. Gradient outputs: conv3x3_backward writes dx and adds into
// dw / db; avgpool_backward and split_add add into gx; upsample_backward
// writes gx.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace pray_gpu {
namespace dn {

// tcgen05 tensor-core version (denoise_tc.cu). A plan holds the input's TMA
// tensor map (the input buffer is fixed) and the launch shape; Cin must be a
// multiple of 16 (pack_input pads the network input), the weights packed by tc_pack_weights
// (cin_pad = Cin of the plan). Levels with few tiles split the taps over CTAs
// and need `partial` (partial_floats floats). *err is set to 1 if one of the
// kernel's bounded mbarrier waits ran out.
struct TcConvPlan {
    alignas(64) unsigned char tmap[128];  // CUtensorMap of x: (C, W, H, N), box (8, 10, 18, 1)
    const __nv_bfloat16 *x;
    int n, h, w, cin, cout, npad, relu;
    int tiles_x, tiles_y, tiles, splits, taps_per_split, taps_per_stage, stages, tmem_cols;
    int nsplit, npad_full;  // output-channel split: nsplit CTAs per tile, npad channels each of npad_full
    int persistent, grid;  // persistent pipelined kernel (no split, weights resident) and its CTAs
    uint32_t w_off, bar_off, halo_stride;
    size_t smem, partial_floats;
};
cudaError_t tc_conv_plan(TcConvPlan &p, const __nv_bfloat16 *x, int n, int h, int w, int cin, int cout, bool relu,
                         int sm_count);
size_t tc_packed_weight_elems(int cin_pad, int cout);
cudaError_t tc_pack_weights(const float *w, __nv_bfloat16 *packed, int cin, int cin_pad, int cout, cudaStream_t st);
// Weights of the backward-data convolution of a forward convolution with
// cin_f inputs and cout_f outputs (w[cout_f][9][cin_f]): a plan with
// cin = cout_f rounded up to 16 and cout = cin_f runs it on the output
// gradient (as BF16, grad_bf16) and writes the input gradient.
cudaError_t tc_pack_weights_bwd(const float *w, __nv_bfloat16 *packed, int cin_f, int cout_f, cudaStream_t st);
// Every packing of a network's weights in one launch: job j packs w (the
// FP32 [cout_f][9][cin_f] weights of one convolution) into out, as
// tc_pack_weights (bwd 0: cin_pad = cin_f rounded up to 16, npad = cout_f
// rounded up) or tc_pack_weights_bwd (bwd 1: cin_pad = cout_f rounded up,
// npad = cin_f rounded up) does; its 9 x cin_pad x npad elements start at
// `begin` of the concatenated range, jobs in increasing begin (at most 64).
struct TcPackJob {
    const float *w;
    __nv_bfloat16 *out;
    unsigned long long begin;
    int cin_f, cout_f, cin_pad, npad, bwd;
};
cudaError_t tc_pack_all(const TcPackJob *jobs_dev, int njobs, size_t total, cudaStream_t st);
// Extra stores of a forward convolution's epilogue, so that the network's
// pooling, upsampling + concatenation, residual and output transform need no
// kernels of their own. Each takes the values exactly as the separate kernel
// would (the BF16-rounded outputs; the FP32 output plus the residual), so the
// results are the same bits.
//   pool: the 2 x 2 average of the BF16 outputs, (h / 2) x (w / 2) x cout;
//   cat:  the BF16 outputs also into channels [cat_off, cat_off + cout) of a
//         cat_c-channel tensor, at the same pixel (cat_up 0) or, nearest 2x
//         upsampling, at the 2 x 2 block of a 2h x 2w tensor (cat_up 1);
//   res:  FP32 output += res[pixel * res_c + channel] (BF16);
//   rad:  (cout 3) rad = expm1(FP32 output) * (max(albedo, 0) + kDemodFloor),
//         the albedo from feat (7 halves per pixel).
// pool and cat need cout a multiple of 16, res and rad the FP32 output; none
// works with a tap split (p.splits > 1).
struct TcFuse {
    __nv_bfloat16 *pool = nullptr;
    __nv_bfloat16 *cat = nullptr;
    int cat_c = 0, cat_off = 0, cat_up = 0;
    const __nv_bfloat16 *res = nullptr;
    int res_c = 0;
    float *rad = nullptr;
    const __half *feat = nullptr;
};
cudaError_t conv3x3_forward_tc(const TcConvPlan &p, const __nv_bfloat16 *wpacked, const float *bias,
                               __nv_bfloat16 *y, float *y32, float *partial, int *err, cudaStream_t st,
                               const TcFuse *fuse = nullptr, bool overlap_prologue = false);
// overlap_prologue: launch with programmatic stream serialisation, so that the
// kernel's prologue (barriers, tensor memory, weight copies) overlaps the
// previous kernel of the stream; its input copies wait for that kernel to
// complete. The previous kernel must not write the weights or the bias.
// Weight gradient of a 3x3 convolution on the tensor cores:
// dw[co][tap][ci] += sum over pixels p of g[p][co] * x[p + offset(tap)][ci],
// a GEMM with M = output channels (padded to 128), N = input channels, K =
// pixels. g: the output gradient as BF16 with cout_pad = cout rounded up to
// 16 channels (grad_bf16); x: the convolution's input, read through the
// forward plan's halo tensor map (fwd: a plan over x with cin = cin_pad).
// Each CTA accumulates the nine taps (or a group of them, as many as tensor
// memory holds) over a group of 16 x 8 tiles and writes them to `partial`
// (partial_floats floats); a second kernel adds the groups in order into dw.
struct TcWgradPlan {
    alignas(64) unsigned char gmap[128];  // CUtensorMap of g: (cout_pad, W, H, N), box (8, 8, 16, 1)
    const __nv_bfloat16 *g;
    int n, h, w, cin, cin_pad, cout, cout_pad;
    int tiles_x, tiles_y, tiles, tiles_per_cta, groups, taps_per_pass, passes, tmem_cols, stages;
    uint32_t b_off, stage_bytes, bar_off;
    size_t smem, partial_floats;
};
cudaError_t tc_wgrad_plan(TcWgradPlan &p, const __nv_bfloat16 *g, int n, int h, int w, int cin, int cin_pad, int cout,
                          int sm_count);
cudaError_t conv3x3_wgrad_tc(const TcWgradPlan &p, const TcConvPlan &fwd, float *dw, float *partial, int *err,
                             cudaStream_t st);
cudaError_t conv3x3_forward(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *b, __nv_bfloat16 *y,
                            float *y32, int n, int h, int wd, int cin, int cout, bool relu, cudaStream_t st);
// gpre: output gradient after the ReLU mask (FP32, n*h*w*cout); dx may be NULL
cudaError_t conv3x3_backward(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *gpre, float *dx, float *dw,
                             float *db, int n, int h, int wd, int cin, int cout, cudaStream_t st);
cudaError_t relu_mask(const __nv_bfloat16 *y, const float *g, float *out, size_t n, cudaStream_t st);
// db[c] += sum over pixels of g[p][c]
cudaError_t bias_grad(const float *g, float *db, size_t pixels, int c, cudaStream_t st);
// One pass over a convolution's output gradient g (pixels x c FP32) for the
// tensor-core backward: the ReLU mask of the convolution's output y (NULL:
// no mask), the masked gradient as BF16 with c_pad >= c channels (the pad
// zero), and the bias gradient: per-block partial sums in part
// (kGradPrepBlocks x c floats), added in block order into db.
constexpr int kGradPrepBlocks = 1024;
cudaError_t grad_prep(const __nv_bfloat16 *y, const float *g, __nv_bfloat16 *out, float *part, float *db,
                      size_t pixels, int c, int c_pad, cudaStream_t st);
// g (pixels x c FP32) as BF16 with c_pad >= c channels (the pad zero)
cudaError_t grad_bf16(const float *g, __nv_bfloat16 *out, size_t pixels, int c, int c_pad, cudaStream_t st);
cudaError_t avgpool(const __nv_bfloat16 *x, __nv_bfloat16 *y, int n, int h, int w, int c, cudaStream_t st);
cudaError_t avgpool_backward(const float *gy, float *gx, int n, int h, int w, int c, cudaStream_t st);
cudaError_t upsample_backward(const float *gy, float *gx, int n, int h, int w, int c, int cy, cudaStream_t st);
cudaError_t split_add(const float *gy, float *gx, size_t pixels, int c, int cy, int off, cudaStream_t st);
// Radiance is demodulated by the first-hit albedo: divided by
// max(albedo, 0) + kDemodFloor (per channel) on the way in and in the loss's
// target, multiplied back on the way out.
constexpr float kDemodFloor = 0.05f;
// x (may be NULL): 10 channels; x16 (may be NULL): the same padded to 16 channels
cudaError_t pack_input(const float *rad, const __half *feat, __nv_bfloat16 *x, __nv_bfloat16 *x16, size_t pixels,
                       cudaStream_t st);
// cat = [nearest 2x upsampling of low (c channels, h x w), skip (cs channels)]
cudaError_t upsample_concat(const __nv_bfloat16 *low, const __nv_bfloat16 *skip, __nv_bfloat16 *cat, int n, int h,
                            int w, int c, int cs, cudaStream_t st);
// L1 loss (mean over the n values, into loss[0]) and its gradient; part:
// scratch of kL1Parts floats (per-block sums, added in a fixed order)
constexpr int kL1Parts = 152 * 32;
cudaError_t l1_loss(const float *out, const float *target, const __half *feat, float *g, float *loss, float *part,
                    size_t n, cudaStream_t st);
// out (3 channels) += the first 3 of x0's x0_c channels (the input's log radiance)
cudaError_t add_input(float *out, const __nv_bfloat16 *x0, int x0_c, size_t pixels, cudaStream_t st);
cudaError_t expm1_out(const float *out, const __half *feat, float *rad, size_t n, cudaStream_t st);
cudaError_t adam(float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, size_t n, float lr, float b1,
                 float b2, float eps, int step, cudaStream_t st);
cudaError_t to_bf16(const float *a, __nv_bfloat16 *b, size_t n, cudaStream_t st);

}  // namespace dn
}  // namespace pray_gpu
