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

// tcgen05 tensor-core version (denoise_tc.cu); *err is set to 1 if one of
// its bounded mbarrier waits ran out
cudaError_t conv3x3_forward_tc(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *b, __nv_bfloat16 *y,
                               float *y32, int n, int h, int wd, int cin, int cout, bool relu, int *err,
                               cudaStream_t st);
cudaError_t conv3x3_forward(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *b, __nv_bfloat16 *y,
                            float *y32, int n, int h, int wd, int cin, int cout, bool relu, cudaStream_t st);
// gpre: output gradient after the ReLU mask (FP32, n*h*w*cout); dx may be NULL
cudaError_t conv3x3_backward(const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *gpre, float *dx, float *dw,
                             float *db, int n, int h, int wd, int cin, int cout, cudaStream_t st);
cudaError_t relu_mask(const __nv_bfloat16 *y, const float *g, float *out, size_t n, cudaStream_t st);
cudaError_t avgpool(const __nv_bfloat16 *x, __nv_bfloat16 *y, int n, int h, int w, int c, cudaStream_t st);
cudaError_t avgpool_backward(const float *gy, float *gx, int n, int h, int w, int c, cudaStream_t st);
cudaError_t upsample(const __nv_bfloat16 *x, __nv_bfloat16 *y, int n, int h, int w, int c, int cy, cudaStream_t st);
cudaError_t upsample_backward(const float *gy, float *gx, int n, int h, int w, int c, int cy, cudaStream_t st);
cudaError_t concat(const __nv_bfloat16 *x, __nv_bfloat16 *y, size_t pixels, int c, int cy, int off, cudaStream_t st);
cudaError_t split_add(const float *gy, float *gx, size_t pixels, int c, int cy, int off, cudaStream_t st);
cudaError_t pack_input(const float *rad, const __half *feat, __nv_bfloat16 *x, size_t pixels, cudaStream_t st);
cudaError_t l1_loss(const float *out, const float *target, float *g, float *loss, size_t n, cudaStream_t st);
cudaError_t add_input(float *out, const __nv_bfloat16 *x0, size_t pixels, cudaStream_t st);
cudaError_t expm1_out(const float *out, float *rad, size_t n, cudaStream_t st);
cudaError_t adam(float *w, const float *g, float *m, float *v, __nv_bfloat16 *wb, size_t n, float lr, float b1,
                 float b2, float eps, int step, cudaStream_t st);
cudaError_t to_bf16(const float *a, __nv_bfloat16 *b, size_t n, cudaStream_t st);

}  // namespace dn
}  // namespace pray_gpu
