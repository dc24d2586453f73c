// U-Net denoiser state on one device (denoise_net.cpp).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "denoise_ops.h"

namespace pray_gpu {

class Denoiser {
  public:
    ~Denoiser();
    cudaError_t init(uint64_t seed);
    size_t num_params() const { return n_params_; }
    cudaError_t set_params(const float *host);
    cudaError_t get_params(float *host) const;
    cudaError_t get_grads(float *host) const;
    // radiance: n*h*w*3 floats, feat: n*h*w*7 halves (albedo, normal, depth);
    // h and w multiples of 16. The network output stays on the device; feat
    // must stay valid through the backward / output_radiance that follow.
    // With out_rad (inference) the denoised radiance also goes there, and the
    // activations that only the backward pass reads may not be stored.
    cudaError_t forward(const float *rad, const __half *feat, int n, int h, int w, cudaStream_t st,
                        float *out_rad = nullptr);
    // after forward: L1 loss against the target radiance, all gradients
    cudaError_t backward(const float *target, cudaStream_t st);
    cudaError_t apply_adam(float lr, cudaStream_t st);
    cudaError_t output_radiance(float *out, cudaStream_t st);
    // forward + output_radiance; a call with the same buffers, sizes and
    // kernel choice as the previous one replays them from a CUDA graph
    cudaError_t denoise(const float *rad, const __half *feat, int n, int h, int w, float *out, cudaStream_t st);
    const float *loss_device() const { return loss_; }
    // forward and backward-data convolutions on the tcgen05 tensor cores
    // (default) or on the CUDA cores
    void set_tensor_cores(bool on) { tensor_cores_ = on; }
    bool tensor_cores() const { return tensor_cores_; }
    // synchronises; false if a tensor-core kernel reported a timed-out wait
    cudaError_t check(bool &ok);
    int device = 0;

  private:
    struct Conv {
        int cin, cout;
        bool relu;
        size_t offset;  // weights [cout][9][cin] then bias [cout] in the parameter vector
    };
    struct Buf {
        int level = 0, c = 0;
        __nv_bfloat16 *x = nullptr;
        float *g = nullptr;
    };
    template <class T>
    cudaError_t take(T *&p, size_t n);
    cudaError_t ensure(int n, int h, int w);
    cudaError_t conv_fwd(int ci, const Buf &in, __nv_bfloat16 *y, float *y32, cudaStream_t st,
                         const dn::TcFuse *fuse = nullptr, bool overlap = false);
    // the tensor-core plan of convolution ci on input `in` (made on first use)
    cudaError_t tc_plan(int ci, const Buf &in, dn::TcConvPlan *&plan);
    // packed BF16 weights of the tensor-core kernel, from the FP32 master copy
    cudaError_t refresh_tc_weights(cudaStream_t st);
    void release();

    std::vector<Conv> convs_;
    std::vector<Buf> act_;
    std::vector<float *> grad_;
    std::vector<void *> owned_;
    size_t n_params_ = 0, cap_pixels_ = 0;
    int n_ = 0, h_ = 0, w_dim_ = 0, step_ = 0;
    float *w_ = nullptr, *g_ = nullptr, *m_ = nullptr, *v_ = nullptr, *loss_ = nullptr;
    __nv_bfloat16 *wb_ = nullptr;
    // tensor-core forward: packed weights (offsets per conv), the input padded
    // to 16 channels, split-tap partial sums, one plan per convolution
    __nv_bfloat16 *wtc_ = nullptr, *x16_ = nullptr;
    std::vector<size_t> tc_off_;
    float *partial_ = nullptr;
    std::vector<dn::TcConvPlan> plans_;
    int sm_count_ = 0;
    // tensor-core backward-data: per convolution the transposed, tap-mirrored
    // packed weights (dn::tc_pack_weights_bwd) and a plan over the output
    // gradient in BF16 (gb16_), and a zero bias
    __nv_bfloat16 *wtcb_ = nullptr, *gb16_ = nullptr;
    std::vector<size_t> tcb_off_;
    std::vector<dn::TcConvPlan> plans_bwd_;
    float *zero_bias_ = nullptr;
    // every forward and backward-data packing as one launch (dn::tc_pack_all)
    dn::TcPackJob *pack_jobs_ = nullptr;
    int n_pack_jobs_ = 0;
    size_t pack_total_ = 0;
    // tensor-core weight gradients: one plan per convolution, per-group partial sums
    std::vector<dn::TcWgradPlan> plans_wg_;
    float *partial_wg_ = nullptr;
    float *bias_part_ = nullptr;  // per-block bias-gradient sums (dn::grad_prep)
    float *out_ = nullptr, *gout_ = nullptr, *gtmp_ = nullptr;
    const __half *feat_ = nullptr;  // features of the last forward (the caller's buffer; used until the call returns)
    int *err_ = nullptr;
    bool tensor_cores_ = true;
    // the captured denoise call and what it was captured for; generation_
    // counts reallocations of the activation buffers
    struct GraphKey {
        const float *rad = nullptr;
        const __half *feat = nullptr;
        float *out = nullptr;
        int n = 0, h = 0, w = 0;
        bool tensor_cores = false;
        uint64_t generation = 0;
        bool operator==(const GraphKey &o) const {
            return rad == o.rad && feat == o.feat && out == o.out && n == o.n && h == o.h && w == o.w &&
                   tensor_cores == o.tensor_cores && generation == o.generation;
        }
    };
    GraphKey graph_key_{};
    cudaGraphExec_t graph_ = nullptr;
    cudaStream_t capture_stream_ = nullptr;
    uint64_t generation_ = 0;
};

}  // namespace pray_gpu
