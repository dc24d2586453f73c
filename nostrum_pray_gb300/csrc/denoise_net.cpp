// The denoiser network on the device: a five-level convolutional U-Net
// (channels 32-48-64-96-128, two 3x3 convolutions with ReLU per level, 2x2
// average pooling down, nearest 2x upsampling up, skip connections by channel
// concatenation, a final 3x3 convolution to RGB). Input per pixel:
// log(1 + radiance) of the noisy render (3), first-hit albedo (3), normal (3)
// and depth (1); output: log(1 + radiance) of the estimate, as the noisy
// input's log(1 + radiance) plus the network's correction. Trained with an L1
// loss in that log space and Adam. Every kernel is in denoise_ops.cu.
#include "denoise_net.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>

namespace pray_gpu {

namespace {

// (cin, cout, relu) of the 19 convolutions in forward order
const int kConvs[][3] = {
    {10, 32, 1}, {32, 32, 1},     // e0
    {32, 48, 1}, {48, 48, 1},     // e1
    {48, 64, 1}, {64, 64, 1},     // e2
    {64, 96, 1}, {96, 96, 1},     // e3
    {96, 128, 1}, {128, 128, 1},  // e4 (bottleneck)
    {224, 96, 1}, {96, 96, 1},    // d3: up(e4) 128 + e3 96
    {160, 64, 1}, {64, 64, 1},    // d2: up(d3) 96 + e2 64
    {112, 48, 1}, {48, 48, 1},    // d1: up(d2) 64 + e1 48
    {80, 32, 1}, {32, 32, 1},     // d0: up(d1) 48 + e0 32
    {32, 3, 0},                   // out
};
constexpr int kNumConvs = 19;
const int kEnc[5] = {32, 48, 64, 96, 128};
// resolution level (size >> level) of each convolution
const int kLevel[kNumConvs] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0};

int pad16(int c) { return (c + 15) / 16 * 16; }

template <class T>
cudaError_t dalloc(T *&p, size_t n) {
    return cudaMalloc(reinterpret_cast<void **>(&p), std::max<size_t>(n, 1) * sizeof(T));
}

}  // namespace

Denoiser::~Denoiser() { release(); }

void Denoiser::release() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
    capture_stream_ = nullptr;
    for (void *p : owned_) cudaFree(p);
    owned_.clear();
    act_.clear();
    grad_.clear();
    cap_pixels_ = 0;
}

template <class T>
cudaError_t Denoiser::take(T *&p, size_t n) {
    cudaError_t e = dalloc(p, n);
    if (e == cudaSuccess) owned_.push_back(p);
    return e;
}

cudaError_t Denoiser::init(uint64_t seed) {
    convs_.resize(kNumConvs);
    size_t total = 0;
    for (int i = 0; i < kNumConvs; i++) {
        Conv &c = convs_[i];
        c.cin = kConvs[i][0];
        c.cout = kConvs[i][1];
        c.relu = kConvs[i][2] != 0;
        c.offset = total;
        total += (size_t)c.cout * 9 * c.cin + c.cout;
    }
    n_params_ = total;
    size_t tc_total = 0;
    tc_off_.resize(kNumConvs);
    for (int i = 0; i < kNumConvs; i++) {
        tc_off_[i] = tc_total;
        tc_total += dn::tc_packed_weight_elems(pad16(convs_[i].cin), convs_[i].cout);
    }
    // backward-data weights: the first convolution's input needs no gradient
    size_t tcb_total = 0;
    tcb_off_.assign(kNumConvs, 0);
    for (int i = 1; i < kNumConvs; i++) {
        tcb_off_[i] = tcb_total;
        tcb_total += dn::tc_packed_weight_elems(pad16(convs_[i].cout), convs_[i].cin);
    }
    plans_.assign(kNumConvs, dn::TcConvPlan{});
    plans_bwd_.assign(kNumConvs, dn::TcConvPlan{});
    plans_wg_.assign(kNumConvs, dn::TcWgradPlan{});
    cudaError_t e;
    if ((e = cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return e;
    if ((e = take(w_, total)) != cudaSuccess || (e = take(g_, total)) != cudaSuccess ||
        (e = take(m_, total)) != cudaSuccess || (e = take(v_, total)) != cudaSuccess ||
        (e = take(wb_, total)) != cudaSuccess || (e = take(wtc_, tc_total)) != cudaSuccess ||
        (e = take(wtcb_, tcb_total)) != cudaSuccess || (e = take(zero_bias_, 256)) != cudaSuccess ||
        (e = cudaMemset(zero_bias_, 0, 256 * sizeof(float))) != cudaSuccess ||
        (e = take(loss_, 1 + dn::kL1Parts)) != cudaSuccess || (e = take(err_, 1)) != cudaSuccess ||
        (e = cudaMemset(err_, 0, sizeof(int))) != cudaSuccess)
        return e;
    // He-normal weights, zero biases, from the seed
    std::vector<float> h(total, 0.f);
    std::mt19937_64 rng(seed);
    for (const Conv &c : convs_) {
        // the output convolution starts small, so the initial estimate is the
        // noisy input
        const float scale = c.relu ? 1.f : 0.1f;
        std::normal_distribution<float> nd(0.f, scale * std::sqrt(2.f / (9.f * c.cin)));
        const size_t nw = (size_t)c.cout * 9 * c.cin;
        for (size_t k = 0; k < nw; k++) h[c.offset + k] = nd(rng);
    }
    std::vector<float> zeros(total, 0.f);
    if ((e = cudaMemcpy(w_, h.data(), total * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m_, zeros.data(), total * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(v_, zeros.data(), total * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    step_ = 0;
    // the packing jobs: each convolution's forward weights, then its
    // backward-data weights (all but the first)
    std::vector<dn::TcPackJob> jobs;
    size_t begin = 0;
    for (int i = 0; i < kNumConvs; i++) {
        const Conv &c = convs_[i];
        for (int bwd = 0; bwd < (i > 0 ? 2 : 1); bwd++) {
            dn::TcPackJob j;
            j.w = w_ + c.offset;
            j.out = bwd ? wtcb_ + tcb_off_[i] : wtc_ + tc_off_[i];
            j.begin = begin;
            j.cin_f = c.cin, j.cout_f = c.cout, j.bwd = bwd;
            j.cin_pad = bwd ? pad16(c.cout) : pad16(c.cin);
            j.npad = bwd ? pad16(c.cin) : pad16(c.cout);
            begin += (size_t)9 * j.cin_pad * j.npad;
            jobs.push_back(j);
        }
    }
    n_pack_jobs_ = (int)jobs.size();
    pack_total_ = begin;
    if ((e = take(pack_jobs_, jobs.size())) != cudaSuccess ||
        (e = cudaMemcpy(pack_jobs_, jobs.data(), jobs.size() * sizeof(dn::TcPackJob), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
        return e;
    if ((e = dn::to_bf16(w_, wb_, total, 0)) != cudaSuccess) return e;
    if ((e = refresh_tc_weights(0)) != cudaSuccess) return e;
    // the converted and packed weights are in place before any stream
    // (blocking or not) runs a pass with them
    return cudaStreamSynchronize(0);
}

cudaError_t Denoiser::refresh_tc_weights(cudaStream_t st) {
    return dn::tc_pack_all(pack_jobs_, n_pack_jobs_, pack_total_, st);
}

cudaError_t Denoiser::set_params(const float *host) {
    cudaError_t e = cudaMemcpy(w_, host, n_params_ * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    if ((e = dn::to_bf16(w_, wb_, n_params_, 0)) != cudaSuccess) return e;
    if ((e = refresh_tc_weights(0)) != cudaSuccess) return e;
    return cudaStreamSynchronize(0);
}

cudaError_t Denoiser::get_params(float *host) const {
    return cudaMemcpy(host, w_, n_params_ * 4, cudaMemcpyDeviceToHost);
}

cudaError_t Denoiser::get_grads(float *host) const {
    return cudaMemcpy(host, g_, n_params_ * 4, cudaMemcpyDeviceToHost);
}

// Activation and gradient buffers for n images of h x w (h, w multiples of 16).
cudaError_t Denoiser::ensure(int n, int h, int w) {
    const size_t px = (size_t)n * h * w;
    if (px <= cap_pixels_ && h == h_ && w == w_dim_ && n == n_) return cudaSuccess;
    // keep the parameters, drop the activations
    std::vector<void *> keep = {w_, g_, m_, v_, wb_, wtc_, wtcb_, zero_bias_, pack_jobs_, loss_, err_};
    partial_ = nullptr;
    x16_ = nullptr;
    gb16_ = nullptr;
    bias_part_ = nullptr;
    partial_wg_ = nullptr;
    plans_.assign(kNumConvs, dn::TcConvPlan{});
    plans_bwd_.assign(kNumConvs, dn::TcConvPlan{});
    plans_wg_.assign(kNumConvs, dn::TcWgradPlan{});
    for (void *p : owned_)
        if (std::find(keep.begin(), keep.end(), p) == keep.end()) cudaFree(p);
    owned_ = keep;
    generation_++;
    act_.clear();
    grad_.clear();
    n_ = n, h_ = h, w_dim_ = w;
    cudaError_t e;
    auto act = [&](int level, int c, bool with_grad) -> cudaError_t {
        const size_t p = (size_t)n * (h >> level) * (w >> level);
        Buf b;
        b.level = level;
        b.c = c;
        cudaError_t er = take(b.x, p * c);
        if (er != cudaSuccess) return er;
        if (with_grad && (er = take(b.g, p * c)) != cudaSuccess) return er;
        act_.push_back(b);
        return cudaSuccess;
    };
    // act_ layout (index: tensor):
    //  0 x0(10)
    //  1 e0a 2 e0 | 3 p1 4 e1a 5 e1 | 6 p2 7 e2a 8 e2 | 9 p3 10 e3a 11 e3 | 12 p4 13 e4a 14 e4
    //  15 cat3 16 d3a 17 d3 | 18 cat2 19 d2a 20 d2 | 21 cat1 22 d1a 23 d1 | 24 cat0 25 d0a 26 d0
    if ((e = act(0, 10, false)) != cudaSuccess) return e;
    for (int l = 0; l < 5; l++) {
        if (l > 0 && (e = act(l, kEnc[l - 1], true)) != cudaSuccess) return e;  // pooled input
        if ((e = act(l, kEnc[l], true)) != cudaSuccess) return e;
        if ((e = act(l, kEnc[l], true)) != cudaSuccess) return e;
    }
    for (int l = 3; l >= 0; l--) {
        const int up = (l == 3) ? kEnc[4] : kEnc[l + 1];
        if ((e = act(l, up + kEnc[l], true)) != cudaSuccess) return e;  // concat
        if ((e = act(l, kEnc[l], true)) != cudaSuccess) return e;
        if ((e = act(l, kEnc[l], true)) != cudaSuccess) return e;
    }
    if ((e = take(out_, px * 3)) != cudaSuccess || (e = take(gout_, px * 3)) != cudaSuccess ||
        (e = take(gtmp_, px * 128)) != cudaSuccess || (e = take(x16_, px * pad16(kConvs[0][0]))) != cudaSuccess ||
        (e = take(gb16_, px * 128)) != cudaSuccess ||
        (e = take(bias_part_, (size_t)dn::kGradPrepBlocks * 128)) != cudaSuccess)
        return e;
    // split-tap partial sums of the tensor-core kernel: the largest need of
    // any forward or backward-data convolution; per-group weight-gradient sums
    size_t partial = 0, partial_wg = 0;
    for (int i = 0; i < kNumConvs; i++) {
        dn::TcConvPlan shape;
        const int l = kLevel[i];
        if (dn::tc_conv_plan(shape, act_[0].x, n, h >> l, w >> l, pad16(kConvs[i][0]), kConvs[i][1], true,
                             sm_count_) == cudaSuccess)
            partial = std::max(partial, shape.partial_floats);
        if (i > 0 && dn::tc_conv_plan(shape, act_[0].x, n, h >> l, w >> l, pad16(kConvs[i][1]), kConvs[i][0], false,
                                      sm_count_) == cudaSuccess)
            partial = std::max(partial, shape.partial_floats);
        dn::TcWgradPlan wg;
        if (dn::tc_wgrad_plan(wg, act_[0].x, n, h >> l, w >> l, kConvs[i][0], pad16(kConvs[i][0]), kConvs[i][1],
                              sm_count_) == cudaSuccess)
            partial_wg = std::max(partial_wg, wg.partial_floats);
    }
    if (partial_wg && (e = take(partial_wg_, partial_wg)) != cudaSuccess) return e;
    if (partial && (e = take(partial_, partial)) != cudaSuccess) return e;
    cap_pixels_ = px;
    return cudaSuccess;
}

cudaError_t Denoiser::check(bool &ok) {
    cudaError_t e = cudaDeviceSynchronize();
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flag, err_, sizeof(int), cudaMemcpyDeviceToHost);
    ok = flag == 0;
    return e;
}

cudaError_t Denoiser::tc_plan(int ci, const Buf &in, dn::TcConvPlan *&plan) {
    const Conv &c = convs_[ci];
    const int h = h_ >> in.level, w = w_dim_ >> in.level;
    const __nv_bfloat16 *x = in.x;
    const int cin = pad16(c.cin);
    if (cin != c.cin) {
        if (ci != 0) return cudaErrorInvalidValue;  // only the 10-channel input is padded (by pack_input)
        x = x16_;
    }
    dn::TcConvPlan &pl = plans_[ci];
    if (pl.x != x || pl.n != n_ || pl.h != h || pl.w != w) {
        cudaError_t e = dn::tc_conv_plan(pl, x, n_, h, w, cin, c.cout, c.relu, sm_count_);
        if (e != cudaSuccess) {
            pl.x = nullptr;
            return e;
        }
    }
    plan = &pl;
    return cudaSuccess;
}

cudaError_t Denoiser::conv_fwd(int ci, const Buf &in, __nv_bfloat16 *y, float *y32, cudaStream_t st,
                               const dn::TcFuse *fuse, bool overlap) {
    const Conv &c = convs_[ci];
    const int h = h_ >> in.level, w = w_dim_ >> in.level;
    const float *bias = w_ + c.offset + (size_t)c.cout * 9 * c.cin;
    if (!tensor_cores_)
        return dn::conv3x3_forward(in.x, wb_ + c.offset, bias, y, y32, n_, h, w, c.cin, c.cout, c.relu, st);
    dn::TcConvPlan *pl = nullptr;
    cudaError_t e = tc_plan(ci, in, pl);
    if (e != cudaSuccess) return e;
    return dn::conv3x3_forward_tc(*pl, wtc_ + tc_off_[ci], bias, y, y32, partial_, err_, st, fuse, overlap);
}

cudaError_t Denoiser::forward(const float *rad, const __half *feat, int n, int h, int w, cudaStream_t st,
                              float *out_rad) {
    if (h % 16 || w % 16 || n <= 0) return cudaErrorInvalidValue;
    cudaError_t e = ensure(n, h, w);
    if (e != cudaSuccess) return e;
    const size_t px = (size_t)n * h * w;
    auto chk = [&](cudaError_t x) { if (x != cudaSuccess && e == cudaSuccess) e = x; };
    feat_ = feat;
    // the tensor cores read the input padded to 16 channels (x16_), also for
    // the residual and the first convolution's weight gradient: the
    // 10-channel copy is written only for the CUDA cores
    chk(dn::pack_input(rad, feat, tensor_cores_ ? nullptr : act_[0].x, tensor_cores_ ? x16_ : nullptr, px, st));
    const __nv_bfloat16 *x0 = tensor_cores_ ? x16_ : act_[0].x;
    const int x0_c = tensor_cores_ ? pad16(kConvs[0][0]) : act_[0].c;
    // On the tensor cores the poolings and the upsampling + concatenations are
    // stores of the convolutions' epilogues (dn::TcFuse): the second
    // convolution of encoder level l < 4 also writes the pooled input of level
    // l + 1 and its output into the skip channels of cat_l; the second
    // convolution of level l > 0 (bottleneck, decoder) writes its output,
    // upsampled, into the first channels of cat_{l-1}. For inference (out_rad)
    // those convolutions' own outputs, which only the backward pass reads,
    // are not stored. Each convolution's prologue overlaps the previous
    // kernel (programmatic dependent launch): the packed weights it loads
    // there are written only by the packing after the optimizer step, which
    // completes before input packing starts.
    const bool fuse = tensor_cores_, infer = out_rad != nullptr;
    const int kCat[4] = {24, 21, 18, 15};  // act_ index of cat_l (layout in ensure)
    int conv = 0;
    // encoder
    int idx = 1, prev = 0;
    for (int l = 0; l < 5; l++) {
        if (l > 0) {
            const Buf &src = act_[prev];
            if (!fuse) chk(dn::avgpool(src.x, act_[idx].x, n, h >> (l - 1), w >> (l - 1), src.c, st));
            prev = idx++;
        }
        chk(conv_fwd(conv++, act_[prev], act_[idx].x, nullptr, st, nullptr, fuse));
        prev = idx++;
        dn::TcFuse f;
        const Buf &cat = act_[kCat[l < 4 ? l : 3]];
        f.cat = cat.x, f.cat_c = cat.c;
        if (l < 4) {
            f.pool = act_[idx + 1].x;
            f.cat_off = cat.c - kEnc[l];
        } else {
            f.cat_up = 1;
        }
        chk(conv_fwd(conv++, act_[prev], fuse && infer ? nullptr : act_[idx].x, nullptr, st, fuse ? &f : nullptr,
                     fuse));
        prev = idx++;
    }
    // decoder: prev = e4 (index 14)
    const int skip_idx[4] = {11, 8, 5, 2};  // e3, e2, e1, e0
    for (int k = 0; k < 4; k++) {
        const int l = 3 - k;
        Buf &cat = act_[idx];
        const Buf &low = act_[prev];
        const Buf &skip = act_[skip_idx[k]];
        if (!fuse)
            chk(dn::upsample_concat(low.x, skip.x, cat.x, n, h >> (l + 1), w >> (l + 1), low.c, skip.c, st));
        prev = idx++;
        chk(conv_fwd(conv++, act_[prev], act_[idx].x, nullptr, st, nullptr, fuse));
        prev = idx++;
        dn::TcFuse f;
        const bool up = fuse && l > 0;
        if (up) f.cat = act_[kCat[l - 1]].x, f.cat_c = act_[kCat[l - 1]].c, f.cat_up = 1;
        chk(conv_fwd(conv++, act_[prev], up && infer ? nullptr : act_[idx].x, nullptr, st, up ? &f : nullptr,
                     fuse));
        prev = idx++;
    }
    // output convolution (no ReLU), FP32; the network predicts a correction
    // to the noisy input's log radiance (residual), and the output transform
    // gives radiance: both in its epilogue unless it splits its taps
    dn::TcConvPlan *pl = nullptr;
    bool fused_out = false;
    if (fuse && e == cudaSuccess) {
        chk(tc_plan(conv, act_[prev], pl));
        fused_out = pl && pl->splits == 1;
    }
    if (fused_out) {
        dn::TcFuse f;
        f.res = x0, f.res_c = x0_c;
        f.rad = out_rad, f.feat = feat;
        chk(conv_fwd(conv, act_[prev], nullptr, out_, st, &f, fuse));
    } else {
        chk(conv_fwd(conv, act_[prev], nullptr, out_, st));
        chk(dn::add_input(out_, x0, x0_c, px, st));
        if (infer) chk(output_radiance(out_rad, st));
    }
    return e;
}

cudaError_t Denoiser::backward(const float *target, cudaStream_t st) {
    const int n = n_, h = h_, w = w_dim_;
    const size_t px = (size_t)n * h * w;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (x != cudaSuccess && e == cudaSuccess) e = x; };
    chk(cudaMemsetAsync(g_, 0, n_params_ * 4, st));
    for (Buf &b : act_)
        if (b.g) chk(cudaMemsetAsync(b.g, 0, (size_t)n * (h >> b.level) * (w >> b.level) * b.c * 4, st));
    chk(dn::l1_loss(out_, target, feat_, gout_, loss_, loss_ + 1, px * 3, st));
    // input gradient (when need_dx) and weight / bias gradients of convolution
    // ci from its output gradient g, masked by the ReLU of its output y (NULL:
    // no ReLU). With the tensor cores the input gradient is a forward
    // convolution of the masked gradient (BF16) with the transposed,
    // tap-mirrored weights, and one pass over g gives that BF16 operand and
    // the bias gradient.
    auto conv_bwd = [&](int ci, Buf &in, const float *g, const __nv_bfloat16 *y, int level, bool need_dx) {
        const Conv &c = convs_[ci];
        const int hh = h >> level, ww = w >> level;
        const size_t p = (size_t)n * hh * ww;
        float *dw = g_ + c.offset, *db = dw + (size_t)c.cout * 9 * c.cin;
        if (!tensor_cores_) {
            const float *gpre = g;
            if (y) {
                chk(dn::relu_mask(y, g, gtmp_, p * c.cout, st));
                gpre = gtmp_;
            }
            chk(dn::conv3x3_backward(in.x, wb_ + c.offset, gpre, need_dx ? in.g : nullptr, dw, db, n, hh, ww, c.cin,
                                     c.cout, st));
            return;
        }
        chk(dn::grad_prep(y, g, gb16_, bias_part_, db, p, c.cout, pad16(c.cout), st));
        if (need_dx) {
            dn::TcConvPlan &pl = plans_bwd_[ci];
            if (pl.x != gb16_ || pl.n != n || pl.h != hh || pl.w != ww) {
                cudaError_t pe = dn::tc_conv_plan(pl, gb16_, n, hh, ww, pad16(c.cout), c.cin, false, sm_count_);
                if (pe != cudaSuccess) {
                    pl.x = nullptr;
                    chk(pe);
                    return;
                }
            }
            // programmatic launch: its prologue loads the transposed weights
            // (packed after the last optimizer step) while the bias
            // gradient's final sums (the last kernel of grad_prep) run
            chk(dn::conv3x3_forward_tc(pl, wtcb_ + tcb_off_[ci], zero_bias_, nullptr, in.g, partial_, err_, st,
                                       nullptr, true));
        }
        dn::TcWgradPlan &wg = plans_wg_[ci];
        if (wg.g != gb16_ || wg.n != n || wg.h != hh || wg.w != ww) {
            cudaError_t pe = dn::tc_wgrad_plan(wg, gb16_, n, hh, ww, c.cin, pad16(c.cin), c.cout, sm_count_);
            if (pe != cudaSuccess) {
                wg.g = nullptr;
                chk(pe);
                return;
            }
        }
        chk(dn::conv3x3_wgrad_tc(wg, plans_[ci], dw, partial_wg_, err_, st));
    };
    // output conv: input d0 (26), no ReLU
    conv_bwd(18, act_[26], gout_, nullptr, 0, true);
    // layer tensor i was produced by conv j from tensor i-1 (within a level)
    // backward through (conv j: i-1 -> i) with the ReLU mask on i's gradient
    auto through = [&](int ci, int out_idx) {
        Buf &o = act_[out_idx];
        conv_bwd(ci, act_[out_idx - 1], o.g, o.x, o.level, true);
    };
    const int skip_idx[4] = {11, 8, 5, 2};
    // decoder, deepest last in forward => first here: d0 (convs 16,17), d1 (14,15), d2 (12,13), d3 (10,11)
    for (int k = 3; k >= 0; k--) {
        const int l = 3 - k;
        const int cat_idx = 15 + 3 * k;
        through(11 + 2 * k - 0 + 0 * l, cat_idx + 2);  // second conv of the level
        through(10 + 2 * k, cat_idx + 1);              // first conv (input: concat)
        Buf &cat = act_[cat_idx];
        const Buf &skip = act_[skip_idx[k]];
        const int low_idx = (k == 0) ? 14 : cat_idx - 1;  // e4 or the previous level's second conv
        Buf &low = act_[low_idx];
        const size_t p = (size_t)n * (h >> l) * (w >> l);
        chk(dn::split_add(cat.g, act_[skip_idx[k]].g, p, skip.c, cat.c, low.c, st));
        chk(dn::upsample_backward(cat.g, low.g, n, h >> (l + 1), w >> (l + 1), low.c, cat.c, st));
    }
    // encoder, deepest first: level l tensors: pooled (l>0), a, b
    for (int l = 4; l >= 0; l--) {
        const int b_idx = (l == 0) ? 2 : 3 * l + 2;
        through(2 * l + 1, b_idx);
        if (l == 0) {
            // first conv's input is x0 (no gradient needed): weights only
            conv_bwd(0, act_[0], act_[1].g, act_[1].x, 0, false);
        } else {
            through(2 * l, b_idx - 1);
            // pooled tensor (b_idx - 2) came from the previous level's output
            const int src = (l == 1) ? 2 : 3 * (l - 1) + 2;
            const Buf &pooled = act_[b_idx - 2];
            chk(dn::avgpool_backward(pooled.g, act_[src].g, n, h >> (l - 1), w >> (l - 1), pooled.c, st));
        }
    }
    return e;
}

cudaError_t Denoiser::apply_adam(float lr, cudaStream_t st) {
    step_++;
    cudaError_t e = dn::adam(w_, g_, m_, v_, wb_, n_params_, lr, 0.9f, 0.999f, 1e-8f, step_, st);
    return e == cudaSuccess ? refresh_tc_weights(st) : e;
}

cudaError_t Denoiser::output_radiance(float *out, cudaStream_t st) {
    return dn::expm1_out(out_, feat_, out, (size_t)n_ * h_ * w_dim_ * 3, st);
}

cudaError_t Denoiser::denoise(const float *rad, const __half *feat, int n, int h, int w, float *out,
                              cudaStream_t st) {
    GraphKey key;
    key.rad = rad, key.feat = feat, key.out = out, key.n = n, key.h = h, key.w = w;
    key.tensor_cores = tensor_cores_, key.generation = generation_;
    if (graph_ && key == graph_key_) return cudaGraphLaunch(graph_, st);
    // new buffers or sizes: run on the stream (allocating and planning as
    // needed), then record the same launches for the calls that follow
    cudaError_t e = forward(rad, feat, n, h, w, st, out);
    if (e != cudaSuccess) return e;
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    if (!capture_stream_ && (e = cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking)) != cudaSuccess) {
        capture_stream_ = nullptr;
        return e;
    }
    if ((e = cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    cudaError_t le = forward(rad, feat, n, h, w, capture_stream_, out);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(capture_stream_, &g);
    if (le == cudaSuccess && e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
    if (g) cudaGraphDestroy(g);
    if (le != cudaSuccess || e != cudaSuccess) {
        graph_ = nullptr;
        return le != cudaSuccess ? le : e;
    }
    key.generation = generation_;
    graph_key_ = key;
    return cudaSuccess;
}

}  // namespace pray_gpu
