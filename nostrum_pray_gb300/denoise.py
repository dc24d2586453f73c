"""Learned denoising on top of the path tracer: data generation, training and
evaluation of the U-Net (pray_denoiser_* in include/nostrum_pray.h).

Data: seeded procedural rooms (scenes.random_room), each rendered with the
next-event-estimation path tracer at a few samples per pixel (the noisy
input; optionally with its paths cut at fewer bounces), with its first-hit
features, and at many samples per pixel
accumulated in FP64 (the reference). The denoiser divides radiance by the
first-hit albedo (+0.05) before the network and multiplies it back after
(pray_denoise). The network
is trained by its own CUDA forward/backward kernels with an L1 loss in
log(1 + radiance) space and Adam, on random crops.

Evaluation on held-out rooms: relMSE (mean over pixels and channels of
(x - r)^2 / (r^2 + 0.01), FP64 on the GPU) of the noisy input, the denoised
image and plain renders at increasing sample counts; the time each needs to
reach relMSE <= 0.01 (for plain rendering, the render at the smallest sample
count that reaches it, found by bisection); and a fallback: when the predicted error of a denoised
image (half the relMSE between the denoised results of two independent
renders) exceeds the target, the image is re-rendered plainly at the sample
count that reached the target on the training rooms.
"""
from __future__ import annotations

import dataclasses
import time
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import native, scenes


@dataclasses.dataclass
class DenoiseConfig:
    res: int = 512           # evaluation image size
    train_res: int = 512     # training image size
    crop: int = 128          # training crop
    spp_in: int = 4
    spp_ref: int = 1024
    depth: int = 8
    depth_in: int = 0        # path depth of the noisy input (0: depth); references and plain renders use depth
    rr_in: int = -1          # Russian roulette from this depth in the noisy input (-1: rr_depth); unbiased
    rr_depth: int = 3
    train_rooms: int = 96
    eval_rooms: int = 16
    room_grid: int = 16
    steps: int = 1000
    batch: int = 8
    lr: float = 1e-3
    target: float = 0.01
    seed: int = 1000


# (cin, cout, level) of the network's 19 3x3 convolutions in forward order
# (the table of csrc/denoise_net.cpp; level l runs at (h >> l) x (w >> l))
CONVS = [(10, 32, 0), (32, 32, 0), (32, 48, 1), (48, 48, 1), (48, 64, 2), (64, 64, 2), (64, 96, 3), (96, 96, 3),
         (96, 128, 4), (128, 128, 4), (224, 96, 3), (96, 96, 3), (160, 64, 2), (64, 64, 2), (112, 48, 1),
         (48, 48, 1), (80, 32, 0), (32, 32, 0), (32, 3, 0)]


def num_params() -> int:
    return sum(9 * ci * co + co for ci, co, _ in CONVS)


def forward_flops(h: int, w: int, n: int = 1) -> int:
    """Multiply-add FLOPs (2 per MAC) of the convolutions of one forward pass."""
    return n * sum(2 * 9 * ci * co * (h >> l) * (w >> l) for ci, co, l in CONVS)


def forward_bytes(h: int, w: int, n: int = 1) -> int:
    """Algorithmic DRAM bytes of one inference forward pass on the tensor
    cores: every tensor read once and written once (halo re-reads excluded),
    BF16 activations. Input packing reads the radiance (12 B per pixel) and
    the features (14 B) and writes the 16-channel input; each convolution
    reads its input (channels padded to 16) and writes, by the fused
    epilogues: the encoder's second convolutions of levels 0-3 the pooled
    tensor and the skip channels of the concatenation (not their own
    output), the second convolutions of levels 4-1 their output upsampled
    into the next concatenation (4 pixels each), the output convolution the
    log-space and the final radiance (FP32) after reading 3 channels of the
    input and the albedo; the others their output."""
    px0 = n * h * w
    total = px0 * (12 + 14 + 32)
    for i, (ci, co, l) in enumerate(CONVS):
        px = n * (h >> l) * (w >> l)
        rd = 2 * (-(-ci // 16) * 16)
        if i in (1, 3, 5, 7):
            wr = 2 * co // 4 + 2 * co
        elif i in (9, 11, 13, 15):
            wr = 4 * 2 * co
        elif i == len(CONVS) - 1:
            rd += 6 + 6
            wr = 12 + 12
        else:
            wr = 2 * co
        total += px * (rd + wr)
    return total


def denoise_launches(h: int, w: int, n: int = 1, sm_count: int = 152, tensor_cores: bool = True) -> int:
    """Kernels one pray_denoise call launches. On the CUDA cores: input
    packing, 4 poolings, 4 upsample-concatenations, the 19 convolutions, the
    residual add and the output transform. On the tensor cores the poolings,
    concatenations, residual and output transform are stores of the
    convolutions' epilogues: input packing and the 19 convolutions. There a
    convolution with fewer than two 16x8-pixel tiles per SM splits its output
    channels over CTAs, or, with a single 16-channel chunk, its taps, which
    adds a finalize kernel (the rule of tc_conv_plan in
    csrc/denoise_tc.cu); the output convolution split so keeps the residual
    and output kernels."""
    convs, split = 0, False
    for _, co, l in CONVS:
        tiles = n * -(-(w >> l) // 8) * -(-(h >> l) // 16)
        npad = -(-co // 16) * 16
        split = tensor_cores and tiles < 2 * sm_count and npad < 32
        convs += 2 if split else 1
    if not tensor_cores:
        return 1 + 4 + 4 + convs + 2
    return 1 + convs + (2 if split else 0)


def _setup(cfg: DenoiseConfig, res: Optional[int] = None):
    r = res or cfg.res
    return scenes.room_setup(r, r, spp=cfg.spp_in, max_depth=cfg.depth)


def _params(cfg, st, spp, seed, offset=0, depth=None, rr_depth=None):
    return native.pt_params(st, spp=spp, max_depth=cfg.depth if depth is None else depth, seed=seed,
                            mode=native.PT_NEE, rr_depth=cfg.rr_depth if rr_depth is None else rr_depth,
                            scheduler=native.SCHED_AUTO, sample_offset=offset)


def input_params(cfg, st, seed):
    """The noisy input's render: spp_in samples per pixel, paths cut at
    depth_in bounces when it is set (the network then also restores the light
    of the longer paths, which the references and plain renders keep), and
    Russian roulette from depth rr_in when it is set (an unbiased way to
    shorten the input's paths: it trades their length for variance)."""
    return _params(cfg, st, cfg.spp_in, seed, depth=cfg.depth_in or cfg.depth,
                   rr_depth=cfg.rr_in if cfg.rr_in >= 0 else None)


def render_room(cfg: DenoiseConfig, room_seed: int, torch, res: Optional[int] = None):
    """(scene, noisy radiance, features, reference radiance FP64) on the device."""
    st = _setup(cfg, res)
    sc = native.Scene.from_setup(scenes.random_room(room_seed, grid=cfg.room_grid), st)
    h = w = st.width
    rad = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    rgb = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    sc.render_pt(input_params(cfg, st, seed=room_seed * 7 + 1), rgb, rad)
    feat = torch.empty((h, w, 7), dtype=torch.float16, device="cuda")
    sc.render_features(_params(cfg, st, 1, seed=0), feat)
    ref = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
    chunk = 256
    for off in range(0, cfg.spp_ref, chunk):
        sc.accumulate_pt(_params(cfg, st, min(chunk, cfg.spp_ref - off), seed=room_seed * 7 + 2, offset=off), ref)
    ref /= cfg.spp_ref
    return sc, rad, feat, ref


def relmse(img, ref, torch) -> float:
    """FP64 relMSE on the device (pray_relmse)."""
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    native.relmse(img.to(torch.float64).contiguous(), 1.0, ref.contiguous(), 1.0, out)
    return float(out.item())


def make_dataset(cfg: DenoiseConfig, seeds: List[int], torch, res: Optional[int] = None, keep_scenes: bool = True):
    """(scenes, noisy radiance, features, references) stacked over `seeds`;
    with keep_scenes False each scene is closed once rendered (its device
    memory, including the path tracer's scratch, is released) and the scene
    list is empty."""
    rads, feats, refs, scs = [], [], [], []
    for s in seeds:
        sc, rad, feat, ref = render_room(cfg, s, torch, res)
        rads.append(rad)
        feats.append(feat)
        refs.append(ref.to(torch.float32) if not keep_scenes else ref)
        if keep_scenes:
            scs.append(sc)
        else:
            sc.close()
    return scs, torch.stack(rads), torch.stack(feats), torch.stack(refs)


def iter_rooms(cfg: DenoiseConfig, seeds: List[int], torch):
    """(seed, scene, FP64 reference) for each seed, rendered when reached; the
    scene is closed when the caller moves on, so only one room's device memory
    is held at a time."""
    for s in seeds:
        sc, _, _, ref = render_room(cfg, s, torch)
        try:
            yield s, sc, ref
        finally:
            sc.close()


def train(den: native.Denoiser, rad, feat, ref, cfg: DenoiseConfig, torch, log_every: int = 100):
    n = rad.shape[0]
    target = ref.to(torch.float32).contiguous()
    g = torch.Generator(device="cpu").manual_seed(cfg.seed)
    losses = []
    size = rad.shape[1]
    for step in range(cfg.steps):
        idx = torch.randperm(n, generator=g)[:cfg.batch].cuda()
        r, f, t = rad.index_select(0, idx), feat.index_select(0, idx), target.index_select(0, idx)
        if cfg.crop and cfg.crop < size:
            oy, ox = (int(v) for v in torch.randint(0, size - cfg.crop + 1, (2,), generator=g))
            r, f, t = (a[:, oy:oy + cfg.crop, ox:ox + cfg.crop] for a in (r, f, t))
        # random flips keep the data small but varied
        if step % 2:
            r, f, t = r.flip(2), f.flip(2), t.flip(2)
        want = (step % log_every == 0) or step == cfg.steps - 1
        lr = cfg.lr * 0.5 * (1.0 + np.cos(np.pi * step / cfg.steps))  # cosine decay
        loss = den.train_step(r.contiguous(), f.contiguous(), t.contiguous(), lr, want_loss=want)
        if want:
            losses.append((step, loss))
    return losses


def timed(fn, torch) -> float:
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3


def plain_curve(cfg: DenoiseConfig, sc, ref, room_seed: int, torch, spps=(4, 8, 16, 32, 64, 128, 256, 512)):
    """relMSE and render time of plain renders at each sample count (seeds
    independent of the reference's)."""
    st = _setup(cfg)
    out = []
    rad = torch.empty((cfg.res, cfg.res, 3), dtype=torch.float32, device="cuda")
    for spp in spps:
        p = _params(cfg, st, spp, seed=room_seed * 7 + 3)
        sc.render_pt(p, None, rad)  # warm (graph capture)
        t = timed(lambda: sc.render_pt(p, None, rad), torch)
        out.append((spp, relmse(rad, ref, torch), t))
    return out


def smallest_spp(curve, target: float, measure):
    """Smallest sample count whose plain render meets the target, with its
    relMSE and render time: bisection between the last count of the curve
    above the target and the first at or below it; measure(spp) renders and
    returns (relMSE, time). Renders of one seed share their leading samples
    (sample k of a pixel draws from the stream (seed, pixel, k)), so the error
    falls with the count up to noise. None when no count of the curve met the
    target."""
    ok = [i for i, (_, e, _) in enumerate(curve) if e <= target]
    if not ok:
        return None
    i = ok[0]
    lo = curve[i - 1][0] if i > 0 else 0
    hi, e_hi, t_hi = curve[i]
    while hi - lo > 1:
        mid = (lo + hi) // 2
        e, t = measure(mid)
        if e <= target:
            hi, e_hi, t_hi = mid, e, t
        else:
            lo = mid
    return hi, e_hi, t_hi


def plain_to_target(cfg: DenoiseConfig, sc, ref, room_seed: int, torch, curve):
    """smallest_spp for a room, rendering as plain_curve does."""
    st = _setup(cfg)
    rad = torch.empty((cfg.res, cfg.res, 3), dtype=torch.float32, device="cuda")

    def measure(spp):
        p = _params(cfg, st, spp, seed=room_seed * 7 + 3)
        sc.render_pt(p, None, rad)  # warm (graph capture)
        t = timed(lambda: sc.render_pt(p, None, rad), torch)
        return relmse(rad, ref, torch), t

    return smallest_spp(curve, cfg.target, measure)


def denoised_eval(cfg: DenoiseConfig, den, sc, ref, room_seed: int, torch):
    """Denoised relMSE, time (render + features + inference) and predicted
    error from two independent renders."""
    st = _setup(cfg)
    h = w = cfg.res
    rad = torch.empty((1, h, w, 3), dtype=torch.float32, device="cuda")
    rad2 = torch.empty((1, h, w, 3), dtype=torch.float32, device="cuda")
    feat = torch.empty((1, h, w, 7), dtype=torch.float16, device="cuda")
    out = torch.empty((1, h, w, 3), dtype=torch.float32, device="cuda")
    out2 = torch.empty((1, h, w, 3), dtype=torch.float32, device="cuda")
    p = input_params(cfg, st, seed=room_seed * 7 + 5)
    p2 = input_params(cfg, st, seed=room_seed * 7 + 6)
    pf = _params(cfg, st, 1, seed=0)
    side = torch.cuda.Stream()

    def run():
        # the first-hit features do not depend on the path-traced radiance:
        # they render on a second stream beside it
        main = torch.cuda.current_stream()
        side.wait_stream(main)
        sc.render_features(pf, feat[0], stream=side)
        sc.render_pt(p, None, rad[0])
        main.wait_stream(side)
        den.denoise(rad, feat, out)

    def run_with_prediction():
        # the fallback decision: a second independent input, denoised, and
        # half the relMSE between the two outputs read back to the host
        run()
        sc.render_pt(p2, None, rad2[0])
        den.denoise(rad2, feat, out2)
        return 0.5 * relmse(out[0], out2[0].to(torch.float64), torch)

    run()
    t = timed(run, torch)
    t_render = timed(lambda: sc.render_pt(p, None, rad[0]), torch)
    t_infer = timed(lambda: den.denoise(rad, feat, out), torch)
    run_with_prediction()
    t_pred = timed(run_with_prediction, torch)
    pred = run_with_prediction()
    e = relmse(out[0], ref, torch)
    e_noisy = relmse(rad[0], ref, torch)
    return {"relmse_denoised": e, "relmse_noisy": e_noisy, "time_s": t, "render_s": t_render,
            "inference_s": t_infer, "predicted": pred, "time_with_prediction_s": t_pred}


def evaluate(cfg: DenoiseConfig, den, eval_rooms, torch, fallback_spp: int) -> Dict:
    """eval_rooms: a dict seed -> (scene, reference), or an iterable of
    (seed, scene, reference) such as iter_rooms."""
    rows = []
    items = ((s, sc, ref) for s, (sc, ref) in eval_rooms.items()) if isinstance(eval_rooms, dict) else eval_rooms
    for seed, sc, ref in items:
        curve = plain_curve(cfg, sc, ref, seed, torch, spps=(1, 2, 4, 8, 16, 32, 64, 128, 256))
        plain = plain_to_target(cfg, sc, ref, seed, torch, curve)
        d = denoised_eval(cfg, den, sc, ref, seed, torch)
        t_plain = plain[2] if plain else float("nan")
        spp_plain = plain[0] if plain else None
        # fallback: predicted error above target -> plain render at the calibrated spp
        t_final, e_final, used_fallback = d["time_s"], d["relmse_denoised"], False
        if d["predicted"] > cfg.target:
            used_fallback = True
            fb = [(spp, e, t) for spp, e, t in curve if spp == fallback_spp]
            if fb:
                t_final = d["time_s"] + fb[0][2]
                e_final = fb[0][1]
        rows.append({"seed": seed, "spp_plain_to_target": spp_plain, "time_plain_s": t_plain, **d,
                     "fallback": used_fallback, "time_final_s": t_final, "relmse_final": e_final,
                     "time_final_with_prediction_s": t_final - d["time_s"] + d["time_with_prediction_s"]})
    return {"rooms": rows}


def fallback_spp_from(curves: List[List[Tuple[int, float, float]]], target: float) -> int:
    """Smallest sample count whose plain relMSE reached the target on every
    calibration room (the largest tried if none did)."""
    spps = [c[0] for c in curves[0]]
    for i, spp in enumerate(spps):
        if all(c[i][1] <= target for c in curves):
            return spp
    return spps[-1]
