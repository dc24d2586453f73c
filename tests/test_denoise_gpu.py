"""Denoiser kernels against the FP64 oracle (oracle/denoise_oracle.cpp):
network output, L1 loss and every parameter gradient, on random inputs;
training on a fixed batch must reduce the loss; first-hit features must equal
the oracle's hit data exactly."""
import numpy as np
import pytest

from nostrum_pray_gb300 import native, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    native.lib()


CONVS = [(10, 32), (32, 32), (32, 48), (48, 48), (48, 64), (64, 64), (64, 96), (96, 96), (96, 128), (128, 128),
         (224, 96), (96, 96), (160, 64), (64, 64), (112, 48), (48, 48), (80, 32), (32, 32), (32, 3)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def random_batch(seed, n, h, w):
    rng = np.random.default_rng(seed)
    rad = (rng.random((n, h, w, 3)) * 2).astype(np.float32)
    feat = rng.random((n, h, w, 7)).astype(np.float16)
    tgt = rng.random((n, h, w, 3)).astype(np.float32)
    return rad, feat, tgt


# resolution level of each convolution (size >> level)
LEVELS = [0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0]


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_gradients_match_fp64_oracle(oracle, tensor_cores):
    """Loss, output and every parameter's gradient against the FP64 oracle
    (which rounds stored activations to BF16 at the same points), with the
    forward pass on the tensor cores and on the CUDA cores. Tolerances: the
    gradient vector as a whole within 2 %; each convolution's weights within
    3 % at levels 0-2 and 8 % at levels 3-4 (8 x 8 and 4 x 4 pixels here),
    where a BF16 rounding flip of one stored activation (or of a ReLU sign)
    weighs more: measured 2-5 % there on both paths."""
    den = native.Denoiser(seed=5)
    den.set_tensor_cores(tensor_cores)
    params = den.get_params()
    rad, feat, tgt = random_batch(1, 2, 64, 64)
    t = lambda a: torch.from_numpy(a).cuda()
    loss, g = den.gradients(t(rad), t(feat), t(tgt))
    out = torch.empty((2, 64, 64, 3), dtype=torch.float32, device="cuda")
    den.denoise(t(rad), t(feat), out)
    torch.cuda.synchronize()
    oloss, oout, og = oracle.unet(params, rad, feat, tgt)
    assert abs(loss - oloss) <= 2e-3 * abs(oloss)
    # the output is re-modulated by the albedo; the oracle returns the network output in log space
    dm = (np.maximum(feat[..., 0:3].astype(np.float32), 0) + np.float32(0.05)).astype(np.float64)
    assert rel(np.log1p(out.cpu().numpy().astype(np.float64) / dm), oout) < 5e-3
    assert rel(g, og) < 2e-2
    off = 0
    for (cin, cout), level in zip(CONVS, LEVELS):
        nw = cout * 9 * cin
        tol = 3e-2 if level <= 2 else 8e-2
        assert rel(g[off:off + nw], og[off:off + nw]) < tol, (cin, cout)
        assert rel(g[off + nw:off + nw + cout], og[off + nw:off + nw + cout]) < tol, (cin, cout, "bias")
        off += nw + cout
    assert off == den.num_params


def test_gradients_deterministic():
    """Loss and every gradient are the same bits on every call (fixed-order
    reductions throughout, no floating-point atomics)."""
    den = native.Denoiser(seed=6)
    rad, feat, tgt = random_batch(2, 2, 80, 48)
    t = lambda a: torch.from_numpy(a).cuda()
    runs = [den.gradients(t(rad), t(feat), t(tgt)) for _ in range(3)]
    for loss, g in runs[1:]:
        assert loss == runs[0][0]
        assert np.array_equal(g.view(np.uint32), runs[0][1].view(np.uint32))


def test_training_reduces_loss():
    den = native.Denoiser(seed=2)
    rad, feat, tgt = random_batch(3, 4, 32, 32)
    tgt = np.clip(rad * 0.5 + 0.1, 0, None).astype(np.float32)  # learnable map
    t = lambda a: torch.from_numpy(a).cuda()
    rad_t, feat_t, tgt_t = t(rad), t(feat), t(tgt)
    first = den.train_step(rad_t, feat_t, tgt_t, 1e-3, want_loss=True)
    for _ in range(150):
        den.train_step(rad_t, feat_t, tgt_t, 1e-3)
    last = den.train_step(rad_t, feat_t, tgt_t, 1e-3, want_loss=True)
    assert last < 0.5 * first, (first, last)


def test_features_match_oracle_hits(oracle):
    m = scenes.room(grid=6)
    st = scenes.room_setup(48, 32)
    sc = native.Scene.from_setup(m, st)
    feat = torch.empty((32, 48, 7), dtype=torch.float16, device="cuda")
    sc.render_features(native.pt_params(st, spp=1, max_depth=1), feat)
    torch.cuda.synchronize()
    got = feat.cpu().numpy().reshape(-1, 7)
    orc = oracle.OracleScene.from_setup(m, st)
    rays = oracle.primary_rays(st.width, st.height, st.fov, st.cam_pos, st.cam_look)
    ids, ts = orc.trace(rays, st.det_eps)
    pre = orc.precompute()
    want = np.zeros((ids.size, 7), np.float32)
    hit = ids >= 0
    want[hit, 0:3] = m.colors[ids[hit]]
    want[hit, 3:6] = pre[ids[hit], 15:18]
    want[hit, 6] = ts[hit]
    np.testing.assert_array_equal(got, want.astype(np.float16))


@pytest.mark.parametrize("shape", [(1, 16, 16), (2, 48, 32), (2, 80, 48), (2, 256, 256), (1, 512, 512)])
def test_tensor_core_forward_matches_cuda_cores(shape):
    """The tcgen05 implicit-GEMM convolutions give the CUDA-core result (same
    BF16 operands, FP32 accumulation; only the summation order differs).
    Shapes cover partial tiles (80 x 48 and 16 x 16 down to 5 x 3 and 1 x 1
    at the deepest level), two images, all three tap splits (1 from 304
    tiles up, 3 from 102, 9 below) and the persistent pipelined kernel (the
    unsplit levels of 256^2 and 512^2 frames). Compared: the network's
    correction (output minus input in log space), which every convolution
    feeds."""
    n, h, w = shape
    den = native.Denoiser(seed=9)
    rad, feat, _ = random_batch(4, n, h, w)
    t = lambda a: torch.from_numpy(a).cuda()
    outs = []
    for tc in (False, True):
        den.set_tensor_cores(tc)
        out = torch.empty((n, h, w, 3), dtype=torch.float32, device="cuda")
        den.denoise(t(rad), t(feat), out)
        den.check()
        outs.append(out.cpu().numpy())
    base = np.log1p(rad.astype(np.float64))
    corr = [np.log1p(o.astype(np.float64)) - base for o in outs]
    assert rel(np.log1p(outs[1].astype(np.float64)), np.log1p(outs[0].astype(np.float64))) < 5e-3
    assert rel(corr[1], corr[0]) < 2e-2


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_denoise_graph_replays(tensor_cores):
    """pray_denoise records its launches in a CUDA graph on the first call
    with a set of buffers and replays the graph after. Replays equal the first
    (stream-launched) call bit for bit, read new contents of the same buffers
    and new weights (training steps at the same size and at another size, the
    latter reallocating the activations), and new buffers record a new graph;
    each result equals a fresh denoiser's first call with the same weights."""
    den = native.Denoiser(seed=11)
    den.set_tensor_cores(tensor_cores)
    n, h, w = 1, 64, 48
    rad, feat, tgt = random_batch(6, n, h, w)
    t = lambda a: torch.from_numpy(a).cuda()
    rad_t, feat_t, tgt_t = t(rad), t(feat), t(tgt)
    out = torch.empty((n, h, w, 3), dtype=torch.float32, device="cuda")

    def run(d, r, o):
        d.denoise(r, feat_t, o)
        d.check()
        return o.cpu().numpy().copy()

    def fresh(r):
        f = native.Denoiser(seed=0)
        f.set_tensor_cores(tensor_cores)
        f.set_params(den.get_params())
        return run(f, r, torch.empty_like(out))

    first = run(den, rad_t, out)
    np.testing.assert_array_equal(run(den, rad_t, out), first)
    rad_t.copy_(t(random_batch(7, n, h, w)[0]))
    np.testing.assert_array_equal(run(den, rad_t, out), fresh(rad_t))
    den.train_step(rad_t, feat_t, tgt_t, 1e-3)
    np.testing.assert_array_equal(run(den, rad_t, out), fresh(rad_t))
    r2, f2, t2 = random_batch(8, 2, 32, 32)
    den.train_step(t(r2), t(f2), t(t2), 1e-3)
    np.testing.assert_array_equal(run(den, rad_t, out), fresh(rad_t))
    out2 = torch.empty_like(out)
    np.testing.assert_array_equal(run(den, rad_t, out2), fresh(rad_t))
    assert not np.array_equal(first, out2.cpu().numpy())


def test_trained_denoiser_beats_its_input():
    """What the learned part adds: trained on a few rooms rendered by the path
    tracer (4 spp inputs, 512-spp FP64 references), the denoiser lowers the
    relMSE of 4-spp renders of held-out rooms below that of the renders
    themselves (the method without it)."""
    from nostrum_pray_gb300 import denoise as D
    cfg = D.DenoiseConfig(res=128, train_res=128, crop=64, spp_ref=512, steps=400, batch=8, train_rooms=12,
                          eval_rooms=2, room_grid=8)
    _, rad, feat, ref = D.make_dataset(cfg, list(range(500, 500 + cfg.train_rooms)), torch, cfg.train_res)
    den = native.Denoiser(seed=3)
    D.train(den, rad, feat, ref, cfg, torch)
    scs, _, _, refs = D.make_dataset(cfg, [9000, 9001], torch)
    gains = []
    for i, sc in enumerate(scs):
        r = D.denoised_eval(cfg, den, sc, refs[i], 9000 + i, torch)
        gains.append(r["relmse_denoised"] / r["relmse_noisy"])
    den.check()
    assert max(gains) < 0.9, gains
