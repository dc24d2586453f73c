"""Batched path tracing: several scenes of different size and resolution in
one persistent launch must give each scene exactly the frame it gets alone
(same per-pixel code and random streams), for every launch shape the
autotuner may pick."""
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


def small_batch(modes=(native.PT_KAJIYA,)):
    items = scenes.batch_workload(n=5, seed=3, median=3_000, lo=500, hi=20_000, spp=2, depth=4,
                                  resolutions=(24, 40, 56))
    scs, params, outs = [], [], []
    for i, (mesh, st) in enumerate(items):
        scs.append(native.Scene.from_setup(mesh, st))
        params.append(native.pt_params(st, seed=100 + i, mode=modes[i % len(modes)]))
        outs.append((torch.zeros((st.height, st.width, 3), dtype=torch.uint8, device="cuda"),
                     torch.zeros((st.height, st.width, 3), dtype=torch.float32, device="cuda")))
    return items, scs, params, outs


def alone(sc, p):
    img, rad, _ = sc.render_pt_host(p)
    return img, rad


@pytest.mark.parametrize("modes", [(native.PT_KAJIYA,), (native.PT_KAJIYA, native.PT_NEE)],
                         ids=["kajiya", "mixed"])
def test_batch_equals_single_scene_frames(modes):
    """All-Kajiya batches run the per-lane state machine, batches with
    next-event scenes the bounce-by-bounce loop; both equal single frames."""
    items, scs, params, outs = small_batch(modes)
    b = native.Batch(scs, params, outs)
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    want = [alone(sc, p) for sc, p in zip(scs, params)]
    for cfg in (native.BatchConfig(8, 4, 128, 0, 64), native.BatchConfig(32, 1, 64, 2, 64),
                native.BatchConfig(4, 8, 256, 0, 64)):
        b.set_config(cfg)
        for o in outs:
            o[0].zero_(), o[1].zero_()
        cnt.zero_()
        b.render(cnt)
        torch.cuda.synchronize()
        for (img, rad), (o8, of) in zip(want, outs):
            np.testing.assert_array_equal(of.cpu().numpy().view(np.uint32), rad.view(np.uint32))
            np.testing.assert_array_equal(o8.cpu().numpy(), img)
        assert int(cnt[0]) == sum(st.width * st.height * 2 for _, st in items)


def test_autotuner_picks_a_valid_shape_and_keeps_results():
    items, scs, params, outs = small_batch()
    b = native.Batch(scs, params, outs)
    cfg, ms = b.tune()
    assert cfg.tile_w * cfg.tile_h == 32 and ms > 0
    b.render()
    torch.cuda.synchronize()
    for sc, p, (o8, of) in zip(scs, params, outs):
        img, rad = alone(sc, p)
        np.testing.assert_array_equal(of.cpu().numpy(), rad)


@pytest.mark.slow
def test_full_batch_workload_equals_single_scene_frames():
    """The benchmark's 64-scene batch (34.8M pixels; here at 1 spp to keep it
    short): every scene's frame from the one persistent launch equals that
    scene rendered alone, bit for bit."""
    items = scenes.batch_workload(64, seed=0, spp=1)
    scs, params, outs = [], [], []
    for i, (mesh, st) in enumerate(items):
        scs.append(native.Scene.from_setup(mesh, st))
        params.append(native.pt_params(st, seed=i, mode=native.PT_KAJIYA))
        outs.append((torch.empty((st.height, st.width, 3), dtype=torch.uint8, device="cuda"),
                     torch.empty((st.height, st.width, 3), dtype=torch.float32, device="cuda")))
    b = native.Batch(scs, params, outs)
    b.render()
    torch.cuda.synchronize()
    for sc, p, (o8, of) in zip(scs, params, outs):
        img, rad = alone(sc, p)
        np.testing.assert_array_equal(of.cpu().numpy().view(np.uint32), rad.view(np.uint32))
        np.testing.assert_array_equal(o8.cpu().numpy(), img)
