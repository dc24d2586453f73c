"""The allocation-free path-tracing entry point (pray_render_pt_noalloc).

It exists for host applications that must not have this library allocate
device memory while they render: engines that reserve all GPU memory for their
own pool up front, and frame loops that cannot afford cudaMalloc's implicit
synchronisation. Its path pool lives in a fixed static device array instead of
memory allocated on first use. Here it is called through the C ABI twice in a
row (the second call finds the first call's leftovers in the shared array) and
must give the regular wavefront entry point's frame bit for bit: with the same
pool, and with the default pool at a sample count whose paths exceed the
static array (the rounds split differently; the per-pixel sums, added in
sample order, do not change). A call after the first must leave the device's
free memory unchanged. This file is collected last so that a failure here
leaves every other test already run."""
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


def _frame(sc, params, fn):
    h, w = params.height, params.width
    rgb = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    rad = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    fn(params, rgb, rad, cnt)
    torch.cuda.synchronize()
    return rgb.cpu().numpy(), rad.cpu().numpy(), cnt.cpu().numpy()


# (spp, wavefront_paths): the same pool on both paths; the default pool with
# 64 x 48 x 512 = 1,572,864 paths, more than the static array holds
@pytest.mark.parametrize("spp,pool", [(16, 0), (40, 5000), (512, 0)])
def test_no_alloc_matches_wavefront_twice(spp, pool):
    m = scenes.room(grid=8)
    st = scenes.room_setup(64, 48)
    sc = native.Scene.from_setup(m, st)
    p = native.pt_params(st, spp=spp, max_depth=8, seed=21, mode=native.PT_NEE, rr_depth=3,
                         scheduler=native.SCHED_WAVEFRONT, wavefront_paths=pool)
    want_rgb, want_rad, want_cnt = _frame(sc, p, lambda q, a, b, c: sc.render_pt(q, a, b, c))
    for _ in range(2):
        rgb, rad, cnt = _frame(sc, p, lambda q, a, b, c: sc.render_pt_noalloc(q, a, b, c))
        np.testing.assert_array_equal(rad.view(np.uint32), want_rad.view(np.uint32))
        np.testing.assert_array_equal(rgb, want_rgb)
        np.testing.assert_array_equal(cnt, want_cnt)
    sc.close()


def test_no_alloc_leaves_free_memory_unchanged():
    m = scenes.room(grid=8)
    st = scenes.room_setup(96, 64)
    sc = native.Scene.from_setup(m, st)
    p = native.pt_params(st, spp=24, max_depth=8, seed=3, mode=native.PT_NEE, rr_depth=3)
    rgb = torch.empty((st.height, st.width, 3), dtype=torch.uint8, device="cuda")
    rad = torch.empty((st.height, st.width, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    sc.render_pt_noalloc(p, rgb, rad, stream=stream)  # first call on the device: set-up
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    p2 = native.pt_params(st, spp=40, max_depth=8, seed=4, mode=native.PT_NEE, rr_depth=3)
    sc.render_pt_noalloc(p2, rgb, rad, stream=stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == before
    sc.close()


def test_no_alloc_rejects_frames_beyond_its_limit():
    m = scenes.room(grid=4)
    st = scenes.room_setup(1100, 1100)  # 1,210,000 pixels > 1,103,744
    sc = native.Scene.from_setup(m, st)
    p = native.pt_params(st, spp=1, max_depth=2, mode=native.PT_NEE)
    rad = torch.empty((st.height, st.width, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(native.PrayError, match="exceeds the allocation-free path's limit"):
        sc.render_pt_noalloc(p, radiance=rad)
    sc.close()
