"""The allocation-free path-tracing entry point (pray_render_pt_noalloc).

It exists for host applications that must not have this library allocate
device memory while they render: engines that reserve all GPU memory for their
own pool up front, and frame loops that cannot afford cudaMalloc's implicit
synchronisation. Its path pool lives in a fixed static device array instead of
memory allocated on first use. Here it is called through the C ABI twice in a
row (the second call finds the first call's leftovers in the shared array)
and must give the same frame as the regular wavefront entry point, within the
path-tracing tolerance of the other tests. This file is collected last so that
a failure here leaves every other test already run."""
import numpy as np
import pytest

from nostrum_pray_gb300 import native, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL, ATOL = 1e-4, 1e-6


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


def test_no_alloc_matches_wavefront_twice():
    m = scenes.room(grid=8)
    st = scenes.room_setup(64, 48)
    sc = native.Scene.from_setup(m, st)
    for spp, pool in ((16, 0), (40, 5000)):
        p = native.pt_params(st, spp=spp, max_depth=8, seed=21, mode=native.PT_NEE, rr_depth=3,
                             scheduler=native.SCHED_WAVEFRONT, wavefront_paths=pool)
        want_rgb, want_rad, want_cnt = _frame(sc, p, lambda q, a, b, c: sc.render_pt(q, a, b, c))
        for _ in range(2):
            rgb, rad, cnt = _frame(sc, p, lambda q, a, b, c: sc.render_pt_noalloc(q, a, b, c))
            assert np.allclose(rad, want_rad, rtol=RTOL, atol=ATOL)
            assert (np.abs(rgb.astype(int) - want_rgb.astype(int)) <= 1).all()
            np.testing.assert_array_equal(cnt, want_cnt)


def test_no_alloc_rejects_frames_beyond_its_limit():
    m = scenes.room(grid=4)
    st = scenes.room_setup(1100, 1100)  # 1,210,000 pixels > 1,103,744
    sc = native.Scene.from_setup(m, st)
    p = native.pt_params(st, spp=1, max_depth=2, mode=native.PT_NEE)
    rad = torch.empty((st.height, st.width, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(native.PrayError, match="exceeds the allocation-free path's limit"):
        sc.render_pt_noalloc(p, radiance=rad)
