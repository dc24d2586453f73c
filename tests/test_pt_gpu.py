"""Parity of the CUDA path tracer with the oracle (GPU): the reference's
Kajiya recursion with PCG32 streams, and the next-event-estimation mode.
Tolerance: 1e-4 relative per pixel on the mean radiance (plus 1e-6 absolute
for near-black pixels); both sides use the same float operation order, so the
match is expected to be exact."""
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


def compare(oracle, mesh, setup, spp, depth, seed, mode, rr=3):
    sc = native.Scene.from_setup(mesh, setup)
    img, rad, cnt = sc.render_pt_host(native.pt_params(setup, spp=spp, max_depth=depth, seed=seed, mode=mode,
                                                       rr_depth=rr))
    orc = oracle.OracleScene.from_setup(mesh, setup)
    oimg, orad, osegs = orc.render_pt(setup, spp=spp, max_depth=depth, seed=seed, mode=mode, rr_depth=rr)
    bad = ~np.isclose(rad, orad, rtol=RTOL, atol=ATOL)
    assert int(bad.sum()) == 0, f"{int(bad.sum())} radiance values differ; max abs {np.abs(rad - orad).max()}"
    assert int(cnt[0]) == setup.width * setup.height * spp
    assert int(cnt[1]) == osegs
    assert (np.abs(img.astype(int) - oimg.astype(int)) <= 1).all()
    return rad


@pytest.mark.parametrize("depth", [1, 3, 8])
def test_kajiya_room(oracle, depth):
    m = scenes.room(grid=6)
    st = scenes.room_setup(64, 48)
    compare(oracle, m, st, spp=8, depth=depth, seed=3, mode=native.PT_KAJIYA)


def test_nee_room(oracle):
    m = scenes.room(grid=6)
    st = scenes.room_setup(64, 48)
    compare(oracle, m, st, spp=8, depth=8, seed=4, mode=native.PT_NEE, rr=3)


def test_kajiya_background_and_median_tree(oracle):
    m = scenes.soup(2_000, 1)
    m.emit[::7] = 1
    st = scenes.soup_setup(40, 40)
    st.background = (0.3, 0.2, 0.1)
    compare(oracle, m, st, spp=4, depth=4, seed=9, mode=native.PT_KAJIYA)


def test_seeds_differ_and_repeat(oracle):
    m = scenes.room(grid=4)
    st = scenes.room_setup(32, 32)
    sc = native.Scene.from_setup(m, st)
    a = sc.render_pt_host(native.pt_params(st, spp=4, max_depth=3, seed=1))[1]
    b = sc.render_pt_host(native.pt_params(st, spp=4, max_depth=3, seed=1))[1]
    c = sc.render_pt_host(native.pt_params(st, spp=4, max_depth=3, seed=2))[1]
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
