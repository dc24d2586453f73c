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


def test_nee_ragged_frame(oracle):
    """A frame whose size is no multiple of the 8 x 4 warp tile: the per-pixel
    kernel's lanes take pixels from a frame counter, including the slots of
    ragged tiles outside the image."""
    m = scenes.room(grid=5)
    st = scenes.room_setup(37, 23)
    compare(oracle, m, st, spp=3, depth=6, seed=11, mode=native.PT_NEE, rr=2)


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


def test_wavefront_matches_oracle_and_pixel_scheduler(oracle):
    """The wavefront scheduler (path pool, compacted queues, one CUDA graph
    per frame) gives the same radiance as the per-pixel kernel and the
    oracle, with one round and with the samples split over many rounds
    (a pool of 1,000 paths for 384 pixels: 2 samples per pixel per round)."""
    m = scenes.room(grid=6)
    st = scenes.room_setup(24, 16)
    sc = native.Scene.from_setup(m, st)
    got = {}
    for spp, pool in ((8, 0), (96, 0), (96, 1000), (7, 1000)):
        pw = native.pt_params(st, spp=spp, max_depth=8, seed=12, mode=native.PT_NEE, rr_depth=3,
                              scheduler=native.SCHED_WAVEFRONT, wavefront_paths=pool)
        pp = native.pt_params(st, spp=spp, max_depth=8, seed=12, mode=native.PT_NEE, rr_depth=3,
                              scheduler=native.SCHED_PIXEL)
        img_w, rad_w, cnt_w = sc.render_pt_host(pw)
        img_p, rad_p, cnt_p = sc.render_pt_host(pp)
        np.testing.assert_array_equal(rad_w.view(np.uint32), rad_p.view(np.uint32))
        np.testing.assert_array_equal(img_w, img_p)
        assert int(cnt_w[0]) == int(cnt_p[0]) and int(cnt_w[1]) == int(cnt_p[1])
        # repeat: the cached graph replays to the same frame
        np.testing.assert_array_equal(sc.render_pt_host(pw)[1], rad_w)
        got[(spp, pool)] = rad_w
    _, orad, _ = oracle.OracleScene.from_setup(m, st).render_pt(st, spp=96, max_depth=8, seed=12,
                                                                mode=native.PT_NEE, rr_depth=3)
    assert np.allclose(got[(96, 1000)], orad, rtol=RTOL, atol=ATOL)
    np.testing.assert_array_equal(got[(96, 1000)], got[(96, 0)])


def test_wavefront_rejects_kajiya_mode():
    m = scenes.room(grid=4)
    st = scenes.room_setup(8, 8)
    sc = native.Scene.from_setup(m, st)
    with pytest.raises(native.PrayError):
        sc.render_pt_host(native.pt_params(st, spp=1, max_depth=2, mode=native.PT_KAJIYA,
                                           scheduler=native.SCHED_WAVEFRONT))


@pytest.mark.parametrize("scheduler", [0, 1])
def test_fp64_accumulation_in_chunks(oracle, scheduler):
    """FP64 sums over consecutive sample ranges equal the oracle's sequential
    FP64 sums (exactly), whatever the chunking."""
    m = scenes.room(grid=6)
    st = scenes.room_setup(20, 12)
    sc = native.Scene.from_setup(m, st)
    acc = torch.zeros((st.height, st.width, 3), dtype=torch.float64, device="cuda")
    for off, n in ((0, 5), (5, 11), (16, 16)):
        sc.accumulate_pt(native.pt_params(st, spp=n, max_depth=6, seed=2, mode=native.PT_NEE, rr_depth=3,
                                          scheduler=scheduler, sample_offset=off), acc)
    torch.cuda.synchronize()
    want = np.zeros((st.height, st.width, 3), np.float64)
    oracle.OracleScene.from_setup(m, st).render_pt(st, spp=32, max_depth=6, seed=2, mode=native.PT_NEE,
                                                    rr_depth=3, sum64=want)
    np.testing.assert_array_equal(acc.cpu().numpy(), want)


@pytest.mark.parametrize("n", [1, 5, 30_001, 512 * 512 * 3])
def test_relmse_reduction(n):
    """FP64 relMSE over one cluster of CTAs: fewer values than threads, a
    ragged size and a 512^2 frame; the same bits on every call."""
    rng = np.random.default_rng(n)
    a = rng.random(n) * 2
    r = rng.random(n)
    want = np.mean((a * 0.5 - r * 2.0) ** 2 / ((r * 2.0) ** 2 + 0.01))
    ta, tr = torch.from_numpy(a).cuda(), torch.from_numpy(r).cuda()
    got = []
    for _ in range(3):
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        native.relmse(ta, 0.5, tr, 2.0, out)
        torch.cuda.synchronize()
        got.append(out.item())
    assert abs(got[0] - want) <= 1e-12 * max(1.0, want)
    assert got[1] == got[0] and got[2] == got[0]


@pytest.mark.parametrize("depth,n", [(0, 4), (1, 8), (2, 5)])
def test_diffuse_branching_room(oracle, depth, n):
    """The reference's branching mode (evaluatePathRecursiveDiffuse): n bounce
    rays at every hit above max_depth, one estimate per pixel."""
    m = scenes.room(grid=6)
    st = scenes.room_setup(40, 32)
    sc = native.Scene.from_setup(m, st)
    orc = oracle.OracleScene.from_setup(m, st)
    for off in (0, 3):
        p = native.pt_params(st, spp=n, max_depth=depth, seed=7, mode=native.PT_DIFFUSE, sample_offset=off)
        img, rad, cnt = sc.render_pt_host(p)
        oimg, orad, osegs = orc.render_pt(st, spp=n, max_depth=depth, seed=7, mode=native.PT_DIFFUSE,
                                          sample_offset=off)
        bad = ~np.isclose(rad, orad, rtol=RTOL, atol=ATOL)
        assert int(bad.sum()) == 0, f"{int(bad.sum())} radiance values differ"
        assert int(cnt[0]) == st.width * st.height
        assert int(cnt[1]) == osegs
        np.testing.assert_array_equal(img, oimg)
    # rays per pixel can reach 1 + n + ... + n^depth
    assert osegs <= st.width * st.height * sum(n ** k for k in range(depth + 1))


def test_diffuse_mode_limits():
    m = scenes.room(grid=3)
    st = scenes.room_setup(16, 16)
    sc = native.Scene.from_setup(m, st)
    with pytest.raises(native.PrayError):
        sc.render_pt_host(native.pt_params(st, spp=2, max_depth=9, mode=native.PT_DIFFUSE))
    with pytest.raises(native.PrayError):
        sc.render_pt_host(native.pt_params(st, spp=2, max_depth=1, mode=native.PT_DIFFUSE,
                                           scheduler=native.SCHED_WAVEFRONT))
    acc = torch.zeros((16, 16, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(native.PrayError):
        sc.accumulate_pt(native.pt_params(st, spp=2, max_depth=1, mode=native.PT_DIFFUSE), acc)
    rgb = torch.empty((16, 16, 3), dtype=torch.uint8, device="cuda")
    with pytest.raises(native.PrayError):
        native.Batch([sc], [native.pt_params(st, spp=2, max_depth=1, mode=native.PT_DIFFUSE)], [(rgb, None)])


def test_auto_scheduler_gives_the_same_frames():
    """PRAY_SCHED_AUTO (per-pixel kernel below 2^19 paths, wavefront from
    there on) returns the frames of the fixed schedulers, bit for bit."""
    m = scenes.room(grid=6)
    for (w, h, spp) in ((64, 64, 4), (128, 128, 32)):
        st = scenes.room_setup(w, h)
        sc = native.Scene.from_setup(m, st)
        got = {}
        for sched in (native.SCHED_PIXEL, native.SCHED_WAVEFRONT, native.SCHED_AUTO):
            p = native.pt_params(st, spp=spp, max_depth=8, seed=21, mode=native.PT_NEE, rr_depth=3, scheduler=sched)
            got[sched] = sc.render_pt_host(p)[1]
        np.testing.assert_array_equal(got[native.SCHED_AUTO], got[native.SCHED_PIXEL])
        np.testing.assert_array_equal(got[native.SCHED_AUTO], got[native.SCHED_WAVEFRONT])
    # Kajiya frames always run per pixel under AUTO
    st = scenes.room_setup(128, 128)
    sc = native.Scene.from_setup(m, st)
    a = sc.render_pt_host(native.pt_params(st, spp=32, max_depth=4, seed=2, scheduler=native.SCHED_AUTO))[1]
    b = sc.render_pt_host(native.pt_params(st, spp=32, max_depth=4, seed=2, scheduler=native.SCHED_PIXEL))[1]
    np.testing.assert_array_equal(a, b)


@pytest.mark.slow
def test_full_size_room_schedulers_and_chunks_agree():
    """At the benchmark's size (the 101k-triangle room at 1024 x 1024, NEE +
    RR, depth 8), properties that hold at any size: the wavefront and the
    per-pixel schedulers give the same radiance bit for bit, and FP64 sums
    accumulated over two sample ranges equal one call over both."""
    m = scenes.room()
    st = scenes.room_setup(1024, 1024)
    sc = native.Scene.from_setup(m, st)
    rads = []
    for sched in (native.SCHED_PIXEL, native.SCHED_WAVEFRONT):
        rad = torch.empty((1024, 1024, 3), dtype=torch.float32, device="cuda")
        sc.render_pt(native.pt_params(st, spp=8, max_depth=8, seed=3, mode=native.PT_NEE, rr_depth=3,
                                      scheduler=sched), None, rad)
        rads.append(rad.cpu().numpy())
    np.testing.assert_array_equal(rads[0].view(np.uint32), rads[1].view(np.uint32))
    one = torch.zeros((1024, 1024, 3), dtype=torch.float64, device="cuda")
    two = torch.zeros_like(one)
    p = lambda spp, off: native.pt_params(st, spp=spp, max_depth=8, seed=3, mode=native.PT_NEE, rr_depth=3,
                                          scheduler=native.SCHED_WAVEFRONT, sample_offset=off)
    sc.accumulate_pt(p(8, 0), one)
    sc.accumulate_pt(p(3, 0), two)
    sc.accumulate_pt(p(5, 3), two)
    torch.cuda.synchronize()
    assert torch.equal(one, two)
    # the mean of the FP64 sums is the radiance of the 8-sample frame up to FP32 rounding
    np.testing.assert_allclose((one / 8).cpu().numpy(), rads[0], rtol=1e-5, atol=1e-6)
