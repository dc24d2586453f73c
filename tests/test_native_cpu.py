"""Host-side checks of the native library that need no GPU: the C ABI loads
and exports every symbol the public headers declare, the host tree builders
reproduce the reference's trees (digests from tests/golden/), the camera
constants match the oracle bit for bit, the shared sampling code is accurate,
and bad arguments come back as errors."""
import os
import re

import numpy as np
import pytest

from golden_util import dump_hash
from nostrum_pray_gb300 import native, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nostrum_pray_gb300 import build
    build.build()


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(pray_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    # PRAY_HD helpers of the sampling header are inline, not exported
    return {s for s in syms if not s.startswith(("pray_pcg32", "pray_uniform", "pray_sincos", "pray_normalize",
                                                  "pray_sample_hemisphere"))}


def test_library_exports_every_declared_symbol():
    L = native.lib()
    syms = declared_symbols()
    assert "pray_render_rt" in syms and "pray_scene_create" in syms
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing
    assert set(native.EXPORTED) == syms
    assert L.pray_api_version() == 1


def test_cli_binary_built():
    assert os.access(native.CLI_PATH, os.X_OK)


@pytest.mark.parametrize("key,setup_fn", [
    ("soup_s0", lambda: scenes.soup_setup()),
    ("soup_s1", lambda: scenes.soup_setup()),
])
def test_host_median_tree_matches_reference(golden, key, setup_fn):
    hashes, _ = golden
    seed = int(key[-1])
    t = native.HostTree(scenes.soup(10_000, seed), native.tree_options(setup_fn()))
    assert [int(x) for x in t.tree_stats()] == hashes[key]["stats"]
    assert dump_hash(t.tree_dump()) == hashes[key]["tree"]


def test_host_sah_tree_matches_reference(golden):
    hashes, small = golden
    st = scenes.soup_setup()
    st.tree, st.leaf_size, st.max_depth = "sah", 32, 20
    for seed in (0, 1, 2):
        t = native.HostTree(scenes.soup(10_000, seed), native.tree_options(st))
        assert dump_hash(t.tree_dump()) == hashes[f"soup_s{seed}_sah"]["tree"]
    t = native.HostTree(scenes.icosphere(5), native.tree_options(scenes.icosphere_setup()))
    d = t.tree_dump()
    for k in ("boxes", "split", "info", "refs"):
        np.testing.assert_array_equal(d[k], small[f"ico5_eps0_tree_{k}"])


@pytest.mark.slow
def test_host_sah_tree_full_icosphere(golden):
    hashes, _ = golden
    t = native.HostTree(scenes.icosphere(8), native.tree_options(scenes.icosphere_setup()))
    assert [int(x) for x in t.tree_stats()] == hashes["ico8_eps0"]["stats"]
    assert dump_hash(t.tree_dump()) == hashes["ico8_eps0"]["tree"]


@pytest.mark.parametrize("threads", [1, 3, 16])
def test_host_sah_tree_independent_of_threads(golden, threads):
    """The parallel builder (subtrees and the root's event sort split over
    threads) gives the reference's tree for any thread count."""
    hashes, _ = golden
    o = native.tree_options(scenes.icosphere_setup())
    o.build_threads = threads
    t = native.HostTree(scenes.icosphere(8), o)
    assert [int(x) for x in t.tree_stats()] == hashes["ico8_eps0"]["stats"]
    assert dump_hash(t.tree_dump()) == hashes["ico8_eps0"]["tree"]


def test_host_precompute_matches_reference(golden):
    _, small = golden
    t = native.HostTree(scenes.soup(10_000, 0), native.tree_options(scenes.soup_setup()))
    np.testing.assert_array_equal(t.precompute()[:256].view(np.uint32), small["soup_s0_precompute"].view(np.uint32))


@pytest.mark.parametrize("name", ["cube", "head_fov30", "plant"])
def test_host_tree_examples(golden, name):
    hashes, small = golden
    m = scenes.Mesh(small[f"ex_{name}_verts"], small[f"ex_{name}_colors"], small[f"ex_{name}_emit"])
    t = native.HostTree(m, native.tree_options(tree=native.TREE_MEDIAN))
    assert dump_hash(t.tree_dump()) == hashes[f"ex_{name}"]["tree"]


def test_empty_tree():
    m = scenes.Mesh(np.zeros((0, 9), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.uint8))
    t = native.HostTree(m, native.tree_options())
    assert [int(x) for x in t.tree_stats()] == [1, 0, 0, 0, 0]


@pytest.mark.parametrize("cam", [
    (1920, 1080, 45, (0, 0, -3), (0, 0, 1)),
    (512, 512, 60, (0.5, 0.5, -1.5), (0, 0, 1)),
    (400, 400, 30, (1.5, 5.0, 6.0), (-0.1, -0.5, -1.0)),
    (800, 600, 130, (0.0, 1.0, 0.9), (0.0, 0.0, -1.0)),
    (33, 17, 90, (2.0, 3.0, 3.0), (0.0, 0.0, 1.0)),
])
def test_camera_matches_oracle(oracle, cam):
    a = native.camera(*cam)
    b = oracle.camera(*cam)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


def test_sincos_turns_accuracy(oracle):
    u = (np.arange(0, 1 << 24, 13, dtype=np.float64) / (1 << 24))
    s, c = oracle.sincos_turns(u.astype(np.float32))
    assert np.abs(s - np.sin(2 * np.pi * u)).max() < 3e-7
    assert np.abs(c - np.cos(2 * np.pi * u)).max() < 3e-7


def test_hemisphere_directions(oracle):
    rng = np.random.default_rng(1)
    n = rng.normal(size=(20000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    u = rng.random((20000, 2)).astype(np.float32)
    d = oracle.sample_hemisphere(n, u)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    cosang = (d * n).sum(1)
    assert (cosang >= -1e-6).all()
    # cosine-weighted: E[cos] = 2/3
    assert abs(cosang.mean() - 2 / 3) < 0.01


def test_bad_tree_options_rejected():
    m = scenes.soup(50, 0)
    for kw in ({"max_depth": 31}, {"leaf_size": 0}, {"tree": 7}, {"sah_intersection_cost": 0.0}):
        with pytest.raises(native.PrayError):
            native.HostTree(m, native.tree_options(**kw))


@pytest.mark.parametrize("refine", [0, 1, 4, 16])
def test_device_layout_valid(refine):
    for mesh, st in ((scenes.soup(10_000, 0), scenes.soup_setup()), (scenes.icosphere(5), scenes.icosphere_setup()),
                     (scenes.room(grid=8), scenes.room_setup())):
        t = native.HostTree(mesh, native.tree_options(st))
        nodes, refs, refined, added = (int(x) for x in t.device_layout(refine))
        st_ = t.tree_stats()
        assert refs == int(st_[4])  # every reference kept exactly once
        if refine == 0:
            assert refined == 0 and added == 0 and nodes == int(st_[0]) + 1
        else:
            assert nodes == int(st_[0]) + 1 + added


def test_denoiser_table_matches_oracle(oracle):
    """The conv table used for FLOP counts has the oracle network's parameter
    count; 47.6 GFLOP per 512x512 forward."""
    from nostrum_pray_gb300 import denoise
    assert denoise.num_params() == int(oracle.lib().orc_unet_num_params()) == 1_016_419
    assert denoise.forward_flops(512, 512) == 47_563_407_360


def test_denoiser_pass_accounting():
    """Launches and algorithmic DRAM bytes of one inference pass. On the
    tensor cores a 512^2 frame is input packing plus the 19 convolutions
    (pooling, concatenation, residual and output transform are epilogue
    stores); a 128^2 frame's output convolution splits its taps (a finalize
    kernel) and so keeps the residual and output kernels; the CUDA-core pass
    launches every kernel. Bytes: every tensor read and written once, 311.3
    MB per 512^2 frame (157.5 MB read, 153.8 MB written), linear in frames."""
    from nostrum_pray_gb300 import denoise
    assert denoise.denoise_launches(512, 512) == 20
    assert denoise.denoise_launches(512, 512, tensor_cores=False) == 30
    assert denoise.denoise_launches(128, 128) == 1 + 19 + 1 + 2
    assert denoise.forward_bytes(512, 512) == 311_296_000
    assert denoise.forward_bytes(512, 512, 8) == 8 * 311_296_000


def test_denoiser_fallback_sample_count():
    """The fallback render's sample count: the smallest count whose plain
    renders met the target on every calibration room, else the largest tried."""
    from nostrum_pray_gb300 import denoise
    curves = [[(4, 0.05, 1.0), (8, 0.009, 2.0), (16, 0.004, 4.0)],
              [(4, 0.08, 1.0), (8, 0.02, 2.0), (16, 0.008, 4.0)]]
    assert denoise.fallback_spp_from(curves, 0.01) == 16
    assert denoise.fallback_spp_from(curves, 0.03) == 8
    assert denoise.fallback_spp_from(curves, 0.001) == 16


def test_plain_time_to_target_bisects():
    """The plain renderer's time to the target comes from the smallest sample
    count that meets it: bisection between the curve's last count above the
    target and its first below, rendering only the counts in between."""
    from nostrum_pray_gb300 import denoise
    err = lambda spp: 0.1 / spp  # meets 0.01 from 10 spp
    curve = [(s, err(s), s * 1e-3) for s in (1, 2, 4, 8, 16, 32)]
    seen = []

    def measure(spp):
        seen.append(spp)
        return err(spp), spp * 1e-3

    assert denoise.smallest_spp(curve, 0.01, measure) == (10, 0.01, 10e-3)
    assert seen == [12, 10, 9]
    seen.clear()
    assert denoise.smallest_spp(curve, 0.2, measure) == (1, 0.1, 1e-3) and not seen
    assert denoise.smallest_spp(curve, 0.001, measure) is None and not seen
    # the first count already meets it: bisect from zero
    assert denoise.smallest_spp(curve[2:], 0.04, measure) == (3, 0.1 / 3, 3e-3)


def test_denoiser_input_depth():
    """A cut input depth applies to the noisy input's render only: the
    references and the plain renders keep the full path depth."""
    from nostrum_pray_gb300 import denoise
    cfg = denoise.DenoiseConfig(res=64, spp_in=1, depth_in=3)
    st = denoise._setup(cfg)
    p_in = denoise.input_params(cfg, st, seed=5)
    assert (p_in.max_depth, p_in.num_samples, p_in.rr_depth) == (3, 1, cfg.rr_depth)
    assert denoise._params(cfg, st, 16, seed=5).max_depth == cfg.depth == 8
    full = denoise.DenoiseConfig(res=64, spp_in=4)
    assert denoise.input_params(full, denoise._setup(full), seed=5).max_depth == 8
