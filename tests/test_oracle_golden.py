"""Pins the oracle (oracle/pray_oracle.cpp) against outputs of the reference
itself, recorded in tests/golden/ by make_golden.py from the reference's own
sources: tree dumps, triangle precompute, primary rays, per-ray hit ids and
distances, and ray-traced images."""
import numpy as np
import pytest

from golden_util import dump_hash, mesh_hash, sha
from nostrum_pray_gb300 import scenes


def _trace(O, osc, st):
    rays = O.primary_rays(st.width, st.height, st.fov, st.cam_pos, st.cam_look)
    ids, ts = osc.trace(rays, st.det_eps)
    return rays, ids.astype(np.int32), ts


def test_soup_seed0_arrays(oracle, golden):
    hashes, small = golden
    m = scenes.soup(10_000, 0)
    assert mesh_hash(m) == hashes["soup_s0"]["mesh"], "scene generator drifted"
    st = scenes.soup_setup()
    osc = oracle.OracleScene.from_setup(m, st)
    d = osc.tree_dump()
    for k in ("boxes", "split", "info", "refs"):
        np.testing.assert_array_equal(d[k], small[f"soup_s0_tree_{k}"])
    np.testing.assert_array_equal(osc.precompute()[:256].view(np.uint32),
                                  small["soup_s0_precompute"].view(np.uint32))
    rays, ids, ts = _trace(oracle, osc, st)
    np.testing.assert_array_equal(ids, small["soup_s0_ids"])
    np.testing.assert_array_equal(ts.view(np.uint32), small["soup_s0_t"].view(np.uint32))
    img, nsh = osc.render_rt(st)
    np.testing.assert_array_equal(img, small["soup_s0_image"])
    assert nsh > 0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_soup_hashes(oracle, golden, seed):
    hashes, _ = golden
    key = f"soup_s{seed}"
    m = scenes.soup(10_000, seed)
    st = scenes.soup_setup()
    osc = oracle.OracleScene.from_setup(m, st)
    g = hashes[key]
    assert [int(x) for x in osc.tree_stats()] == g["stats"]
    assert dump_hash(osc.tree_dump()) == g["tree"]
    rays, ids, ts = _trace(oracle, osc, st)
    assert sha(rays) == g["rays"]
    assert sha(ids) == g["ids"] and sha(ts) == g["t"]
    assert sha(osc.render_rt(st)[0]) == g["image"]
    # the reference's SAH tree (default constants) on the same soup
    st.tree, st.leaf_size, st.max_depth = "sah", 32, 20
    osc2 = oracle.OracleScene.from_setup(m, st)
    g2 = hashes[key + "_sah"]
    assert [int(x) for x in osc2.tree_stats()] == g2["stats"]
    assert dump_hash(osc2.tree_dump()) == g2["tree"]
    _, ids2, ts2 = _trace(oracle, osc2, st)
    assert sha(ids2) == g2["ids"] and sha(ts2) == g2["t"]
    assert sha(osc2.render_rt(st)[0]) == g2["image"]


@pytest.mark.parametrize("eps", [0.0, 1e-4])
def test_icosphere_level5(oracle, golden, eps):
    hashes, small = golden
    key = f"ico5_eps{eps:g}"
    m = scenes.icosphere(5)
    assert mesh_hash(m) == hashes[key]["mesh"]
    st = scenes.icosphere_setup(480, 270, det_eps=eps)
    osc = oracle.OracleScene.from_setup(m, st)
    d = osc.tree_dump()
    assert dump_hash(d) == hashes[key]["tree"]
    rays, ids, ts = _trace(oracle, osc, st)
    assert sha(ids) == hashes[key]["ids"] and sha(ts) == hashes[key]["t"]
    img, _ = osc.render_rt(st)
    assert sha(img) == hashes[key]["image"]
    if eps == 0.0:
        np.testing.assert_array_equal(ids, small[key + "_ids"])
        np.testing.assert_array_equal(img, small[key + "_image"])


@pytest.mark.slow
def test_icosphere_level8_full(oracle, golden):
    """The 1.31M-triangle sphere at 1920x1080: SAH tree, hits and image."""
    hashes, _ = golden
    m = scenes.icosphere(8)
    assert mesh_hash(m) == hashes["ico8_eps0"]["mesh"]
    st = scenes.icosphere_setup(det_eps=0.0)
    osc = oracle.OracleScene.from_setup(m, st)
    assert [int(x) for x in osc.tree_stats()] == hashes["ico8_eps0"]["stats"]
    assert dump_hash(osc.tree_dump()) == hashes["ico8_eps0"]["tree"]
    for eps in (0.0, 1e-4):
        key = f"ico8_eps{eps:g}"
        st = scenes.icosphere_setup(det_eps=eps)
        rays, ids, ts = _trace(oracle, osc, st)
        assert sha(rays) == hashes[key]["rays"]
        assert int((ids >= 0).sum()) == hashes[key]["hits"]
        assert sha(ids) == hashes[key]["ids"] and sha(ts) == hashes[key]["t"]
        assert sha(osc.render_rt(st)[0]) == hashes[key]["image"]


@pytest.mark.parametrize("name", ["cube", "head_fov30", "plant"])
def test_examples_render(oracle, golden, name):
    """Reference example scenes (triangles as the reference's loader read them),
    rendered at 160x120 with their own camera and lights."""
    hashes, small = golden
    if f"ex_{name}_verts" not in small:
        pytest.skip("example not recorded")
    info = small[f"ex_{name}_info"]
    m = scenes.Mesh(small[f"ex_{name}_verts"], small[f"ex_{name}_colors"], small[f"ex_{name}_emit"])
    lights = small[f"ex_{name}_lights"]
    st = scenes.RenderSetup(width=160, height=120, fov=int(info[2]), cam_pos=tuple(info[6:9]),
                            cam_look=tuple(info[9:12]), lights=[tuple(l) for l in lights],
                            background=tuple(info[12:15]), tree="median")
    osc = oracle.OracleScene.from_setup(m, st)
    assert [int(x) for x in osc.tree_stats()] == hashes[f"ex_{name}"]["stats"]
    assert dump_hash(osc.tree_dump()) == hashes[f"ex_{name}"]["tree"]
    img, _ = osc.render_rt(st)
    np.testing.assert_array_equal(img, small[f"ex_{name}_image160"])


def test_oracle_detects_planted_mistake(oracle):
    """A mistake planted in the oracle's input (one vertex pushed out of the
    root box by one ulp) changes the tree digest: the golden comparison is
    sensitive to single-ulp differences."""
    m = scenes.soup(2_000, 3)
    st = scenes.soup_setup()
    a = dump_hash(oracle.OracleScene.from_setup(m, st).tree_dump())
    k = int(np.argmax(m.verts[:, 0::3].max(1)))
    m.verts[k, 0::3] = np.nextafter(m.verts[k, 0::3].max(), np.float32(2))
    b = dump_hash(oracle.OracleScene.from_setup(m, st).tree_dump())
    assert a != b


@pytest.mark.parametrize("depth,n", [(0, 4), (1, 4), (1, 3), (2, 3)])
def test_oracle_branching_known_answer(oracle, depth, n):
    """The branching path tracer (evaluatePathRecursiveDiffuse,
    src/pray.cpp:315-340) on one front-facing triangle: bounce rays leave
    through its front side and are culled by the one-sided test, so every
    bounce returns the background and a covered pixel is exactly
    (bg + ... + bg) * albedo / n at depth >= 1 (black at depth 0); other
    pixels show the background. Rays: one per pixel plus n per covered pixel."""
    m = scenes.Mesh(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32), np.array([[0.5, 0.25, 0.75]], np.float32),
                    np.zeros(1, np.uint8))
    st = scenes.RenderSetup(width=24, height=20, fov=60, cam_pos=(0.25, 0.25, 2.0), cam_look=(0, 0, -1), lights=[],
                            background=(0.5, 0.5, 0.5))
    osc = oracle.OracleScene.from_setup(m, st)
    rays = oracle.primary_rays(st.width, st.height, st.fov, st.cam_pos, st.cam_look)
    ids, _ = osc.trace(rays, st.det_eps)
    covered = (ids >= 0).reshape(st.height, st.width)
    assert 0 < covered.sum() < covered.size
    img, rad, segs = osc.render_pt(st, spp=n, max_depth=depth, seed=1, mode=2)
    bg = np.float32(0.5)
    s = np.float32(0)
    for _ in range(n):
        s = np.float32(s + bg)
    hit = (s * m.colors[0]) / np.float32(n) if depth >= 1 else np.zeros(3, np.float32)
    want = np.where(covered[..., None], hit[None, None, :], np.full(3, bg, np.float32)).astype(np.float32)
    np.testing.assert_array_equal(rad, want)
    assert segs == covered.size + (n * int(covered.sum()) if depth >= 1 else 0)
