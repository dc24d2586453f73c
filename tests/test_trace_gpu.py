"""Parity of the CUDA ray-tracing path with the oracle (GPU).

Every comparison is bit-exact: hit triangle ids, hit distances (as bit
patterns) and image bytes. The oracle itself is pinned against the reference
(test_oracle_golden.py), and the full-size cases are also checked against the
digests the reference produced (tests/golden/golden_hashes.json)."""
import json
import os

import numpy as np
import pytest

from golden_util import sha
from nostrum_pray_gb300 import native, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    native.lib()
    torch.cuda.set_device(0)


def render(sc, setup):
    h, w = setup.height, setup.width
    rgb = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    ids = torch.empty((h, w), dtype=torch.int32, device="cuda")
    ts = torch.empty((h, w), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    sc.render_rt(setup, rgb, ids, ts, cnt)
    torch.cuda.synchronize()
    return rgb.cpu().numpy(), ids.cpu().numpy().reshape(-1), ts.cpu().numpy().reshape(-1), cnt.cpu().numpy()


def trace(sc, rays, eps):
    r = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    n = rays.shape[0]
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    ts = torch.empty(n, dtype=torch.float32, device="cuda")
    sc.trace_closest(r, eps, ids, ts)
    torch.cuda.synchronize()
    return ids.cpu().numpy(), ts.cpu().numpy()


def check_frame(oracle, mesh, setup, traversal=native.TRAVERSAL_AUTO):
    sc = native.Scene.from_setup(mesh, setup)
    sc.set_traversal(traversal)
    img, ids, ts, cnt = render(sc, setup)
    orc = oracle.OracleScene.from_setup(mesh, setup)
    want_img, want_sh = orc.render_rt(setup)
    rays = oracle.primary_rays(setup.width, setup.height, setup.fov, setup.cam_pos, setup.cam_look)
    want_ids, want_t = orc.trace(rays, setup.det_eps)
    mism = int((ids != want_ids.astype(np.int32)).sum())
    assert mism == 0, f"{mism} hit ids differ"
    np.testing.assert_array_equal(ts.view(np.uint32), want_t.view(np.uint32))
    np.testing.assert_array_equal(img, want_img)
    assert int(cnt[0]) == setup.width * setup.height
    assert int(cnt[1]) == want_sh
    # host-memory entry point gives the same frame
    himg, rays_cast = sc.render_rt_host(setup)
    np.testing.assert_array_equal(himg, want_img)
    assert int(rays_cast[1]) == want_sh
    return img, ids, ts


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_soup_frame(oracle, seed):
    check_frame(oracle, scenes.soup(10_000, seed), scenes.soup_setup())


@pytest.mark.parametrize("traversal", [native.TRAVERSAL_LANES, native.TRAVERSAL_PACKETS,
                                       native.TRAVERSAL_PRIMARY_PACKETS])
@pytest.mark.parametrize("scene", ["soup", "sphere", "sah_soup", "far_camera"])
def test_frame_traversals(oracle, traversal, scene):
    """Each traversal of the ray-traced frame (per lane; warp packets over a
    pixel tile for the primary and occlusion rays, or for the primary rays
    only) gives the oracle's frame: hit ids, distances, image. The distant
    camera's rays take the exact node copy, which packet warps leave to the
    per-lane walk."""
    if scene == "soup":
        m, st = scenes.soup(10_000, 3), scenes.soup_setup(256, 192)
    elif scene == "sphere":
        m, st = scenes.icosphere(6), scenes.icosphere_setup(320, 240)
    elif scene == "sah_soup":
        m, st = scenes.soup(10_000, 4), scenes.soup_setup(320, 240)
        st.tree, st.leaf_size, st.max_depth, st.sah_ct = "sah", 32, 20, 1.0
    else:
        m, st = scenes.soup(10_000, 5), scenes.soup_setup(160, 120)
        st.cam_pos, st.fov = (0.5, 0.5, -30.0), 3
    check_frame(oracle, m, st, traversal)


def test_traversal_choice():
    """AUTO picks one of the traversals on the first frame and keeps it; an
    explicit choice is kept as given."""
    m, st = scenes.soup(2_000, 1), scenes.soup_setup(64, 64)
    sc = native.Scene.from_setup(m, st)
    assert sc.traversal() == native.TRAVERSAL_AUTO
    sc.render_rt_host(st)
    assert sc.traversal() in (native.TRAVERSAL_LANES, native.TRAVERSAL_PACKETS, native.TRAVERSAL_PRIMARY_PACKETS)
    sc.set_traversal(native.TRAVERSAL_PACKETS)
    sc.render_rt_host(st)
    assert sc.traversal() == native.TRAVERSAL_PACKETS
    with pytest.raises(native.PrayError):
        sc.set_traversal(5)


def test_soup_sah_default_constants(oracle):
    st = scenes.soup_setup(320, 240)
    st.tree, st.leaf_size, st.max_depth = "sah", 32, 20
    check_frame(oracle, scenes.soup(10_000, 4), st)


@pytest.mark.parametrize("eps", [0.0, 1e-4])
def test_icosphere_level5(oracle, golden, eps):
    hashes, small = golden
    st = scenes.icosphere_setup(480, 270, det_eps=eps)
    img, ids, ts = check_frame(oracle, scenes.icosphere(5), st)
    key = f"ico5_eps{eps:g}"
    assert sha(img) == hashes[key]["image"]  # the reference's own frame
    assert sha(ids) == hashes[key]["ids"] and sha(ts) == hashes[key]["t"]


@pytest.mark.parametrize("name", ["cube", "head_fov30", "plant"])
def test_examples(oracle, golden, name):
    hashes, small = golden
    info = small[f"ex_{name}_info"]
    m = scenes.Mesh(small[f"ex_{name}_verts"], small[f"ex_{name}_colors"], small[f"ex_{name}_emit"])
    st = scenes.RenderSetup(width=160, height=120, fov=int(info[2]), cam_pos=tuple(info[6:9]),
                            cam_look=tuple(info[9:12]), lights=[tuple(l) for l in small[f"ex_{name}_lights"]],
                            background=tuple(info[12:15]), tree="median")
    img, _, _ = check_frame(oracle, m, st)
    np.testing.assert_array_equal(img, small[f"ex_{name}_image160"])


def test_random_rays_inside_scene(oracle):
    """Rays from inside the soup in random directions, including exact axis
    directions and zero components (infinite inverse directions)."""
    m = scenes.soup(10_000, 5)
    st = scenes.soup_setup()
    sc = native.Scene.from_setup(m, st)
    orc = oracle.OracleScene.from_setup(m, st)
    rng = np.random.default_rng(0)
    n = 200_000
    o = rng.uniform(-0.2, 1.2, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 10, 1:] = 0.0          # +-x axis rays
    d[n // 10: n // 5, 0] = 0.0      # rays in the yz plane
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    with np.errstate(divide="ignore"):
        inv = (1.0 / d).astype(np.float32)
    rays = np.concatenate([o, d, inv], 1)
    for eps in (1e-4, 0.0):
        ids, ts = trace(sc, rays, eps)
        wid, wt = orc.trace(rays, eps)
        assert int((ids != wid.astype(np.int32)).sum()) == 0
        np.testing.assert_array_equal(ts.view(np.uint32), wt.view(np.uint32))


@pytest.mark.parametrize("tree", ["median", "sah"])
def test_occlusion_rays(oracle, tree):
    """pray_trace_occluded against the reference's shadow test on the
    oracle's closest hits (occluded iff a hit with dist2 > t * t,
    src/pray.cpp:39-43): random rays inside the soup with distances around
    their closest hits, including dist2 exactly t * t (not occluded), the
    next float above it (occluded), zero, negative and infinite."""
    m = scenes.soup(10_000, 6)
    st = scenes.soup_setup()
    st.tree = tree
    sc = native.Scene.from_setup(m, st)
    orc = oracle.OracleScene.from_setup(m, st)
    rng = np.random.default_rng(3)
    n = 120_000
    o = rng.uniform(-0.2, 1.2, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 20, 1:] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    with np.errstate(divide="ignore"):
        inv = (1.0 / d).astype(np.float32)
    rays = np.concatenate([o, d, inv], 1).astype(np.float32)
    for eps in (1e-4, 0.0):
        wid, wt = orc.trace(rays, eps)
        hit = wid >= 0
        tt = np.where(hit, wt, 1.0).astype(np.float32)
        t2 = (tt * tt).astype(np.float32)
        kind = rng.integers(0, 7, n)
        dist2 = np.select([kind == 0, kind == 1, kind == 2, kind == 3, kind == 4, kind == 5],
                          [t2, np.nextafter(t2, np.float32(np.inf)), np.float32(0), np.float32(-1),
                           np.float32(np.inf), t2 * np.float32(0.25)],
                          rng.uniform(0, 4, n).astype(np.float32) * t2).astype(np.float32)
        want = (hit & (dist2 > t2)).astype(np.uint8)
        r = torch.from_numpy(rays).cuda()
        dd = torch.from_numpy(dist2).cuda()
        occ = torch.empty(n, dtype=torch.uint8, device="cuda")
        sc.trace_occluded(r, dd, eps, occ)
        torch.cuda.synchronize()
        got = occ.cpu().numpy()
        assert int((got != want).sum()) == 0, f"{int((got != want).sum())} occlusion answers differ"
        assert 0 < int(want.sum()) < n


def test_ties_duplicated_triangles(oracle):
    """Coincident copies of each triangle: equal distances, so the first in
    the reference's depth-first order must win."""
    base = scenes.soup(3_000, 9)
    m = scenes.Mesh(np.concatenate([base.verts, base.verts[::-1]]), np.concatenate([base.colors, base.colors]),
                    np.zeros(6_000, np.uint8))
    for tree in ("median", "sah"):
        st = scenes.soup_setup(256, 256)
        st.tree = tree
        check_frame(oracle, m, st)


def test_empty_and_tiny_scenes(oracle):
    st = scenes.soup_setup(33, 17)  # ragged size: partial 8x4 tiles
    st.background = (0.25, 0.5, 1.0)
    empty = scenes.Mesh(np.zeros((0, 9), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.uint8))
    sc = native.Scene.from_setup(empty, st)
    img, _ = sc.render_rt_host(st)
    want = np.array([int(np.float32(c) * np.float32(255) + np.float32(0.5)) for c in st.background], np.uint8)
    assert (img == want).all()
    one = scenes.Mesh(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32) + np.float32(0.5) * 0,
                      np.array([[0.5, 0.6, 0.7]], np.float32), np.zeros(1, np.uint8))
    st2 = scenes.RenderSetup(width=64, height=48, fov=60, cam_pos=(0.2, 0.2, -2.0), cam_look=(0, 0, 1),
                             lights=[(0.2, 0.2, -1.0, 1, 1, 1)])
    check_frame(oracle, one, st2)


def test_invalid_arguments_raise():
    st = scenes.soup_setup(16, 16)
    m = scenes.soup(100, 0)
    with pytest.raises(native.PrayError):
        native.Scene(m, native.tree_options(st, max_depth=31))
    sc = native.Scene.from_setup(m, st)
    bad = scenes.soup_setup(0, 16)
    with pytest.raises(native.PrayError):
        sc.render_rt_host(bad)


@pytest.mark.slow
def test_icosphere_level8_full(oracle, golden):
    """The 1.31M-triangle displaced sphere at 1920x1080 with the SAH tree:
    GPU frame == oracle frame == the reference's frame (digests)."""
    hashes, _ = golden
    m = scenes.icosphere(8)
    for eps in (0.0, 1e-4):
        st = scenes.icosphere_setup(det_eps=eps)
        img, ids, ts = check_frame(oracle, m, st)
        key = f"ico8_eps{eps:g}"
        assert sha(img) == hashes[key]["image"]
        assert sha(ids) == hashes[key]["ids"] and sha(ts) == hashes[key]["t"]


def test_rays_through_vertices_and_edges(oracle):
    """Rays aimed at triangle vertices, edge midpoints and edge thirds (u or v
    at or next to 0 and 1, u + v at 1): the intersector's early outs must
    decide exactly as the reference's full computation."""
    m = scenes.soup(4_000, 12)
    st = scenes.soup_setup()
    sc = native.Scene.from_setup(m, st)
    orc = oracle.OracleScene.from_setup(m, st)
    rng = np.random.default_rng(5)
    v = m.verts.reshape(-1, 3, 3).astype(np.float64)
    tri = rng.integers(0, m.n, 60_000)
    which = rng.integers(0, 6, tri.size)
    a, b, c = v[tri, 0], v[tri, 1], v[tri, 2]
    targets = np.where((which == 0)[:, None], a, np.where((which == 1)[:, None], b, np.where(
        (which == 2)[:, None], c, np.where((which == 3)[:, None], (a + b) / 2, np.where(
            (which == 4)[:, None], (b + c) / 2, a + (c - a) / 3)))))
    o = rng.uniform(-1.0, 2.0, (tri.size, 3))
    d = targets - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    with np.errstate(divide="ignore"):
        rays = np.concatenate([o.astype(np.float32), d, (1.0 / d).astype(np.float32)], 1)
    for eps in (1e-4, 0.0):
        ids, ts = trace(sc, rays, eps)
        wid, wt = orc.trace(rays, eps)
        assert int((ids != wid.astype(np.int32)).sum()) == 0
        np.testing.assert_array_equal(ts.view(np.uint32), wt.view(np.uint32))


@pytest.mark.parametrize("dist", [0.3, 1.5, 3.5, 6.0, 100.0, 3000.0])
def test_distant_origins(oracle, dist):
    """Rays from origins `dist` scene diagonals from the scene's centre (from
    inside the scene to far beyond the reach of the padded culling boxes,
    where the exact node copy serves them), aimed at a cluster of small
    triangles next to the world origin inside a scene of large ones: the
    float error of a slab test grows with the distance travelled, not with
    the small boxes' coordinates."""
    rng = np.random.default_rng(int(dist * 10))
    small = scenes.soup(20_000, 7)
    big = scenes.soup(300, 8, spread=0.05)
    m = scenes.Mesh(np.concatenate([small.verts * np.float32(0.02), big.verts * np.float32(2) - np.float32(1)]),
                    np.concatenate([small.colors, big.colors]), np.zeros(20_300, np.uint8))
    st = scenes.room_setup(64, 64)
    sc = native.Scene.from_setup(m, st)
    orc = oracle.OracleScene.from_setup(m, st)
    v = m.verts.reshape(-1, 3).astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    centre, diag = (lo + hi) / 2, float(np.linalg.norm(hi - lo))
    n = 60_000
    u = rng.normal(size=(n, 3))
    o = centre + dist * diag * u / np.linalg.norm(u, axis=1, keepdims=True)
    tgt = np.where((rng.random(n) < 0.7)[:, None], rng.uniform(-0.001, 0.021, (n, 3)), rng.uniform(lo, hi, (n, 3)))
    o = o.astype(np.float32)
    d = (tgt - o.astype(np.float64))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays = np.concatenate([o, d, (1.0 / d).astype(np.float32)], 1)
    ids, ts = trace(sc, rays, 0.0)
    wid, wt = orc.trace(rays, 0.0)
    assert (wid >= 0).sum() > n // 3
    assert int((ids != wid.astype(np.int32)).sum()) == 0
    np.testing.assert_array_equal(ts.view(np.uint32), wt.view(np.uint32))


def test_host_rays_from_many_threads(oracle):
    """pray_trace_closest_host, the entry point behind the reference-side
    SpatialDatabase::intersect binding: host rays in, host ids and distances
    out, called concurrently from eight host threads on one scene (the
    reference's renderers query the database from OpenMP threads), with
    batches of one ray up to whole frames; bit-exact against the oracle."""
    from concurrent.futures import ThreadPoolExecutor
    mesh = scenes.soup(10_000, 2)
    st = scenes.soup_setup(96, 80)
    sc = native.Scene.from_setup(mesh, st)
    rays = oracle.primary_rays(st.width, st.height, st.fov, st.cam_pos, st.cam_look)
    want_ids, want_t = oracle.OracleScene.from_setup(mesh, st).trace(rays, st.det_eps)
    sizes = [1, 7, 64, 1000, rays.shape[0]]

    def job(k):
        n = sizes[k % len(sizes)]
        lo = (k * 977) % (rays.shape[0] - n + 1)
        ids, ts = sc.trace_closest_host(rays[lo:lo + n], st.det_eps)
        return lo, n, ids, ts

    with ThreadPoolExecutor(8) as ex:
        results = list(ex.map(job, range(64)))
    for lo, n, ids, ts in results:
        np.testing.assert_array_equal(ids, want_ids[lo:lo + n].astype(np.int32))
        np.testing.assert_array_equal(ts.view(np.uint32), want_t[lo:lo + n].view(np.uint32))
    assert int((want_ids >= 0).sum()) > 500
    ids, ts = sc.trace_closest_host(rays[:0], st.det_eps)
    assert ids.size == 0
    sc.close()
