"""The warp-packet walk's FMA slab test (traverse.cuh slab_fma: p * inv plus
the once-rounded -o * inv, one FMA per plane) on the culling copy's padded
boxes (host/flatten.cpp padded_box): for rays from anywhere within the
culling reach (4 scene diagonals of the scene's centre) aimed at points of a
triangle -- its vertices included, which lie on the planes of its tight box
-- the padded box passes the test with the hit distance inside [tn, tf],
near the world origin and far from it, for near-axis directions too. The
same rays against unpadded boxes fail, so the pad is what the argument rests
on. float32 arithmetic is emulated in numpy: a product of two float32 values
is exact in float64, and an FMA is its float64 sum rounded to float32."""
import numpy as np
import pytest

F32 = np.float32
FLT_MAX = float(np.finfo(np.float32).max)
PAD_REL = 2.0 ** -16   # kPadRel
PAD_SCENE = 2.0 ** -16  # kPadScene
REACH = 4.0             # kCullReach


def make_rays(o, p):
    """make_ray of traverse.cuh in float32: normalised direction, 1 / d."""
    d = (p - o.astype(np.float64)).astype(F32)
    n2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(F32)
    inv = (F32(1.0) / np.sqrt(n2)).astype(F32)
    d = (d * inv[:, None]).astype(F32)
    with np.errstate(divide="ignore"):
        ind = (F32(1.0) / d).astype(F32)
    return d, ind


def padded_boxes(tris, diag, pad=True):
    """padded_box of one triangle per row (float32, as the flattener)."""
    lo = tris.min(axis=1).astype(F32)
    hi = tris.max(axis=1).astype(F32)
    if not pad:
        return lo, hi
    p = ((np.abs(lo) + np.abs(hi) + (hi - lo)) * F32(PAD_REL) + F32(diag * PAD_SCENE) + F32(1e-30)).astype(F32)
    return (lo - p).astype(F32), (hi + p).astype(F32)


def slab_fma(lo, hi, o, ind):
    no = (-(o.astype(np.float64) * ind.astype(np.float64))).astype(F32)
    t1 = (lo.astype(np.float64) * ind.astype(np.float64) + no.astype(np.float64)).astype(F32)
    t2 = (hi.astype(np.float64) * ind.astype(np.float64) + no.astype(np.float64)).astype(F32)
    mn, mx = np.minimum(t1, t2), np.maximum(t1, t2)
    tn = np.maximum(mn.max(axis=1), F32(-FLT_MAX))
    tf = np.minimum(mx.min(axis=1), F32(FLT_MAX))
    return tn, tf


def scene(center, n, rng):
    """n small triangles in a box of edge 2 around `center` (float32)."""
    c = rng.uniform(-1.0, 1.0, (n, 1, 3)) + np.asarray(center, np.float64)
    tris = (c + rng.uniform(-0.05, 0.05, (n, 3, 3))).astype(F32)
    lo, hi = tris.reshape(-1, 3).min(0).astype(np.float64), tris.reshape(-1, 3).max(0).astype(np.float64)
    return tris, float(np.linalg.norm(hi - lo)), (lo + hi) / 2


def rays_at_triangles(tris, diag, centre, rng, n):
    """Origins within the reach, aimed at vertices (half) or interior points
    of random triangles; a tenth of them nearly parallel to an axis plane."""
    k = rng.integers(0, len(tris), n)
    t = tris[k].astype(np.float64)
    w = rng.dirichlet([1.0, 1.0, 1.0], n)
    vert = rng.integers(0, 3, n)
    on_vertex = rng.random(n) < 0.5
    w[on_vertex] = np.eye(3)[vert[on_vertex]]
    p = np.einsum("ni,nij->nj", w, t)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    o = centre + u * (REACH * diag * rng.random((n, 1)) ** (1 / 3))
    flat = rng.random(n) < 0.1
    axis = rng.integers(0, 3, n)
    idx = np.nonzero(flat)[0]
    near = p[idx, axis[idx]]
    o[idx, axis[idx]] = near + rng.uniform(-1.0, 1.0, idx.size) * (1e-5 * diag + 2.0 ** -18 * np.abs(near))
    o = o.astype(F32)
    # keep the origins within the reach after rounding, and off the points
    keep = (np.linalg.norm(o.astype(np.float64) - centre, axis=1) <= REACH * diag) & \
        (np.linalg.norm(p - o.astype(np.float64), axis=1) > 1e-3 * diag)
    return k[keep], p[keep], o[keep]


@pytest.mark.parametrize("center", [(0.0, 0.0, 0.0), (3.0, -2.0, 1.0), (3000.0, -1000.0, 500.0),
                                    (-2.0e5, 7.0e4, 1.0e3)])
def test_fma_slab_keeps_hits_inside_padded_boxes(center):
    rng = np.random.default_rng(abs(int(center[0])) + 17)
    tris, diag, centre = scene(center, 2000, rng)
    k, p, o = rays_at_triangles(tris, diag, centre, rng, 200_000)
    d, ind = make_rays(o, p)
    # the rays the packet walk takes (traverse_coherent: finite 1 / d and o / d)
    with np.errstate(invalid="ignore", over="ignore"):
        ok = np.isfinite(ind).all(1) & np.isfinite((o * ind).astype(F32)).all(1)
    assert ok.mean() > 0.98
    k, p, o, d, ind = k[ok], p[ok], o[ok], d[ok], ind[ok]
    # distance along the float32 ray to the closest approach to the point
    t_hit = np.einsum("nj,nj->n", p - o.astype(np.float64), d.astype(np.float64)) / \
        np.einsum("nj,nj->n", d.astype(np.float64), d.astype(np.float64))
    lo, hi = padded_boxes(tris[k], diag)
    tn, tf = slab_fma(lo, hi, o, ind)
    assert (tn <= tf).all()
    assert (tn.astype(np.float64) <= t_hit).all() and (tf.astype(np.float64) >= t_hit).all()
    # the pruning bound: a box entered by the winning hit is never pruned
    assert (tn.astype(np.float64) <= t_hit * (1 + 2.0 ** -12)).all()
    # control: the unpadded boxes lose some of the same hits
    lo0, hi0 = padded_boxes(tris[k], diag, pad=False)
    tn0, tf0 = slab_fma(lo0, hi0, o, ind)
    lost = (tn0 > tf0) | (tn0.astype(np.float64) > t_hit) | (tf0.astype(np.float64) < t_hit)
    assert lost.sum() > 100
