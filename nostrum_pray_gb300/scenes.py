"""Seeded synthetic scenes for the ray/path-tracing workloads.

Every generator returns plain numpy arrays in the layout the reference's
``Triangle`` constructor takes (``include/geometry.h:236-239``): per triangle the
three vertices ``a, b, c`` (9 float32), an RGB colour (3 float32: diffuse
albedo, or radiance for an emitter) and an emitter flag.  ``RenderSetup`` holds
what the reference reads from the scene JSON (``src/io.cpp:60-101``) plus the
compile-time constants of the reference that these workloads change (leaf
size, depth limit, SAH costs, det threshold), which this framework takes at run
time.
"""
from __future__ import annotations

import dataclasses
import json
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np


@dataclasses.dataclass
class Mesh:
    verts: np.ndarray  # (n, 9) float32: a.xyz, b.xyz, c.xyz
    colors: np.ndarray  # (n, 3) float32
    emit: np.ndarray  # (n,) uint8

    @property
    def n(self) -> int:
        return int(self.verts.shape[0])

    def __post_init__(self):
        self.verts = np.ascontiguousarray(self.verts, dtype=np.float32).reshape(-1, 9)
        self.colors = np.ascontiguousarray(self.colors, dtype=np.float32).reshape(-1, 3)
        self.emit = np.ascontiguousarray(self.emit, dtype=np.uint8).reshape(-1)


@dataclasses.dataclass
class RenderSetup:
    width: int
    height: int
    fov: int  # degrees; the reference stores it as an unsigned integer
    cam_pos: Tuple[float, float, float]
    cam_look: Tuple[float, float, float]
    lights: List[Tuple[float, float, float, float, float, float]]  # position, colour
    background: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    tree: str = "median"  # "median" | "sah"
    leaf_size: int = 32  # include/kd_tree.h:50 THRESHOLD
    max_depth: int = 20  # include/kd_tree.h:52 MAX_DEPTH
    sah_ct: float = 5.0  # include/kd_tree_sah.h:49 traversalCost
    sah_ci: float = 1.5  # include/kd_tree_sah.h:50 triangleIntersectionCost
    det_eps: float = 1e-4  # include/geometry.h:12 EPSILON
    method: str = "ray_tracing"  # or "path_tracing"
    max_depth_pt: int = 0
    num_samples: int = 0

    def lights_array(self) -> np.ndarray:
        return np.asarray(self.lights, dtype=np.float32).reshape(-1, 6)


# --------------------------------------------------------------------------
# Triangle soup: 10,000 triangles, centre U[0,1]^3, vertex offsets
# U[-0.02,0.02]^3, albedo U[0.2,0.9]^3.


def soup(n: int = 10_000, seed: int = 0, spread: float = 0.02) -> Mesh:
    rng = np.random.default_rng(seed)
    centre = rng.uniform(0.0, 1.0, size=(n, 1, 3))
    offs = rng.uniform(-spread, spread, size=(n, 3, 3))
    verts = (centre + offs).reshape(n, 9).astype(np.float32)
    colors = rng.uniform(0.2, 0.9, size=(n, 3)).astype(np.float32)
    return Mesh(verts, colors, np.zeros(n, np.uint8))


def soup_setup(width: int = 512, height: int = 512) -> RenderSetup:
    return RenderSetup(width=width, height=height, fov=60, cam_pos=(0.5, 0.5, -1.5),
                       cam_look=(0.0, 0.0, 1.0), lights=[(0.5, 2.0, 0.5, 1.0, 1.0, 1.0)],
                       tree="median", leaf_size=8, max_depth=24)


# --------------------------------------------------------------------------
# Displaced icosphere: 20 faces subdivided `level` times (20 * 4^level
# triangles), radius r, vertices moved radially by amp * value noise.


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, f


def _subdivide(v: np.ndarray, f: np.ndarray):
    nv = v.shape[0]
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
    e.sort(axis=1)
    key = e[:, 0] * nv + e[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a, b = uniq // nv, uniq % nv
    mid = v[a] + v[b]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    v2 = np.concatenate([v, mid], axis=0)
    nf = f.shape[0]
    m01 = nv + inv[:nf]
    m12 = nv + inv[nf:2 * nf]
    m20 = nv + inv[2 * nf:]
    f2 = np.concatenate([
        np.stack([f[:, 0], m01, m20], 1),
        np.stack([f[:, 1], m12, m01], 1),
        np.stack([f[:, 2], m20, m12], 1),
        np.stack([m01, m12, m20], 1)], axis=0)
    return v2, f2


def _hash3(ix, iy, iz, seed: int) -> np.ndarray:
    """Integer lattice hash -> uniform value in [-1, 1] (32-bit mixing)."""
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) \
        ^ (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32((seed * 0x9E3779B9) & 0xFFFFFFFF)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x7FEB352D)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x846CA68B)
    h ^= h >> np.uint32(16)
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise(p: np.ndarray, freq: float, seed: int) -> np.ndarray:
    """Trilinearly interpolated lattice value noise at points p (n, 3)."""
    q = p * freq
    i0 = np.floor(q).astype(np.int64)
    fr = q - i0
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        wx = fr[:, 0] if dx else 1.0 - fr[:, 0]
        for dy in (0, 1):
            wy = fr[:, 1] if dy else 1.0 - fr[:, 1]
            for dz in (0, 1):
                wz = fr[:, 2] if dz else 1.0 - fr[:, 2]
                out += wx * wy * wz * _hash3(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed)
    return out


def icosphere(level: int = 8, radius: float = 1.0, amp: float = 0.05, base_freq: float = 4.0,
              seed: int = 0, albedo=(0.8, 0.8, 0.8)) -> Mesh:
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    if amp != 0.0:
        n = (value_noise(v, base_freq, seed) + 0.5 * value_noise(v, 2 * base_freq, seed + 1)
             + 0.25 * value_noise(v, 4 * base_freq, seed + 2)) / 1.75
        v = v * (radius * (1.0 + amp * n))[:, None]
    else:
        v = v * radius
    verts = v[f].reshape(-1, 9)
    # outward normals: (b - a) x (c - a) points away from the centre so that the
    # one-sided intersector sees the outside
    a, b, c = verts[:, 0:3], verts[:, 3:6], verts[:, 6:9]
    nrm = np.cross(b - a, c - a)
    flip = (nrm * (a + b + c)).sum(1) < 0
    verts[flip] = np.concatenate([a, c, b], axis=1)[flip]
    nt = verts.shape[0]
    colors = np.tile(np.asarray(albedo, np.float32), (nt, 1))
    return Mesh(verts.astype(np.float32), colors, np.zeros(nt, np.uint8))


def icosphere_setup(width: int = 1920, height: int = 1080, det_eps: float = 0.0) -> RenderSetup:
    """1.31M-triangle displaced sphere at 1080p: camera at distance 3 looking at
    the origin, fov 45, two white-ish point lights, SAH kd tree with traversal
    cost 1 and intersection cost 1.5.  det_eps 0 keeps the reference's one-sided
    test but drops its absolute 1e-4 threshold, which culls every triangle of a
    unit sphere this fine (|ab x ac| ~ 2e-5)."""
    return RenderSetup(width=width, height=height, fov=45, cam_pos=(0.0, 0.0, -3.0),
                       cam_look=(0.0, 0.0, 1.0),
                       lights=[(2.0, 2.5, -3.0, 6.0, 6.0, 6.0), (-3.0, 1.0, -2.0, 3.0, 3.5, 4.0)],
                       tree="sah", leaf_size=32, max_depth=20, sah_ct=1.0, sah_ci=1.5,
                       det_eps=det_eps)


# --------------------------------------------------------------------------
# Scene files: the reference's JSON + OBJ/MTL format (src/io.cpp:27-137).


def write_scene(path_json: str, mesh: Mesh, setup: RenderSetup, obj_name: Optional[str] = None) -> None:
    """Writes a JSON scene plus an OBJ/MTL pair the reference's loader accepts.
    Vertices are printed with %.9g so that they read back bit-exactly."""
    base = os.path.dirname(os.path.abspath(path_json))
    stem = obj_name or (os.path.splitext(os.path.basename(path_json))[0] + ".obj")
    mtl = os.path.splitext(stem)[0] + ".mtl"
    cols, inv = np.unique(np.concatenate([mesh.colors, mesh.emit[:, None].astype(np.float32)], 1),
                          axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    with open(os.path.join(base, mtl), "w") as fm:
        for k, c in enumerate(cols):
            fm.write(f"newmtl m{k}\n")
            if c[3] != 0:
                fm.write("Kd 0 0 0\nKe %.9g %.9g %.9g\n" % (c[0], c[1], c[2]))
            else:
                fm.write("Kd %.9g %.9g %.9g\n" % (c[0], c[1], c[2]))
    order = np.argsort(inv, kind="stable")
    lines = [f"mtllib {mtl}\n", "o mesh\n"]
    v = mesh.verts.reshape(-1, 3)
    lines += ["v %.9g %.9g %.9g\n" % tuple(p) for p in v]
    # faces grouped by material keep the triangle order when the materials are
    # used in order; write one usemtl per run of equal material in file order
    cur = -1
    for i in range(mesh.n):
        if inv[i] != cur:
            cur = inv[i]
            lines.append(f"usemtl m{cur}\n")
        lines.append(f"f {3 * i + 1} {3 * i + 2} {3 * i + 3}\n")
    del order
    with open(os.path.join(base, stem), "w") as fo:
        fo.writelines(lines)
    doc = {
        "obj_file": stem,
        "resolution_x": setup.width,
        "resolution_y": setup.height,
        "camera_position": list(setup.cam_pos),
        "camera_look": list(setup.cam_look),
        "fov": setup.fov,
        "lights": [{"position": list(l[:3]), "color": list(l[3:])} for l in setup.lights],
        "background": list(setup.background),
    }
    if setup.method == "path_tracing":
        doc["method"] = "path_tracing"
        doc["max_depth"] = setup.max_depth_pt
        doc["num_samples"] = setup.num_samples
    with open(path_json, "w") as fj:
        json.dump(doc, fj, indent=1)


# --------------------------------------------------------------------------
# Closed box room for path tracing: 2x2x2 room (x in [-1,1], y in [0,2],
# z in [-1,1]) with inward-facing walls (white 0.75, red left wall, green right
# wall), an emissive 0.5x0.5 ceiling quad just below the ceiling, and boxes
# rotated about the vertical axis. Every face is a grid of quads split into
# two triangles each; `grid` sets the quads per face edge (53 gives ~101k
# triangles). The camera sits inside, in front of the front wall.

WHITE = (0.75, 0.75, 0.75)
RED = (0.63, 0.06, 0.05)
GREEN = (0.14, 0.45, 0.09)


def _quad_grid(origin, eu, ev, n: int) -> np.ndarray:
    """Triangles of an n x n grid over the parallelogram origin + s*eu + t*ev,
    wound so that (b-a) x (c-a) points along eu x ev."""
    o, eu, ev = (np.asarray(x, np.float64) for x in (origin, eu, ev))
    s = np.arange(n + 1) / n
    P = o[None, None, :] + s[:, None, None] * eu[None, None, :] + s[None, :, None] * ev[None, None, :]
    p00 = P[:-1, :-1].reshape(-1, 3)
    p10 = P[1:, :-1].reshape(-1, 3)
    p01 = P[:-1, 1:].reshape(-1, 3)
    p11 = P[1:, 1:].reshape(-1, 3)
    t1 = np.concatenate([p00, p10, p11], 1)
    t2 = np.concatenate([p00, p11, p01], 1)
    return np.stack([t1, t2], 1).reshape(-1, 9)


def _box_faces(center, size, angle_deg, n: int) -> List[np.ndarray]:
    """Outward-facing faces of a box rotated about +y, resting on y = 0."""
    cx, cz = center
    sx, sy, sz = size
    a = np.radians(angle_deg)
    R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    hx, hz = sx / 2, sz / 2
    local = [  # (origin, eu, ev) with eu x ev outward
        ((-hx, 0, -hz), (0, sy, 0), (2 * hx, 0, 0)),  # -z face
        ((-hx, 0, hz), (2 * hx, 0, 0), (0, sy, 0)),  # +z
        ((-hx, 0, -hz), (0, 0, 2 * hz), (0, sy, 0)),  # -x
        ((hx, 0, -hz), (0, sy, 0), (0, 0, 2 * hz)),  # +x
        ((-hx, sy, -hz), (0, 0, 2 * hz), (2 * hx, 0, 0)),  # top
        ((-hx, 0, -hz), (2 * hx, 0, 0), (0, 0, 2 * hz)),  # bottom
    ]
    out = []
    for o, eu, ev in local:
        o = R @ np.asarray(o, float) + np.array([cx, 0.0, cz])
        out.append(_quad_grid(o, R @ np.asarray(eu, float), R @ np.asarray(ev, float), n))
    return out


def room(grid: int = 53, light_grid: int = 4, boxes=None, wall_albedo=WHITE, light_size: float = 0.5,
         light_radiance=(17.0, 12.0, 4.0)) -> Mesh:
    if boxes is None:
        boxes = [((-0.35, -0.3), (0.55, 1.1, 0.55), 20.0, WHITE), ((0.4, 0.35), (0.55, 0.55, 0.55), -18.0, WHITE)]
    parts, cols, emit = [], [], []

    def add(tris, col, e=0):
        parts.append(tris)
        cols.append(np.tile(np.asarray(col, np.float64), (tris.shape[0], 1)))
        emit.append(np.full(tris.shape[0], e, np.uint8))

    # inward-facing walls (eu x ev points into the room)
    add(_quad_grid((-1, 0, -1), (0, 0, 2), (2, 0, 0), grid), wall_albedo)  # floor, normal +y
    add(_quad_grid((-1, 2, -1), (2, 0, 0), (0, 0, 2), grid), wall_albedo)  # ceiling, normal -y
    add(_quad_grid((-1, 0, -1), (2, 0, 0), (0, 2, 0), grid), wall_albedo)  # back z=-1, normal +z
    add(_quad_grid((-1, 0, 1), (0, 2, 0), (2, 0, 0), grid), wall_albedo)  # front z=+1, normal -z
    add(_quad_grid((-1, 0, -1), (0, 2, 0), (0, 0, 2), grid), RED)  # left x=-1, normal +x
    add(_quad_grid((1, 0, -1), (0, 0, 2), (0, 2, 0), grid), GREEN)  # right x=+1, normal -x
    h = light_size / 2
    add(_quad_grid((-h, 1.999, -h), (2 * h, 0, 0), (0, 0, 2 * h), light_grid), light_radiance, 1)  # normal -y
    for center, size, ang, col in boxes:
        for f in _box_faces(center, size, ang, grid):
            add(f, col)
    verts = np.concatenate(parts).astype(np.float32)
    return Mesh(verts, np.concatenate(cols).astype(np.float32), np.concatenate(emit))


def room_setup(width: int = 1024, height: int = 1024, spp: int = 64, max_depth: int = 8) -> RenderSetup:
    return RenderSetup(width=width, height=height, fov=60, cam_pos=(0.0, 1.0, 0.98), cam_look=(0.0, 0.0, -1.0),
                       lights=[], tree="sah", leaf_size=32, max_depth=20, sah_ct=1.0, sah_ci=1.5, det_eps=0.0,
                       method="path_tracing", max_depth_pt=max_depth, num_samples=spp)


def random_room(seed: int, grid: int = 16) -> Mesh:
    """Procedural room: 1-6 random boxes, wall albedo U[0.1,0.9]^3, light size
    U[0.3,0.8]."""
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(1, 7))
    boxes = []
    for _ in range(nb):
        c = tuple(rng.uniform(-0.6, 0.6, 2))
        s = (float(rng.uniform(0.2, 0.6)), float(rng.uniform(0.2, 1.2)), float(rng.uniform(0.2, 0.6)))
        boxes.append((c, s, float(rng.uniform(-45, 45)), tuple(rng.uniform(0.1, 0.9, 3))))
    return room(grid=grid, boxes=boxes, wall_albedo=tuple(rng.uniform(0.1, 0.9, 3)),
                light_size=float(rng.uniform(0.3, 0.8)))


# --------------------------------------------------------------------------
# Batched workload: n independent scenes, each a displaced icosphere or a
# triangle soup with a lognormal triangle count (median 40k, clipped to
# [1k, 500k], sigma 1), a square resolution from {256, 512, 768, 1024}, a
# random camera on a sphere of radius 3 looking at the origin, a sky
# background, 16 spp, depth 6, SAH trees.

def batch_workload(n: int = 64, seed: int = 0, median: int = 40_000, sigma: float = 1.0, lo: int = 1_000,
                   hi: int = 500_000, spp: int = 16, depth: int = 6, resolutions=(256, 512, 768, 1024)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        count = int(np.clip(np.exp(rng.normal(np.log(median), sigma)), lo, hi))
        sphere = bool(rng.random() < 0.5)
        res = int(resolutions[int(rng.integers(len(resolutions)))])
        az, el = rng.uniform(0, 2 * np.pi), rng.uniform(-1.0, 1.0)
        pos = 3.0 * np.array([np.cos(el) * np.cos(az), np.sin(el), np.cos(el) * np.sin(az)])
        albedo = tuple(float(x) for x in rng.uniform(0.3, 0.9, 3))
        if sphere:
            level = int(np.clip(round(np.log(count / 20.0) / np.log(4.0)), 2, 7))
            mesh = icosphere(level, seed=seed * 1000 + i, albedo=albedo)
        else:
            mesh = soup(count, seed * 1000 + i)
            mesh.verts = (mesh.verts * 2.0 - 1.0).astype(np.float32)
            mesh.colors[:] = np.asarray(albedo, np.float32)
        setup = RenderSetup(width=res, height=res, fov=45, cam_pos=tuple(float(x) for x in pos),
                            cam_look=tuple(float(x) for x in -pos), lights=[], background=(0.7, 0.8, 1.0),
                            tree="sah", leaf_size=32, max_depth=20, sah_ct=1.0, sah_ci=1.5, det_eps=0.0,
                            method="path_tracing", max_depth_pt=depth, num_samples=spp)
        out.append((mesh, setup))
    return out
