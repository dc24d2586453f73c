"""ORACLE — test infrastructure, not product code.

ctypes front ends for
  * ``OracleScene``: the CPU restatement in ``pray_oracle.cpp`` (built by
    ``build()`` into ``oracle/_build/liboracle.so``), and
  * ``ReferenceScene``: the reference's own scalar tracer compiled from its
    sources by ``build_ref.sh`` into ``oracle/_ref/`` (present only where the
    reference sources were available when it was built).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD_DIR, "liboracle.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64


def build(verbose: bool = False) -> str:
    """Compiles pray_oracle.cpp (no FMA contraction, OpenMP) if stale."""
    srcs = [os.path.join(HERE, "pray_oracle.cpp"), os.path.join(HERE, "denoise_oracle.cpp")]
    deps = srcs + [os.path.join(os.path.dirname(HERE), "include", "nostrum_pray_sampling.h")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(d) for d in deps):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
               *srcs, "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True, capture_output=not verbose)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_scene_new.restype = _vp
        L.orc_scene_new.argtypes = [_f32p, _f32p, _u8p, _u64]
        L.orc_scene_free.argtypes = [_vp]
        L.orc_scene_build.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                      ctypes.c_float]
        L.orc_triangle_precompute.argtypes = [_vp, _f32p]
        L.orc_tree_stats.argtypes = [_vp, _u64p]
        L.orc_tree_dump.argtypes = [_vp, _f32p, _f32p, _i32p, _i64p]
        L.orc_primary_rays.argtypes = [_u64, _u64, _u64, _f32p, _f32p, _f32p]
        L.orc_camera.argtypes = [_u64, _u64, _u64, _f32p, _f32p, _f32p]
        L.orc_trace.argtypes = [_vp, _f32p, _u64, ctypes.c_float, _i64p, _f32p, ctypes.c_int]
        L.orc_last_threads.restype = ctypes.c_int
        L.orc_last_threads.argtypes = []
        L.orc_render_rt.restype = _u64
        L.orc_render_rt.argtypes = [_vp, _u64, _u64, _u64, _f32p, _f32p, _f32p, ctypes.c_int, _f32p,
                                    ctypes.c_float, _u64, _u64, _u8p, ctypes.c_int]
        L.orc_sincos_turns.argtypes = [_f32p, _u64, _f32p, _f32p]
        L.orc_unet_num_params.restype = _u64
        L.orc_unet.restype = ctypes.c_double
        L.orc_unet.argtypes = [_f32p, _f32p, np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS"), _f32p,
                               ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, _f64p]
        L.orc_sample_hemisphere.argtypes = [_f32p, _f32p, _u64, _f32p]
        L.orc_render_pt.restype = _u64
        L.orc_render_pt.argtypes = [_vp, _u64, _u64, _u64, _f32p, _f32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                    _u64, ctypes.c_float, ctypes.c_int, ctypes.c_uint32, _u64, _u64, _u8p,
                                    _vp, ctypes.c_int, ctypes.c_uint32, _vp]
        _lib = L
    return _lib


def _f3(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, np.float32).reshape(-1))


def last_threads() -> int:
    """Threads that OpenMP ran the most recent frame loop (render_rt /
    render_pt) with."""
    return int(lib().orc_last_threads())


def default_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def primary_rays(width, height, fov, cam_pos, cam_look) -> np.ndarray:
    out = np.empty((width * height, 9), np.float32)
    lib().orc_primary_rays(width, height, fov, _f3(cam_pos), _f3(cam_look), out)
    return out


def camera(width, height, fov, cam_pos, cam_look) -> np.ndarray:
    out = np.empty(13, np.float32)
    lib().orc_camera(width, height, fov, _f3(cam_pos), _f3(cam_look), out)
    return out


def unet(params, rad, feat_f16, target):
    """FP64 U-Net forward + L1 loss + backward: (loss, output, grads)."""
    n, h, w, _ = rad.shape
    out = np.empty((n, h, w, 3), np.float64)
    g = np.empty(int(lib().orc_unet_num_params()), np.float64)
    loss = lib().orc_unet(np.ascontiguousarray(params, np.float32), np.ascontiguousarray(rad, np.float32),
                          np.ascontiguousarray(feat_f16).view(np.uint16), np.ascontiguousarray(target, np.float32),
                          n, h, w, out, g)
    return loss, out, g


def sincos_turns(u: np.ndarray):
    u = np.ascontiguousarray(u, np.float32)
    s = np.empty_like(u)
    c = np.empty_like(u)
    lib().orc_sincos_turns(u, u.size, s, c)
    return s, c


def sample_hemisphere(normals: np.ndarray, u: np.ndarray) -> np.ndarray:
    normals = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
    out = np.empty_like(normals)
    lib().orc_sample_hemisphere(normals, u, normals.shape[0], out)
    return out


class _TreeDumpMixin:
    def tree_dump(self):
        st = self.tree_stats()
        nn, nref = int(st[0]), int(st[4])
        boxes = np.empty((nn, 6), np.float32)
        split = np.empty(nn, np.float32)
        info = np.empty((nn, 4), np.int32)
        refs = np.empty(max(nref, 1), np.int64)
        self._dump(boxes, split, info, refs)
        return {"boxes": boxes, "split": split, "info": info, "refs": refs[:nref]}


class OracleScene(_TreeDumpMixin):
    """Triangles + tree (median or SAH) in the oracle."""

    def __init__(self, mesh, tree: str = "median", leaf_size: int = 32, max_depth: int = 20,
                 sah_ct: float = 5.0, sah_ci: float = 1.5):
        L = lib()
        self._h = L.orc_scene_new(mesh.verts, mesh.colors, mesh.emit, mesh.n)
        L.orc_scene_build(self._h, 1 if tree == "sah" else 0, leaf_size, max_depth, sah_ct, sah_ci)
        self.n = mesh.n

    @classmethod
    def from_setup(cls, mesh, setup):
        return cls(mesh, setup.tree, setup.leaf_size, setup.max_depth, setup.sah_ct, setup.sah_ci)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_scene_free(self._h)
            self._h = None

    def precompute(self) -> np.ndarray:
        out = np.empty((self.n, 18), np.float32)
        lib().orc_triangle_precompute(self._h, out)
        return out

    def tree_stats(self) -> np.ndarray:
        out = np.zeros(5, np.uint64)
        lib().orc_tree_stats(self._h, out)
        return out

    def _dump(self, boxes, split, info, refs):
        lib().orc_tree_dump(self._h, boxes, split, info, refs)

    def trace(self, rays: np.ndarray, det_eps: float = 1e-4, threads: Optional[int] = None):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 9)
        n = rays.shape[0]
        ids = np.empty(n, np.int64)
        ts = np.empty(n, np.float32)
        lib().orc_trace(self._h, rays, n, det_eps, ids, ts, threads or default_threads())
        return ids, ts

    def render_rt(self, setup, rows: Optional[Sequence[int]] = None, threads: Optional[int] = None):
        """Returns (rgb uint8 (rows, width, 3), shadow rays cast)."""
        r0, r1 = (0, setup.height) if rows is None else rows
        out = np.empty((r1 - r0, setup.width, 3), np.uint8)
        lights = setup.lights_array()
        nsh = lib().orc_render_rt(self._h, setup.width, setup.height, setup.fov, _f3(setup.cam_pos),
                                  _f3(setup.cam_look), np.ascontiguousarray(lights.reshape(-1)),
                                  lights.shape[0], _f3(setup.background), setup.det_eps, r0, r1, out,
                                  threads or default_threads())
        return out, int(nsh)

    def render_pt(self, setup, spp: int, max_depth: int, seed: int = 0, mode: int = 0, rr_depth: int = 3,
                  rows: Optional[Sequence[int]] = None, threads: Optional[int] = None, sample_offset: int = 0,
                  sum64: Optional[np.ndarray] = None):
        """Returns (rgb uint8 (rows, width, 3), mean radiance float32, segments).
        sum64 (rows, width, 3) float64, if given, is added to in sample order."""
        r0, r1 = (0, setup.height) if rows is None else rows
        out = np.empty((r1 - r0, setup.width, 3), np.uint8)
        rad = np.empty((r1 - r0, setup.width, 3), np.float32)
        if sum64 is not None:
            assert sum64.dtype == np.float64 and sum64.flags.c_contiguous
        segs = lib().orc_render_pt(self._h, setup.width, setup.height, setup.fov, _f3(setup.cam_pos),
                                   _f3(setup.cam_look), _f3(setup.background), max_depth, spp, seed,
                                   setup.det_eps, mode, rr_depth, r0, r1, out, rad.ctypes.data,
                                   threads or default_threads(), sample_offset,
                                   None if sum64 is None else sum64.ctypes.data)
        return out, rad, int(segs)


# --------------------------------------------------------------------------
# The reference built from source (only where oracle/_ref was built).

REF_VARIANTS = {
    (32, 20, 5.0, 1e-4): "default",
    (8, 24, 5.0, 1e-4): "leaf8",
    (32, 20, 1.0, 1e-4): "sahct1",
    (32, 20, 1.0, 0.0): "sahct1_eps0",
    (8, 24, 5.0, 0.0): "leaf8_eps0",
}

_ref_libs = {}


def ref_variant(setup) -> str:
    key = (setup.leaf_size, setup.max_depth, float(setup.sah_ct), float(np.float32(setup.det_eps)))
    for k, v in REF_VARIANTS.items():
        if (k[0], k[1], k[2]) == key[:3] and np.float32(k[3]) == np.float32(setup.det_eps):
            return v
    raise KeyError(f"no reference build for constants {key}")


def ref_available(variant: str = "default") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libprayref_{variant}.so"))


def ref_lib(variant: str):
    if variant not in _ref_libs:
        path = os.path.join(REF_DIR, f"libprayref_{variant}.so")
        L = ctypes.CDLL(path)
        L.ref_constants.argtypes = [_f64p]
        L.ref_scene_from_tris.restype = _vp
        L.ref_scene_from_tris.argtypes = [_f32p, _f32p, _u8p, ctypes.c_size_t]
        L.ref_scene_from_json.restype = _vp
        L.ref_scene_from_json.argtypes = [ctypes.c_char_p]
        L.ref_scene_info.argtypes = [_vp, _f64p]
        L.ref_scene_get.argtypes = [_vp, _f32p, _f32p, _u8p, _f32p]
        L.ref_triangle_precompute.argtypes = [_vp, _f32p]
        L.ref_scene_prepare.argtypes = [_vp, ctypes.c_int]
        L.ref_scene_free.argtypes = [_vp]
        L.ref_tree_stats.argtypes = [_vp, _u64p]
        L.ref_tree_dump.argtypes = [_vp, _f32p, _f32p, _i32p, _i64p]
        L.ref_primary_rays.argtypes = [_u64, _u64, _u64, _f32p, _f32p, _f32p]
        L.ref_trace.argtypes = [_vp, _f32p, ctypes.c_size_t, _i64p, _f32p]
        L.ref_render_rt.argtypes = [_vp, _u64, _u64, _u64, _f32p, _f32p, _f32p, ctypes.c_int, _f32p, _u8p]
        L.ref_gpu_tree_size.argtypes = [_vp, _u64p, _u64p]
        L.ref_gpu_tree.argtypes = [_vp, _i32p, _i32p, _u8p, _u64p, _u64p, _f32p, _u8p, _f32p, _i32p, _u64p]
        L.ref_path_moments.argtypes = [_vp, _u64, _u64, _u64, _f32p, _f32p, _f32p, _u64, _u64, ctypes.c_int, _u64,
                                       _f64p, _f64p]
        _ref_libs[variant] = L
    return _ref_libs[variant]


class ReferenceScene(_TreeDumpMixin):
    """The reference's Scene + KDTree/KDTreeSAH, built by its own code."""

    def __init__(self, mesh, tree: str = "median", variant: str = "default"):
        self.L = ref_lib(variant)
        self._h = self.L.ref_scene_from_tris(mesh.verts, mesh.colors, mesh.emit, mesh.n)
        self.L.ref_scene_prepare(self._h, 1 if tree == "sah" else 0)
        self.n = mesh.n

    @classmethod
    def from_setup(cls, mesh, setup):
        return cls(mesh, setup.tree, ref_variant(setup))

    def __del__(self):
        if getattr(self, "_h", None):
            self.L.ref_scene_free(self._h)
            self._h = None

    def precompute(self) -> np.ndarray:
        out = np.empty((self.n, 18), np.float32)
        self.L.ref_triangle_precompute(self._h, out)
        return out

    def tree_stats(self) -> np.ndarray:
        out = np.zeros(5, np.uint64)
        self.L.ref_tree_stats(self._h, out)
        return out

    def _dump(self, boxes, split, info, refs):
        self.L.ref_tree_dump(self._h, boxes, split, info, refs)

    def trace(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 9)
        n = rays.shape[0]
        ids = np.empty(n, np.int64)
        ts = np.empty(n, np.float32)
        self.L.ref_trace(self._h, rays, n, ids, ts)
        return ids, ts

    def render_rt(self, setup) -> np.ndarray:
        out = np.empty((setup.height, setup.width, 3), np.uint8)
        lights = setup.lights_array()
        self.L.ref_render_rt(self._h, setup.width, setup.height, setup.fov, _f3(setup.cam_pos),
                             _f3(setup.cam_look), np.ascontiguousarray(lights.reshape(-1)), lights.shape[0],
                             _f3(setup.background), out)
        return out

    def gpu_tree(self):
        """The reference's breadth-first GPU tree (buildGPUTreeFromKDTree) as
        a dict of per-node fields and the leaf index array. Consumes the
        scene: the reference moves the triangles out of its tree."""
        nn, ni = np.zeros(1, np.uint64), np.zeros(1, np.uint64)
        self.L.ref_gpu_tree_size(self._h, nn, ni)
        n, m = int(nn[0]), int(ni[0])
        out = {"left": np.empty(n, np.int32), "right": np.empty(n, np.int32), "is_leaf": np.empty(n, np.uint8),
               "first": np.empty(n, np.uint64), "count": np.empty(n, np.uint64),
               "box": np.empty((n, 6), np.float32), "axis": np.empty(n, np.uint8), "split": np.empty(n, np.float32),
               "ropes": np.empty((n, 6), np.int32)}
        idx = np.empty(max(m, 1), np.uint64)
        self.L.ref_gpu_tree(self._h, out["left"], out["right"], out["is_leaf"], out["first"], out["count"], out["box"],
                            out["axis"], out["split"], out["ropes"], idx)
        return out, idx[:m]

    def path_moments(self, setup, max_depth: int, runs: int, diffuse: bool = False, branching: int = 1):
        """Per-pixel (sum, sum of squares) float64 (height, width, 3) of `runs`
        calls of the reference's own unclamped path estimator per pixel
        (evaluatePathRecursive, or evaluatePathRecursiveDiffuse with
        `branching` rays per hit)."""
        s = np.empty((setup.height, setup.width, 3), np.float64)
        q = np.empty_like(s)
        self.L.ref_path_moments(self._h, setup.width, setup.height, setup.fov, _f3(setup.cam_pos),
                                _f3(setup.cam_look), _f3(setup.background), max_depth, branching,
                                1 if diffuse else 0, runs, s, q)
        return s, q


def ref_primary_rays(width, height, fov, cam_pos, cam_look, variant: str = "default") -> np.ndarray:
    out = np.empty((width * height, 9), np.float32)
    ref_lib(variant).ref_primary_rays(width, height, fov, _f3(cam_pos), _f3(cam_look), out)
    return out
