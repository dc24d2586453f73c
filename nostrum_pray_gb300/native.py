"""ctypes binding of the C ABI (include/nostrum_pray.h) and a small Python
front end in the reference's vocabulary: a ``Scene`` holds the device-resident
tree (``SpatialDatabase`` + ``Scene`` of include/spatial.h / include/pray.h),
``render_rt`` / ``render_pt`` produce the ``Image`` of ``render``
(include/pray.h:50), and ``trace_closest`` is the batched
``SpatialDatabase::intersect``.

The native library is required: importing works without it, but every call
raises if ``libnostrum_pray.so`` has not been built (there is no CPU
fallback)."""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence, Tuple

import numpy as np

from . import scenes as _scenes

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libnostrum_pray.so")
CLI_PATH = os.path.join(_PKG, "_build", "Pray")

PRAY_OK = 0
TREE_MEDIAN, TREE_SAH = 0, 1
PT_KAJIYA, PT_NEE, PT_DIFFUSE = 0, 1, 2
TRAVERSAL_AUTO, TRAVERSAL_LANES, TRAVERSAL_PACKETS, TRAVERSAL_PRIMARY_PACKETS = -1, 0, 1, 2
SCHED_PIXEL, SCHED_WAVEFRONT, SCHED_AUTO = 0, 1, 2

_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_i32 = ctypes.c_int32
_f32 = ctypes.c_float


class TreeOptions(ctypes.Structure):
    _fields_ = [("tree", _i32), ("leaf_size", _i32), ("max_depth", _i32), ("sah_traversal_cost", _f32),
                ("sah_intersection_cost", _f32), ("build_threads", _i32), ("leaf_refine", _i32)]


class RtParams(ctypes.Structure):
    _fields_ = [("width", _u64), ("height", _u64), ("fov", _u64), ("camera_position", _f32 * 3),
                ("camera_look", _f32 * 3), ("background", _f32 * 3), ("lights", ctypes.POINTER(_f32)),
                ("n_lights", _i32), ("det_epsilon", _f32)]


class PtParams(ctypes.Structure):
    _fields_ = [("width", _u64), ("height", _u64), ("fov", _u64), ("camera_position", _f32 * 3),
                ("camera_look", _f32 * 3), ("background", _f32 * 3), ("max_depth", ctypes.c_uint32),
                ("num_samples", ctypes.c_uint32), ("seed", _u64), ("det_epsilon", _f32), ("mode", _i32),
                ("rr_depth", ctypes.c_uint32), ("scheduler", _i32), ("sample_offset", ctypes.c_uint32),
                ("wavefront_paths", ctypes.c_uint32)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("tile_w", _i32), ("tile_h", _i32), ("block_threads", _i32), ("blocks_per_sm", _i32),
                ("stack_entries", _i32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PrayError(RuntimeError):
    pass


_lib = None

# every symbol include/nostrum_pray.h declares
EXPORTED = [
    "pray_last_error", "pray_api_version", "pray_tree_options_default", "pray_host_tree_build",
    "pray_host_tree_destroy", "pray_host_tree_stats", "pray_host_tree_dump", "pray_host_tree_precompute",
    "pray_host_tree_device_layout",
    "pray_camera", "pray_scene_create", "pray_scene_destroy", "pray_scene_stats", "pray_scene_set_traversal",
    "pray_scene_traversal", "pray_trace_closest", "pray_trace_closest_host", "pray_trace_occluded",
    "pray_render_rt", "pray_render_rt_host", "pray_render_rt_counts", "pray_render_pt", "pray_render_pt_host",
    "pray_accumulate_pt", "pray_relmse", "pray_render_pt_noalloc",
    "pray_batch_create", "pray_batch_destroy", "pray_batch_set_config", "pray_batch_tune", "pray_batch_render",
    "pray_render_features", "pray_denoiser_create", "pray_denoiser_destroy", "pray_denoiser_num_params",
    "pray_denoiser_get_params", "pray_denoiser_set_params", "pray_denoise", "pray_denoiser_train_step",
    "pray_denoiser_gradients", "pray_denoiser_set_tensor_cores", "pray_denoiser_check",
]


def lib():
    """Loads the native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PrayError(f"native library missing: {LIB_PATH} (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        L.pray_last_error.restype = ctypes.c_char_p
        L.pray_api_version.restype = _i32
        L.pray_tree_options_default.argtypes = [ctypes.POINTER(TreeOptions)]
        L.pray_host_tree_build.argtypes = [_vp, _u64, ctypes.POINTER(TreeOptions), ctypes.POINTER(_vp)]
        L.pray_host_tree_destroy.argtypes = [_vp]
        L.pray_host_tree_stats.argtypes = [_vp, _vp]
        L.pray_host_tree_dump.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.pray_host_tree_precompute.argtypes = [_vp, _vp]
        L.pray_host_tree_device_layout.argtypes = [_vp, _i32, _vp]
        L.pray_camera.argtypes = [_u64, _u64, _u64, _vp, _vp, _vp]
        L.pray_scene_create.argtypes = [_vp, _vp, _vp, _u64, ctypes.POINTER(TreeOptions), _i32, ctypes.POINTER(_vp)]
        L.pray_scene_destroy.argtypes = [_vp]
        L.pray_scene_stats.argtypes = [_vp, _vp]
        L.pray_scene_set_traversal.argtypes = [_vp, _i32]
        L.pray_scene_traversal.argtypes = [_vp, ctypes.POINTER(_i32)]
        L.pray_trace_closest.argtypes = [_vp, _vp, _u64, _f32, _vp, _vp, _vp]
        L.pray_trace_occluded.argtypes = [_vp, _vp, _vp, _u64, _f32, _vp, _vp]
        L.pray_trace_closest_host.argtypes = [_vp, _vp, _u64, _f32, _vp, _vp]
        L.pray_render_rt.argtypes = [_vp, ctypes.POINTER(RtParams), _vp, _vp, _vp, _vp, _vp]
        L.pray_render_rt_host.argtypes = [_vp, ctypes.POINTER(RtParams), _vp, _vp]
        L.pray_render_rt_counts.argtypes = [_vp, ctypes.POINTER(RtParams), _vp]
        L.pray_render_pt.argtypes = [_vp, ctypes.POINTER(PtParams), _vp, _vp, _vp, _vp]
        L.pray_render_pt_host.argtypes = [_vp, ctypes.POINTER(PtParams), _vp, _vp, _vp]
        L.pray_accumulate_pt.argtypes = [_vp, ctypes.POINTER(PtParams), _vp, _vp, _vp]
        L.pray_render_pt_noalloc.argtypes = [_vp, ctypes.POINTER(PtParams), _vp, _vp, _vp, _vp]
        L.pray_batch_create.argtypes = [_vp, ctypes.POINTER(PtParams), _vp, _vp, _i32, ctypes.POINTER(_vp)]
        L.pray_batch_destroy.argtypes = [_vp]
        L.pray_batch_set_config.argtypes = [_vp, ctypes.POINTER(BatchConfig)]
        L.pray_batch_tune.argtypes = [_vp, ctypes.POINTER(BatchConfig), ctypes.POINTER(_f32)]
        L.pray_batch_render.argtypes = [_vp, _vp, _vp]
        L.pray_render_features.argtypes = [_vp, ctypes.POINTER(PtParams), _vp, _vp]
        L.pray_denoiser_create.argtypes = [_i32, _u64, ctypes.POINTER(_vp)]
        L.pray_denoiser_destroy.argtypes = [_vp]
        L.pray_denoiser_num_params.argtypes = [_vp, ctypes.POINTER(_u64)]
        L.pray_denoiser_get_params.argtypes = [_vp, _vp]
        L.pray_denoiser_set_params.argtypes = [_vp, _vp]
        L.pray_denoise.argtypes = [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp]
        L.pray_denoiser_train_step.argtypes = [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _f32, _vp, _vp]
        L.pray_denoiser_set_tensor_cores.argtypes = [_vp, _i32]
        L.pray_denoiser_check.argtypes = [_vp]
        L.pray_denoiser_gradients.argtypes = [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp]
        L.pray_relmse.argtypes = [_vp, ctypes.c_double, _vp, ctypes.c_double, _u64, _vp, _vp]
        for name in EXPORTED:
            if not hasattr(L, name):
                raise PrayError(f"{LIB_PATH} does not export {name}")
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != PRAY_OK:
        raise PrayError(f"pray status {status}: {lib().pray_last_error().decode(errors='replace')}")


def _ptr(a) -> Optional[int]:
    """Address of a numpy array or a torch tensor (None stays None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def tree_options(setup=None, **kw) -> TreeOptions:
    o = TreeOptions()
    lib().pray_tree_options_default(ctypes.byref(o))
    if setup is not None:
        o.tree = TREE_SAH if setup.tree == "sah" else TREE_MEDIAN
        o.leaf_size, o.max_depth = setup.leaf_size, setup.max_depth
        o.sah_traversal_cost, o.sah_intersection_cost = setup.sah_ct, setup.sah_ci
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def rt_params(setup) -> Tuple[RtParams, np.ndarray]:
    lights = np.ascontiguousarray(setup.lights_array().reshape(-1))
    p = RtParams()
    p.width, p.height, p.fov = setup.width, setup.height, setup.fov
    p.camera_position[:] = list(setup.cam_pos)
    p.camera_look[:] = list(setup.cam_look)
    p.background[:] = list(setup.background)
    p.lights = lights.ctypes.data_as(ctypes.POINTER(_f32))
    p.n_lights = lights.size // 6
    p.det_epsilon = setup.det_eps
    return p, lights  # keep `lights` alive while p is used


def pt_params(setup, spp: Optional[int] = None, max_depth: Optional[int] = None, seed: int = 0,
              mode: int = PT_KAJIYA, rr_depth: int = 3, scheduler: int = SCHED_PIXEL,
              sample_offset: int = 0, wavefront_paths: int = 0) -> PtParams:
    p = PtParams()
    p.width, p.height, p.fov = setup.width, setup.height, setup.fov
    p.camera_position[:] = list(setup.cam_pos)
    p.camera_look[:] = list(setup.cam_look)
    p.background[:] = list(setup.background)
    p.max_depth = setup.max_depth_pt if max_depth is None else max_depth
    p.num_samples = setup.num_samples if spp is None else spp
    p.seed, p.det_epsilon, p.mode, p.rr_depth = seed, setup.det_eps, mode, rr_depth
    p.scheduler, p.sample_offset, p.wavefront_paths = scheduler, sample_offset, wavefront_paths
    return p


def relmse(img_sum, img_scale: float, ref_sum, ref_scale: float, out, stream=None) -> None:
    """FP64 relMSE of two device FP64 images (sums scaled to means) into out[0]."""
    check(lib().pray_relmse(_ptr(img_sum), img_scale, _ptr(ref_sum), ref_scale, img_sum.numel(), _ptr(out),
                            _stream(stream)))


def camera(width, height, fov, cam_pos, cam_look) -> np.ndarray:
    out = np.empty(13, np.float32)
    pos = np.asarray(cam_pos, np.float32)
    look = np.asarray(cam_look, np.float32)
    check(lib().pray_camera(width, height, fov, pos.ctypes.data, look.ctypes.data, out.ctypes.data))
    return out


class HostTree:
    """Tree built on the host only (no GPU needed)."""

    def __init__(self, mesh: _scenes.Mesh, options: TreeOptions):
        h = _vp()
        check(lib().pray_host_tree_build(mesh.verts.ctypes.data, mesh.n, ctypes.byref(options), ctypes.byref(h)))
        self._h = h
        self.n = mesh.n

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pray_host_tree_destroy(self._h)
            self._h = None

    def tree_stats(self) -> np.ndarray:
        out = np.zeros(5, np.uint64)
        check(lib().pray_host_tree_stats(self._h, out.ctypes.data))
        return out

    def tree_dump(self):
        st = self.tree_stats()
        nn, nref = int(st[0]), int(st[4])
        boxes = np.empty((nn, 6), np.float32)
        split = np.empty(nn, np.float32)
        info = np.empty((nn, 4), np.int32)
        refs = np.empty(max(nref, 1), np.int64)
        check(lib().pray_host_tree_dump(self._h, boxes.ctypes.data, split.ctypes.data, info.ctypes.data,
                                        refs.ctypes.data))
        return {"boxes": boxes, "split": split, "info": info, "refs": refs[:nref]}

    def precompute(self) -> np.ndarray:
        out = np.empty((self.n, 18), np.float32)
        check(lib().pray_host_tree_precompute(self._h, out.ctypes.data))
        return out

    def device_layout(self, leaf_refine: int = 4) -> np.ndarray:
        """[node records, triangle references, refined leaves, added nodes]."""
        out = np.zeros(4, np.uint64)
        check(lib().pray_host_tree_device_layout(self._h, leaf_refine, out.ctypes.data))
        return out


class Scene:
    """Device-resident scene: triangles, tree and shading data on one GPU."""

    def __init__(self, mesh: _scenes.Mesh, options: TreeOptions, device: int = 0):
        h = _vp()
        check(lib().pray_scene_create(mesh.verts.ctypes.data, mesh.colors.ctypes.data, mesh.emit.ctypes.data,
                                      mesh.n, ctypes.byref(options), device, ctypes.byref(h)))
        self._h = h
        self.n = mesh.n
        self.device = device

    @classmethod
    def from_setup(cls, mesh, setup, device: int = 0, **kw):
        return cls(mesh, tree_options(setup, **kw), device)

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pray_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def stats(self) -> np.ndarray:
        out = np.zeros(8, np.uint64)
        check(lib().pray_scene_stats(self._h, out.ctypes.data))
        return out

    def set_traversal(self, traversal: int) -> None:
        """TRAVERSAL_AUTO, _LANES, _PACKETS or _PRIMARY_PACKETS (ray-traced frames)."""
        check(lib().pray_scene_set_traversal(self._h, traversal))

    def traversal(self) -> int:
        out = _i32(0)
        check(lib().pray_scene_traversal(self._h, ctypes.byref(out)))
        return int(out.value)

    # -- device-pointer entry points (torch CUDA tensors) --------------------
    def trace_closest(self, rays, det_eps: float, ids, ts, stream=None) -> None:
        n = rays.numel() // 9
        check(lib().pray_trace_closest(self._h, _ptr(rays), n, det_eps, _ptr(ids), _ptr(ts), _stream(stream)))

    def trace_occluded(self, rays, dist2, det_eps: float, occluded, stream=None) -> None:
        """occluded (uint8, n): 1 iff a triangle is hit at t > 0 with t^2 < dist2."""
        n = rays.numel() // 9
        check(lib().pray_trace_occluded(self._h, _ptr(rays), _ptr(dist2), n, det_eps, _ptr(occluded),
                                        _stream(stream)))

    def trace_closest_host(self, rays: np.ndarray, det_eps: float) -> Tuple[np.ndarray, np.ndarray]:
        """Closest hits of host rays (n x 9 float32): (ids int32, distances float32)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 9)
        n = rays.shape[0]
        ids = np.empty(n, np.int32)
        ts = np.empty(n, np.float32)
        check(lib().pray_trace_closest_host(self._h, rays.ctypes.data, n, det_eps, ids.ctypes.data, ts.ctypes.data))
        return ids, ts

    def render_rt(self, setup, rgb, ids=None, ts=None, counters=None, stream=None) -> None:
        p, keep = rt_params(setup)
        check(lib().pray_render_rt(self._h, ctypes.byref(p), _ptr(rgb), _ptr(ids), _ptr(ts), _ptr(counters),
                                   _stream(stream)))
        del keep

    def render_pt_noalloc(self, params: PtParams, rgb=None, radiance=None, counters=None, stream=None) -> None:
        """Allocation-free wavefront frame (static device scratch; see
        pray_render_pt_noalloc in include/nostrum_pray.h)."""
        check(lib().pray_render_pt_noalloc(self._h, ctypes.byref(params), _ptr(rgb), _ptr(radiance), _ptr(counters),
                                           _stream(stream)))

    def render_features(self, params: PtParams, features, stream=None) -> None:
        """First-hit albedo, normal, distance as FP16 (torch.float16 h x w x 7)."""
        check(lib().pray_render_features(self._h, ctypes.byref(params), _ptr(features), _stream(stream)))

    def accumulate_pt(self, params: PtParams, sum64, counters=None, stream=None) -> None:
        check(lib().pray_accumulate_pt(self._h, ctypes.byref(params), _ptr(sum64), _ptr(counters), _stream(stream)))

    def render_pt(self, params: PtParams, rgb, radiance=None, counters=None, stream=None) -> None:
        check(lib().pray_render_pt(self._h, ctypes.byref(params), _ptr(rgb), _ptr(radiance), _ptr(counters),
                                   _stream(stream)))

    # -- host-memory entry points -------------------------------------------
    def render_rt_host(self, setup, out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
        """Returns (image uint8 (height, width, 3), [primary rays, shadow rays]);
        `out`: a C-contiguous uint8 host array of that shape to write the
        image into (a frame loop reuses one, pinned for the fastest copy)."""
        p, keep = rt_params(setup)
        shape = (setup.height, setup.width, 3)
        if out is not None and (out.shape != shape or out.dtype != np.uint8 or not out.flags.c_contiguous):
            raise PrayError(f"out must be a C-contiguous uint8 array of shape {shape}")
        img = np.empty(shape, np.uint8) if out is None else out
        rays = np.zeros(2, np.uint64)
        check(lib().pray_render_rt_host(self._h, ctypes.byref(p), img.ctypes.data, rays.ctypes.data))
        del keep
        return img, rays

    def render_rt_counts(self, setup) -> np.ndarray:
        """[primary rays, occlusion rays, node-pair fetches, triangle fetches,
        shaded hits] of one frame (instrumented run)."""
        p, keep = rt_params(setup)
        out = np.zeros(5, np.uint64)
        check(lib().pray_render_rt_counts(self._h, ctypes.byref(p), out.ctypes.data))
        del keep
        return out

    def render_pt_host(self, params: PtParams, radiance: bool = True, out: Optional[np.ndarray] = None,
                       out_radiance: Optional[np.ndarray] = None):
        """Returns (image uint8, mean radiance float32 or None, [paths, segments]);
        `out` / `out_radiance`: C-contiguous host arrays of shape (height,
        width, 3) to write into (uint8 / float32)."""
        shape = (params.height, params.width, 3)
        for a, dt in ((out, np.uint8), (out_radiance, np.float32)):
            if a is not None and (a.shape != shape or a.dtype != dt or not a.flags.c_contiguous):
                raise PrayError(f"output arrays must be C-contiguous {shape} arrays")
        img = np.empty(shape, np.uint8) if out is None else out
        rad = (np.empty(shape, np.float32) if out_radiance is None else out_radiance) if radiance else None
        rays = np.zeros(2, np.uint64)
        check(lib().pray_render_pt_host(self._h, ctypes.byref(params), img.ctypes.data, _ptr(rad),
                                        rays.ctypes.data))
        return img, rad, rays


def _stream(stream) -> Optional[int]:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available() and torch.cuda.is_initialized():
                return torch.cuda.current_stream().cuda_stream
        except Exception:
            pass
        return None
    return getattr(stream, "cuda_stream", stream)


class Batch:
    """Many scenes, one path-traced frame each, rendered by one persistent
    launch (pray_batch_*). outputs: per scene an (rgb, radiance) pair of torch
    CUDA tensors (either may be None)."""

    def __init__(self, scenes, params, outputs):
        n = len(scenes)
        handles = (_vp * n)(*[sc._h.value for sc in scenes])
        ps = (PtParams * n)(*params)
        rgbs = (_vp * n)(*[_ptr(o[0]) for o in outputs])
        rads = (_vp * n)(*[_ptr(o[1]) for o in outputs])
        h = _vp()
        check(lib().pray_batch_create(handles, ps, rgbs, rads, n, ctypes.byref(h)))
        self._h = h
        self._keep = (scenes, outputs)

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pray_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_config(self, cfg: BatchConfig) -> None:
        check(lib().pray_batch_set_config(self._h, ctypes.byref(cfg)))

    def tune(self):
        cfg = BatchConfig()
        ms = _f32()
        check(lib().pray_batch_tune(self._h, ctypes.byref(cfg), ctypes.byref(ms)))
        return cfg, ms.value

    def render(self, counters=None, stream=None) -> None:
        check(lib().pray_batch_render(self._h, _ptr(counters), _stream(stream)))


class Denoiser:
    """The U-Net denoiser (pray_denoiser_*). Tensors are torch CUDA tensors:
    radiance (n, h, w, 3) float32, features (n, h, w, 7) float16."""

    def __init__(self, seed: int = 0, device: int = 0):
        h = _vp()
        check(lib().pray_denoiser_create(device, seed, ctypes.byref(h)))
        self._h = h
        n = _u64()
        check(lib().pray_denoiser_num_params(self._h, ctypes.byref(n)))
        self.num_params = n.value

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pray_denoiser_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_tensor_cores(self, on: bool) -> None:
        check(lib().pray_denoiser_set_tensor_cores(self._h, 1 if on else 0))

    def check(self) -> None:
        check(lib().pray_denoiser_check(self._h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        check(lib().pray_denoiser_get_params(self._h, out.ctypes.data))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        check(lib().pray_denoiser_set_params(self._h, p.ctypes.data))

    def denoise(self, radiance, features, out, stream=None) -> None:
        n, h, w, _ = radiance.shape
        check(lib().pray_denoise(self._h, _ptr(radiance), _ptr(features), n, h, w, _ptr(out), _stream(stream)))

    def train_step(self, radiance, features, target, lr: float, want_loss: bool = False, stream=None):
        n, h, w, _ = radiance.shape
        loss = np.zeros(1, np.float32)
        check(lib().pray_denoiser_train_step(self._h, _ptr(radiance), _ptr(features), _ptr(target), n, h, w, lr,
                                             loss.ctypes.data if want_loss else None, _stream(stream)))
        return float(loss[0]) if want_loss else None

    def gradients(self, radiance, features, target):
        n, h, w, _ = radiance.shape
        loss = np.zeros(1, np.float32)
        g = np.empty(self.num_params, np.float32)
        check(lib().pray_denoiser_gradients(self._h, _ptr(radiance), _ptr(features), _ptr(target), n, h, w,
                                            loss.ctypes.data, g.ctypes.data))
        return float(loss[0]), g
