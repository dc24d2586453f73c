"""ORACLE — test and baseline infrastructure, not product code.

Runs the reference's own GPU path tracer (src/path_trace.cu, compiled from
the reference's sources into ``oracle/_ref/prayref_path_trace.cubin`` by
``build_ref.sh``) through ``ref_gpu_launch.cpp``, which repeats the host side
of pathTraceOnGPURecursive (src/path_trace.cu:494-555). This module prepares
the reference's device inputs:

* the median kd tree the reference builds for path tracing on the GPU
  (KDTree with its default constants, src/scene_preprocessor.cpp:52-57),
  taken from this library's host builder, whose trees equal the reference's
  (tests/test_native_cpu.py), flattened breadth-first into KDTreeGPUNode
  records as buildGPUTreeFromKDTree does (src/gpu_util.cpp:7-57);
* the triangles with the reference's precomputed fields
  (initialiseTriangles, src/scene_preprocessor.cpp:74-96);
* the primary rays of calculatePrimRays (src/scene_preprocessor.cpp:98-136).

Every index is checked against its array before the launch. Used by the
reference arm of bench.py (``--impl reference --workload cornell``) and by
tests/test_ref_gpu_kernel.py.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "prayref_path_trace.cubin")
LIB = os.path.join(HERE, "_build", "librefgpu.so")

NODE_DTYPE = np.dtype({"names": ["left", "right", "is_leaf", "first", "count", "box", "axis", "split", "ropes"],
                       "formats": ["<i4", "<i4", "u1", "<u8", "<u8", ("<f4", 6), "u1", "<f4", ("<i4", 6)],
                       "offsets": [0, 4, 8, 16, 24, 32, 56, 60, 64], "itemsize": 88})
TRI_DTYPE = np.dtype({"names": ["a", "b", "c", "color", "emit", "normal", "ab", "ac", "mid", "box"],
                      "formats": [("<f4", 3)] * 4 + ["u1"] + [("<f4", 3)] * 4 + [("<f4", 6)],
                      "offsets": [0, 12, 24, 36, 48, 52, 64, 76, 88, 100], "itemsize": 124})


def available() -> bool:
    return os.path.exists(CUBIN)


def build() -> str:
    """Compiles ref_gpu_launch.cpp (CUDA driver API) if stale."""
    src = os.path.join(HERE, "ref_gpu_launch.cpp")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, f"-I{cuda}/include",
               f"-L{cuda}/lib64/stubs", f"-L{cuda}/lib64", "-lcuda", "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True, capture_output=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.refgpu_last_error.restype = ctypes.c_char_p
        L.refgpu_path_trace.restype = ctypes.c_int
        L.refgpu_path_trace.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_float)]
        _lib = L
    return _lib


def gpu_tree(mesh):
    """(nodes KDTreeGPUNode[], triangles Triangle[], indices uint64[]) of the
    reference's median kd tree over `mesh`, breadth-first."""
    from nostrum_pray_gb300 import native
    t = native.HostTree(mesh, native.tree_options(None, tree=native.TREE_MEDIAN))
    d = t.tree_dump()
    boxes, split, info, refs = d["boxes"], d["split"], d["info"], d["refs"]
    n = boxes.shape[0]
    # depth-first pre-order: the left child follows its parent, the right
    # child follows the left subtree
    size = np.ones(n, np.int64)
    right = np.full(n, -1, np.int64)
    for i in range(n - 1, -1, -1):
        if info[i, 0] == 0:
            li = i + 1
            ri = li + size[li]
            right[i] = ri
            size[i] = 1 + size[li] + size[ri]
    nodes = np.zeros(n, NODE_DTYPE)
    idx = []
    order = [0]
    bfs_of = {0: 0}
    head = 0
    while head < len(order):
        i = order[head]
        k = bfs_of[i]
        head += 1
        nodes[k]["box"] = boxes[i]
        nodes[k]["axis"] = info[i, 1] & 0xFF
        nodes[k]["split"] = split[i]
        # ropes stay 0: the reference's rope construction is disabled (src/gpu_util.cpp:55)
        if info[i, 0]:
            nodes[k]["is_leaf"] = 1
            nodes[k]["first"] = len(idx)
            nodes[k]["count"] = info[i, 2]
            idx.extend(int(r) for r in refs[info[i, 3]:info[i, 3] + info[i, 2]])
            nodes[k]["left"] = nodes[k]["right"] = 0
        else:
            for field, c in (("left", i + 1), ("right", int(right[i]))):
                bfs_of[c] = len(order)
                nodes[k][field] = len(order)
                order.append(c)
    pre = t.precompute()  # bbox min, bbox max, midpoint, ab, ac, normal per triangle
    tris = np.zeros(mesh.n, TRI_DTYPE)
    v = mesh.verts.reshape(-1, 3, 3)
    tris["a"], tris["b"], tris["c"] = v[:, 0], v[:, 1], v[:, 2]
    tris["color"] = mesh.colors
    tris["emit"] = mesh.emit != 0
    tris["box"] = pre[:, 0:6]
    tris["mid"] = pre[:, 6:9]
    tris["ab"] = pre[:, 9:12]
    tris["ac"] = pre[:, 12:15]
    tris["normal"] = pre[:, 15:18]
    indices = np.asarray(idx, np.uint64)
    check_tree(nodes, indices, mesh.n)
    return nodes, tris, indices


def check_tree(nodes, indices, n_tris):
    """Every child index, leaf range and triangle index in bounds."""
    n = nodes.shape[0]
    leaf = nodes["is_leaf"] != 0
    inner = ~leaf
    assert n >= 1
    assert ((nodes["left"][inner] > 0) & (nodes["left"][inner] < n)).all()
    assert ((nodes["right"][inner] > 0) & (nodes["right"][inner] < n)).all()
    assert (nodes["first"][leaf] + nodes["count"][leaf] <= indices.size).all()
    assert (indices < n_tris).all() if indices.size else True


def render(mesh, setup, max_depth: int, num_samples: int, diffuse: bool, frames: int = 1, batch: int = 1024):
    """(image uint8 (height, width, 3), device ms of all frames)."""
    from oracle import oracle as O
    assert available(), "reference GPU path tracer not built (oracle/build_ref.sh)"
    nodes, tris, indices = gpu_tree(mesh)
    rays = np.ascontiguousarray(O.primary_rays(setup.width, setup.height, setup.fov, setup.cam_pos, setup.cam_look),
                                np.float32)
    npx = setup.width * setup.height
    assert rays.shape == (npx, 9)
    bg = np.asarray(setup.background, np.float32)
    img = np.empty((setup.height, setup.width, 3), np.uint8)
    ms = ctypes.c_float(0.0)
    rc = lib().refgpu_path_trace(CUBIN.encode(), nodes.ctypes.data, nodes.shape[0], tris.ctypes.data, tris.shape[0],
                                 indices.ctypes.data, indices.size, rays.ctypes.data, npx, bg.ctypes.data, max_depth,
                                 num_samples, 1 if diffuse else 0, batch, frames, img.ctypes.data, ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError(lib().refgpu_last_error().decode())
    return img, float(ms.value)
