"""Writes tests/golden/pt_moments.npz: per-pixel moments of the reference's
own path-tracing estimators, for the statistical parity tests of the path
tracer (tests/test_pt_reference_stats.py, tests/test_pt_stats_gpu.py).

The reference's path tracers draw from a fresh clock-seeded mt19937_64 in
every call (src/pray.cpp:331,357), so no stream can be shared with them; what
can be compared is the estimator's distribution. For every case below this
script calls the reference's evaluatePathRecursive (Kajiya, src/pray.cpp:342-364)
or evaluatePathRecursiveDiffuse (branching, src/pray.cpp:315-340), compiled
from its sources by oracle/build_ref.sh and reached through
oracle/ref_harness.cpp (ref_path_moments), `runs` times per pixel, and stores
per pixel and channel the mean and the unbiased sample variance of the
unclamped value.

Scenes: the closed room of nostrum_pray_gb300.scenes.room(grid=4) (608
triangles, 0.5 x 0.5 emissive quad below the ceiling), the procedural room
scenes.random_room(3, grid=4) (other wall albedo, light size and boxes) and
the reference's
examples/pt_cornell scene as its own loader returned it (the triangles stored
in golden_small.npz under ex_pt_cornell_*), at reduced resolutions with each
scene's own camera.

Usage (needs oracle/_ref built from the reference sources):
    REF_ROOT=<reference checkout> oracle/build_ref.sh && python tests/golden/make_pt_moments.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nostrum_pray_gb300 import scenes  # noqa: E402

# name: scene, width, height, path depth, branching mode, rays per hit, runs per pixel
CASES = {
    "room_kajiya8": ("room", 32, 32, 8, False, 1, 16384),
    "room_diffuse2": ("room", 32, 32, 2, True, 4, 4096),
    "rroom3_kajiya6": ("rroom3", 32, 32, 6, False, 1, 16384),
    "cornell_kajiya4": ("cornell", 40, 30, 4, False, 1, 32768),
    "cornell_diffuse1": ("cornell", 40, 30, 1, True, 16, 8192),
}


def case_scene(name: str, small=None):
    """(mesh, RenderSetup) of a fixture case; `small` is golden_small.npz
    (needed for the Cornell scene)."""
    kind, w, h = CASES[name][:3]
    if kind in ("room", "rroom3"):
        st = scenes.room_setup(w, h, spp=1, max_depth=CASES[name][3])
        return (scenes.room(grid=4) if kind == "room" else scenes.random_room(3, grid=4)), st
    if small is None:
        small = dict(np.load(os.path.join(HERE, "golden_small.npz")))
    info = small["ex_pt_cornell_info"]
    mesh = scenes.Mesh(small["ex_pt_cornell_verts"], small["ex_pt_cornell_colors"], small["ex_pt_cornell_emit"])
    st = scenes.RenderSetup(width=w, height=h, fov=int(info[2]), cam_pos=tuple(float(x) for x in info[6:9]),
                            cam_look=tuple(float(x) for x in info[9:12]), lights=[],
                            background=tuple(float(x) for x in info[12:15]), tree="median",
                            method="path_tracing", max_depth_pt=CASES[name][3], num_samples=1)
    return mesh, st


def main():
    from oracle import oracle as O
    small = dict(np.load(os.path.join(HERE, "golden_small.npz")))
    out = {}
    for name, (kind, w, h, depth, diffuse, branching, runs) in CASES.items():
        mesh, st = case_scene(name, small)
        ref = O.ReferenceScene.from_setup(mesh, st)
        t0 = time.time()
        s, q = ref.path_moments(st, depth, runs, diffuse=diffuse, branching=branching)
        mean = s / runs
        var = np.maximum(q / runs - mean * mean, 0.0) * runs / (runs - 1)
        out[f"{name}_mean"] = mean
        out[f"{name}_var"] = var
        out[f"{name}_runs"] = np.int64(runs)
        print(f"{name}: {mesh.n} triangles, {w}x{h}, {runs} runs in {time.time() - t0:.1f} s, "
              f"image mean {mean.mean((0, 1))}", flush=True)
    np.savez_compressed(os.path.join(HERE, "pt_moments.npz"), **out)


if __name__ == "__main__":
    main()
