"""Writes the golden fixtures in this directory from the reference itself.

Runs the reference's own scene loader, KD-tree builders, scalar intersector and
ray-tracing renderer, compiled from its sources by ``oracle/build_ref.sh``
(``oracle/_ref/libprayref_<variant>.so``), on seeded synthetic scenes and on the
reference's example scenes, and stores what it returns:

* ``golden_small.npz``: full arrays for small cases (tree dumps, per-ray hit
  ids and distances, images, loaded triangles);
* ``golden_hashes.json``: SHA-256 digests and statistics for the full-size
  workloads (10k-triangle soup at 512x512, 1.31M-triangle displaced icosphere
  at 1920x1080), whose arrays are too large to commit.

Usage (needs the reference sources; writes only into this directory):
    export REF_ROOT=<reference checkout>
    oracle/build_ref.sh && python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nostrum_pray_gb300 import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF_ROOT = os.environ.get("REF_ROOT", "")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def mesh_hash(m: scenes.Mesh) -> str:
    return sha(np.concatenate([m.verts.view(np.uint32).reshape(-1), m.colors.view(np.uint32).reshape(-1),
                               m.emit.astype(np.uint32)]))


def dump_hash(d) -> str:
    return sha(np.concatenate([d["boxes"].view(np.uint8).reshape(-1), d["split"].view(np.uint8),
                               d["info"].view(np.uint8).reshape(-1), d["refs"].view(np.uint8)]))


def trace_case(ref, setup):
    rays = O.ref_primary_rays(setup.width, setup.height, setup.fov, setup.cam_pos, setup.cam_look)
    ids, ts = ref.trace(rays)
    return rays, ids.astype(np.int32), ts


def main():
    if not os.path.isdir(os.path.join(REF_ROOT, "examples")):
        sys.exit("make_golden: set REF_ROOT to a checkout of the reference")
    small = {}
    hashes = {}

    # -- C1 soup: median tree leaf <= 8, depth <= 24 ------------------------
    for seed in (0, 1, 2):
        m = scenes.soup(10_000, seed)
        st = scenes.soup_setup()
        ref = O.ReferenceScene.from_setup(m, st)
        d = ref.tree_dump()
        rays, ids, ts = trace_case(ref, st)
        img = ref.render_rt(st)
        key = f"soup_s{seed}"
        hashes[key] = {"mesh": mesh_hash(m), "stats": [int(x) for x in ref.tree_stats()],
                       "tree": dump_hash(d), "rays": sha(rays), "ids": sha(ids), "t": sha(ts),
                       "image": sha(img), "hits": int((ids >= 0).sum()), "variant": O.ref_variant(st)}
        if seed == 0:
            small[key + "_ids"] = ids
            small[key + "_t"] = ts
            small[key + "_image"] = img
            small[key + "_precompute"] = ref.precompute()[:256]
            for k, v in d.items():
                small[f"{key}_tree_{k}"] = v
        # the same soup with the reference's SAH tree and default constants
        st_sah = scenes.soup_setup()
        st_sah.tree, st_sah.leaf_size, st_sah.max_depth = "sah", 32, 20
        ref2 = O.ReferenceScene.from_setup(m, st_sah)
        d2 = ref2.tree_dump()
        _, ids2, ts2 = trace_case(ref2, st_sah)
        hashes[key + "_sah"] = {"stats": [int(x) for x in ref2.tree_stats()], "tree": dump_hash(d2),
                                "ids": sha(ids2), "t": sha(ts2), "image": sha(ref2.render_rt(st_sah)),
                                "variant": O.ref_variant(st_sah)}
        print(key, hashes[key]["stats"], hashes[key]["hits"], flush=True)

    # -- displaced icosphere, SAH (Ct 1, Ci 1.5) ----------------------------
    for level, (w, h) in ((5, (480, 270)), (8, (1920, 1080))):
        m = scenes.icosphere(level)
        for eps in (0.0, 1e-4):
            st = scenes.icosphere_setup(w, h, det_eps=eps)
            ref = O.ReferenceScene.from_setup(m, st)
            d = ref.tree_dump()
            rays, ids, ts = trace_case(ref, st)
            img = ref.render_rt(st)
            key = f"ico{level}_eps{eps:g}"
            hashes[key] = {"mesh": mesh_hash(m), "stats": [int(x) for x in ref.tree_stats()],
                           "tree": dump_hash(d), "rays": sha(rays), "ids": sha(ids), "t": sha(ts),
                           "image": sha(img), "hits": int((ids >= 0).sum()), "variant": O.ref_variant(st)}
            if level == 5 and eps == 0.0:
                small[key + "_ids"] = ids
                small[key + "_t"] = ts
                small[key + "_image"] = img
                for k, v in d.items():
                    small[f"{key}_tree_{k}"] = v
            print(key, hashes[key]["stats"], hashes[key]["hits"], flush=True)
            del ref

    # -- the reference's example scenes through its own loader ---------------
    ex = os.path.join(REF_ROOT, "examples")
    for name, js in (("cube", "cube/cube.json"), ("head_fov30", "head_fov30/head_fov30.json"),
                     ("plant", "plant/plant.json"), ("pt_cornell", "pt_cornell/pt_cornell.json")):
        path = os.path.join(ex, js)
        if not os.path.exists(path):
            continue
        L = O.ref_lib("default")
        hnd = L.ref_scene_from_json(path.encode())
        info = np.zeros(17, np.float64)
        L.ref_scene_info(hnd, info)
        n, nl = int(info[16]), int(info[15])
        verts = np.empty((n, 9), np.float32)
        cols = np.empty((n, 3), np.float32)
        emit = np.empty(n, np.uint8)
        lights = np.empty((max(nl, 1), 6), np.float32)
        L.ref_scene_get(hnd, verts, cols, emit, lights)
        L.ref_scene_free(hnd)
        small[f"ex_{name}_info"] = info
        small[f"ex_{name}_verts"] = verts
        small[f"ex_{name}_colors"] = cols
        small[f"ex_{name}_emit"] = emit
        small[f"ex_{name}_lights"] = lights[:nl]
        m = scenes.Mesh(verts, cols, emit)
        # reduced-resolution render with the scene's own camera and lights
        st = scenes.RenderSetup(width=160, height=120, fov=int(info[2]), cam_pos=tuple(info[6:9]),
                                cam_look=tuple(info[9:12]), lights=[tuple(l) for l in lights[:nl]],
                                background=tuple(info[12:15]), tree="median")
        ref = O.ReferenceScene.from_setup(m, st)
        small[f"ex_{name}_image160"] = ref.render_rt(st)
        d = ref.tree_dump()
        hashes[f"ex_{name}"] = {"stats": [int(x) for x in ref.tree_stats()], "tree": dump_hash(d),
                                "n": n, "lights": nl}
        print("example", name, n, nl, flush=True)

    # -- hand-written OBJ/MTL cases (tests/golden/obj_cases) through the
    #    reference's loader: polygons, negative indices, CRLF, exponent and
    #    bare-fraction numbers, usemtl / o / g flushing
    for name in ("poly", "shapes"):
        L = O.ref_lib("default")
        hnd = L.ref_scene_from_json(os.path.join(HERE, "obj_cases", name + ".json").encode())
        info = np.zeros(17, np.float64)
        L.ref_scene_info(hnd, info)
        n, nl = int(info[16]), int(info[15])
        verts = np.empty((n, 9), np.float32)
        cols = np.empty((n, 3), np.float32)
        emit = np.empty(n, np.uint8)
        lights = np.empty((max(nl, 1), 6), np.float32)
        L.ref_scene_get(hnd, verts, cols, emit, lights)
        L.ref_scene_free(hnd)
        for k, v in (("info", info), ("verts", verts), ("colors", cols), ("emit", emit), ("lights", lights[:nl])):
            small[f"objcase_{name}_{k}"] = v
        print("obj case", name, n, nl)

    # -- loader round trip: scenes.write_scene output read by the reference --
    with tempfile.TemporaryDirectory() as td:
        m = scenes.soup(500, 7)
        m.emit[::50] = 1
        st = scenes.soup_setup(64, 48)
        p = os.path.join(td, "soup.json")
        scenes.write_scene(p, m, st)
        L = O.ref_lib("default")
        hnd = L.ref_scene_from_json(p.encode())
        info = np.zeros(17, np.float64)
        L.ref_scene_info(hnd, info)
        n = int(info[16])
        verts = np.empty((n, 9), np.float32)
        cols = np.empty((n, 3), np.float32)
        emit = np.empty(n, np.uint8)
        lights = np.empty((max(int(info[15]), 1), 6), np.float32)
        L.ref_scene_get(hnd, verts, cols, emit, lights)
        L.ref_scene_free(hnd)
        ok = (np.array_equal(verts, m.verts) and np.array_equal(cols, m.colors) and np.array_equal(emit, m.emit))
        hashes["writer_roundtrip_soup500_s7"] = {"equal": bool(ok), "info": info.tolist()}
        print("writer round trip through the reference loader:", ok)

    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **small)
    with open(os.path.join(HERE, "golden_hashes.json"), "w") as f:
        json.dump(hashes, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
