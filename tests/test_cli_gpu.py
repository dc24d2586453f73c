"""The `Pray <scene.json> <out.bmp>` command line end to end on the GPU
(src/main.cpp:23-109): scene files in, BMP out, compared with the oracle's
frame of the same loaded scene. Ray tracing, the Kajiya path tracer
(max_depth > 1) and the branching path tracer the reference selects for
max_depth <= 1 (src/scene_preprocessor.cpp:34-40)."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from golden_util import load_scene_dump, read_bmp
from nostrum_pray_gb300 import native, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = os.path.join(HERE, "golden", "obj_cases")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    native.lib()


def run_cli(tmp_path, desc):
    for f in os.listdir(CASES):
        if not f.endswith(".json"):
            shutil.copy(os.path.join(CASES, f), tmp_path / f)
    js = tmp_path / "scene.json"
    js.write_text(json.dumps(desc))
    out = tmp_path / "out.bmp"
    p = subprocess.run([native.CLI_PATH, str(js), str(out)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    info, verts, cols, emit, lights = load_scene_dump(str(js))
    mesh = scenes.Mesh(verts.copy(), cols.copy(), emit.copy())
    st = scenes.RenderSetup(width=int(info[0]), height=int(info[1]), fov=int(info[2]), cam_pos=tuple(info[6:9]),
                            cam_look=tuple(info[9:12]), lights=[tuple(l) for l in lights],
                            background=tuple(info[12:15]), tree="median")
    return read_bmp(str(out)), p.stdout, mesh, st


def base_desc(**kw):
    d = json.load(open(os.path.join(CASES, "shapes.json")))
    d.update(kw)
    return d


def test_cli_ray_tracing(oracle, tmp_path):
    img, log, mesh, st = run_cli(tmp_path, base_desc(method="ray_tracing", resolution_x=64, resolution_y=48))
    want, _ = oracle.OracleScene.from_setup(mesh, st).render_rt(st)
    np.testing.assert_array_equal(img, want)


@pytest.mark.parametrize("depth,samples,mode", [(3, 8, 0), (1, 6, 2), (0, 3, 2)])
def test_cli_path_tracing_modes(oracle, tmp_path, depth, samples, mode):
    img, log, mesh, st = run_cli(tmp_path, base_desc(max_depth=depth, num_samples=samples, background=[0.2, 0.3, 0.4]))
    assert ("Using diffuse path tracing." in log) == (mode == 2)
    want, _, _ = oracle.OracleScene.from_setup(mesh, st).render_pt(st, spp=samples, max_depth=depth, seed=0,
                                                                    mode=mode)
    assert (np.abs(img.astype(int) - want.astype(int)) <= 1).all()
