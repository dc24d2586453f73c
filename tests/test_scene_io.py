"""The command line's scene loader against the reference's own loader
(readSceneDescription, src/io.cpp:27-137, with the vendored tinyobjloader):
triangles, colours, emitter flags, lights and JSON fields must come out
bit-identical. Reference outputs are in tests/golden/ (make_golden.py)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from golden_util import load_scene_dump, ref_root
from nostrum_pray_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DUMP = os.path.join(ROOT, "nostrum_pray_gb300", "_build", "pray_scene_dump")
CASES = os.path.join(ROOT, "tests", "golden", "obj_cases")
REF_EXAMPLES = os.path.join(ref_root() or "", "examples")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from nostrum_pray_gb300 import build
    build.build()


def load(json_path):
    return load_scene_dump(json_path)


def same(got, small, prefix):
    info, verts, cols, emit, lights = got
    np.testing.assert_array_equal(info[:15], small[prefix + "_info"][:15])
    np.testing.assert_array_equal(verts.view(np.uint32), small[prefix + "_verts"].view(np.uint32))
    np.testing.assert_array_equal(cols.view(np.uint32), small[prefix + "_colors"].view(np.uint32))
    np.testing.assert_array_equal(emit, small[prefix + "_emit"])
    np.testing.assert_array_equal(lights.view(np.uint32), small[prefix + "_lights"].view(np.uint32))


@pytest.mark.parametrize("name", ["poly", "shapes"])
def test_handwritten_obj_cases(golden, name):
    _, small = golden
    same(load(os.path.join(CASES, name + ".json")), small, f"objcase_{name}")


@pytest.mark.parametrize("name,js", [("cube", "cube/cube.json"), ("head_fov30", "head_fov30/head_fov30.json"),
                                     ("plant", "plant/plant.json"), ("pt_cornell", "pt_cornell/pt_cornell.json")])
def test_reference_examples(golden, name, js):
    _, small = golden
    path = os.path.join(REF_EXAMPLES, js)
    if not os.path.exists(path):
        pytest.skip("reference example scenes not present on this machine")
    same(load(path), small, f"ex_{name}")


def test_writer_round_trip(golden):
    """scenes.write_scene -> loader gives back the exact floats (the reference
    loader does too: golden 'writer_roundtrip_soup500_s7')."""
    hashes, _ = golden
    assert hashes["writer_roundtrip_soup500_s7"]["equal"]
    m = scenes.soup(500, 7)
    m.emit[::50] = 1
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "soup.json")
        scenes.write_scene(p, m, scenes.soup_setup(64, 48))
        info, verts, cols, emit, lights = load(p)
    np.testing.assert_array_equal(verts, m.verts)
    np.testing.assert_array_equal(cols, m.colors)
    np.testing.assert_array_equal(emit, m.emit)
    np.testing.assert_array_equal(info[:15], hashes["writer_roundtrip_soup500_s7"]["info"][:15])


def test_missing_file_is_an_error():
    p = subprocess.run([DUMP, "/nonexistent/scene.json", "/tmp/x.bin"], capture_output=True, text=True)
    assert p.returncode == 1 and "Error opening file" in p.stderr


def test_cli_usage_exit_code():
    from nostrum_pray_gb300 import native
    p = subprocess.run([native.CLI_PATH], capture_output=True, text=True)
    assert p.returncode == 1 and "usage" in p.stdout
