"""Digests used by the golden fixtures (same definitions as make_golden.py)
and readers of the command-line tools' outputs."""
import hashlib
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "nostrum_pray_gb300", "_build")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def mesh_hash(m) -> str:
    return sha(np.concatenate([m.verts.view(np.uint32).reshape(-1), m.colors.view(np.uint32).reshape(-1),
                               m.emit.astype(np.uint32)]))


def dump_hash(d) -> str:
    return sha(np.concatenate([d["boxes"].view(np.uint8).reshape(-1), d["split"].view(np.uint8),
                               d["info"].view(np.uint8).reshape(-1), d["refs"].view(np.uint8)]))


def load_scene_dump(json_path):
    """The scene as the command line loads it (pray_scene_dump): info[17]
    (width, height, fov, path tracing, max depth, samples, camera position,
    look, background, light count, triangle count), vertices, colours,
    emitter flags, lights."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "scene.bin")
        p = subprocess.run([os.path.join(BUILD, "pray_scene_dump"), json_path, out], capture_output=True, text=True)
        assert p.returncode == 0, p.stderr
        raw = open(out, "rb").read()
    info = np.frombuffer(raw[:17 * 8], np.float64)
    n, nl = int(info[16]), int(info[15])
    o = 17 * 8
    verts = np.frombuffer(raw[o:o + 36 * n], np.float32).reshape(n, 9)
    o += 36 * n
    cols = np.frombuffer(raw[o:o + 12 * n], np.float32).reshape(n, 3)
    o += 12 * n
    emit = np.frombuffer(raw[o:o + n], np.uint8)
    o += n
    lights = np.frombuffer(raw[o:o + 24 * nl], np.float32).reshape(nl, 6)
    return info, verts, cols, emit, lights


def read_bmp(path) -> np.ndarray:
    """A 24-bit uncompressed BMP as (height, width, 3) RGB, top row first."""
    raw = open(path, "rb").read()
    assert raw[:2] == b"BM"
    off = int.from_bytes(raw[10:14], "little")
    w = int.from_bytes(raw[18:22], "little", signed=True)
    h = int.from_bytes(raw[22:26], "little", signed=True)
    assert int.from_bytes(raw[28:30], "little") == 24
    pitch = (3 * w + 3) & ~3
    rows = np.frombuffer(raw[off:off + pitch * abs(h)], np.uint8).reshape(abs(h), pitch)[:, :3 * w]
    img = rows.reshape(abs(h), w, 3)[:, :, ::-1]
    return np.ascontiguousarray(img if h < 0 else img[::-1])
