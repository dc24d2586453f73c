"""Digests used by the golden fixtures (same definitions as make_golden.py)
and readers of the command-line tools' outputs."""
import hashlib
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "nostrum_pray_gb300", "_build")


def ref_root():
    """A checkout of the reference, for tests that read its files: REF_ROOT
    from the environment, else the location oracle/build_ref.sh recorded
    when it built the reference; None where there is none."""
    r = os.environ.get("REF_ROOT")
    if not r:
        rec = os.path.join(ROOT, "oracle", "_ref", "ref_root.txt")
        if os.path.exists(rec):
            r = open(rec).read().strip()
    return r if r and os.path.isdir(os.path.join(r, "include")) else None


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


# -- statistical comparison of path-tracing estimators -----------------------

def pt_moments_fixture():
    """tests/golden/pt_moments.npz (make_pt_moments.py): per case, the
    reference estimator's per-pixel mean, sample variance and run count."""
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "pt_moments.npz")))


def batch_moments(frames):
    """Mean and variance of the mean over independent frames (each the
    per-pixel mean of an equal number of samples), in float64."""
    a = np.asarray(frames, np.float64)
    return a.mean(0), a.var(0, ddof=1) / a.shape[0]


def same_expectation(mean_a, varmean_a, mean_b, varmean_b, max_z=6.0, z2_band=(0.6, 1.3), max_image_z=4.5):
    """Whether two per-pixel estimates of the same image agree within their
    sampling error. z = (a - b) / sqrt(var_a + var_b) per pixel and channel;
    the estimates agree when no |z| exceeds max_z, the mean of z^2 lies in
    z2_band (it is 1 for equal expectations and correctly estimated
    variances), the image means per channel differ by less than max_image_z
    standard errors, and pixels whose both variances are zero have equal
    means. Returns (ok, description)."""
    a, b = np.asarray(mean_a, np.float64), np.asarray(mean_b, np.float64)
    va, vb = np.asarray(varmean_a, np.float64), np.asarray(varmean_b, np.float64)
    se = np.sqrt(va + vb)
    live = se > 0
    dead_bad = int((np.abs(a - b)[~live] > 1e-6 * np.maximum(1.0, np.abs(a[~live]))).sum())
    z = (a - b)[live] / se[live]
    n_pix = a.shape[0] * a.shape[1]
    img_z = (a.mean((0, 1)) - b.mean((0, 1))) / (np.sqrt((va + vb).sum((0, 1))) / n_pix)
    z2 = float((z * z).mean()) if z.size else 1.0
    zmax = float(np.abs(z).max()) if z.size else 0.0
    ok = (dead_bad == 0 and zmax < max_z and z2_band[0] <= z2 <= z2_band[1]
          and bool((np.abs(img_z) < max_image_z).all()))
    desc = (f"max|z| {zmax:.2f} over {z.size}, mean z^2 {z2:.3f}, image z {np.round(img_z, 2).tolist()}, "
            f"{dead_bad} zero-variance pixels differ")
    return ok, desc
