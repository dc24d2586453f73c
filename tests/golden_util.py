"""Digests used by the golden fixtures (same definitions as make_golden.py)."""
import hashlib

import numpy as np


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def mesh_hash(m) -> str:
    return sha(np.concatenate([m.verts.view(np.uint32).reshape(-1), m.colors.view(np.uint32).reshape(-1),
                               m.emit.astype(np.uint32)]))


def dump_hash(d) -> str:
    return sha(np.concatenate([d["boxes"].view(np.uint8).reshape(-1), d["split"].view(np.uint8),
                               d["info"].view(np.uint8).reshape(-1), d["refs"].view(np.uint8)]))
