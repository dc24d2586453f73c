"""The reference-side binding (integration/gpu_kdtree.{h,cpp}: a
SpatialDatabase subclass, include/spatial.h:10-39 of the reference, answered
by the GPU kd tree) compiles against the reference's own headers in every
instruction-set variant its include/options.h selects (scalar; SSE3 and AVX
on x86), and uses only entry points this library exports. Skipped where no
checkout of the reference is present (REF_ROOT, or the location
oracle/build_ref.sh recorded). Its GPU work goes through
pray_trace_closest_host, pray_render_rt_host and pray_render_pt_host, which
the GPU tests call directly (test_trace_gpu.py::test_host_rays_from_many_threads)."""
import os
import platform
import re
import subprocess

import pytest

from golden_util import ref_root

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "integration", "gpu_kdtree.cpp")


def variants():
    out = [("scalar", [])]
    if platform.machine() in ("x86_64", "AMD64"):
        out += [("sse3", ["-msse3"]), ("avx", ["-mavx"])]
    return out


@pytest.mark.parametrize("name,flags", variants(), ids=[v[0] for v in variants()])
def test_binding_compiles_against_reference_headers(name, flags):
    ref = ref_root()
    if ref is None:
        pytest.skip("no checkout of the reference on this machine")
    cmd = ["g++", "-std=c++14", *flags, "-fsyntax-only", "-Wall", "-Wextra", "-Wno-reorder", "-Werror",
           "-include", "limits", "-include", "fstream", f"-I{ref}/include", f"-I{ref}/ext",
           f"-I{os.path.join(ROOT, 'include')}", SRC]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]


def test_binding_calls_only_exported_entry_points():
    from nostrum_pray_gb300 import native
    src = open(SRC).read() + open(SRC.replace(".cpp", ".h")).read()
    called = set(re.findall(r"\b(pray_[a-z_]+)\s*\(", src))
    assert {"pray_scene_create", "pray_trace_closest_host", "pray_render_rt_host", "pray_render_pt_host"} <= called
    assert called <= set(native.EXPORTED), called - set(native.EXPORTED)
