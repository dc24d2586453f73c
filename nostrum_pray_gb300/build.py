"""In-tree native build: the CUDA kernels (sm_103a) and host C++ into
``nostrum_pray_gb300/_build/libnostrum_pray.so``, and the ``Pray`` command-line
binary. Plain nvcc / g++ invocations, compiled in parallel; a target is rebuilt
when any of its sources or headers is newer than it."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
from typing import List, Sequence

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libnostrum_pray.so")
CLI = os.path.join(BUILD, "Pray")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["trace.cu", "pt.cu", "wavefront.cu", "wavefront_noalloc.cu", "batch.cu", "denoise_ops.cu", "denoise_tc.cu"]
CPP_SOURCES = ["capi.cpp", "host/kdtree.cpp", "host/camera.cpp", "host/flatten.cpp", "denoise_net.cpp"]
CLI_SOURCES = ["cli/pray_main.cpp", "cli/scene_io.cpp"]
DUMP_SOURCES = ["cli/scene_dump.cpp"]
DUMP = os.path.join(BUILD, "pray_scene_dump")

NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall",
             f"-I{CUDA_HOME}/include"]


def _headers() -> List[str]:
    hs = glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(target: str, deps: Sequence[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: List[str], log: List[str]) -> None:
    p = subprocess.run(cmd, capture_output=True, text=True)
    log.append(" ".join(cmd) + "\n" + p.stdout + p.stderr)
    if p.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")


def _obj(src: str) -> str:
    return os.path.join(BUILD, "obj", src.replace("/", "_").rsplit(".", 1)[0] + ".o")


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc") or nvcc
    hdrs = _headers()
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        o = _obj(s)
        if force or _stale(o, [src] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", o])
    for s in CPP_SOURCES + CLI_SOURCES + DUMP_SOURCES:
        src = os.path.join(CSRC, s)
        o = _obj(s)
        if force or _stale(o, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", o])
    log: List[str] = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(lambda c: _run(c, log), jobs))
    lib_objs = [_obj(s) for s in CU_SOURCES + CPP_SOURCES]
    cudalib = os.path.join(CUDA_HOME, "lib64")
    if force or _stale(LIB, lib_objs):
        _run(["g++", "-shared", "-o", LIB + ".tmp"] + lib_objs +
             [f"-L{cudalib}", "-lcudart_static", "-ldl", "-lrt", "-lpthread"], log)
        os.replace(LIB + ".tmp", LIB)
    cli_objs = [_obj(s) for s in CLI_SOURCES]
    if force or _stale(CLI, cli_objs + [LIB]):
        _run(["g++", "-o", CLI + ".tmp"] + cli_objs + [LIB, "-Wl,-rpath,$ORIGIN", "-pthread"], log)
        os.replace(CLI + ".tmp", CLI)
    dump_objs = [_obj("cli/scene_dump.cpp"), _obj("cli/scene_io.cpp")]
    if force or _stale(DUMP, dump_objs):
        _run(["g++", "-o", DUMP + ".tmp"] + dump_objs, log)
        os.replace(DUMP + ".tmp", DUMP)
    if verbose:
        sys.stdout.write("\n".join(log))
    with open(os.path.join(BUILD, "build.log"), "a") as f:
        f.write("\n".join(log))
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
