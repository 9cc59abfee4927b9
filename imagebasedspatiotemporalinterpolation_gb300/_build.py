"""In-tree build of the native libraries (no CMake, no pip install).

  _lib/libisti.so        CUDA kernels + C ABI (include/isti.h), sm_103a only
  _lib/libisti_scene.so  procedural keyframe generator (host C, OpenMP)

The interpolation arithmetic is compiled with -fmad=false (no multiply-add
contraction) and IEEE division / square root, and host code with
-ffp-contract=off, so results do not depend on the compiler's contraction
choices and match the oracle bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
LIB_DIR = os.path.join(PKG_DIR, "_lib")
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")

CUDA_ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CUDA_SOURCES = ["isti_render.cu"]  # includes isti_kernels.cuh


def _nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def cuda_lib_path() -> str:
    return os.path.join(LIB_DIR, "libisti.so")


def scene_lib_path() -> str:
    return os.path.join(LIB_DIR, "libisti_scene.so")


def _cuda_cmd(out: str) -> list[str]:
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES]
    return [
        _nvcc(), "-std=c++20", "-O3", CUDA_ARCH, "-lineinfo", "-fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared", "-I", INCLUDE, "-I", CSRC,
        *srcs, "-o", out,
    ]


def _scene_cmd(out: str) -> list[str]:
    return ["gcc", "-std=c11", "-O2", "-fopenmp", "-fPIC", "-shared",
            os.path.join(CSRC, "isti_scene.c"), "-o", out, "-lm"]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps_cuda() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return out


def build_all(force: bool = False, verbose: bool = False) -> None:
    """Compile every native library of the package, in parallel."""
    os.makedirs(LIB_DIR, exist_ok=True)
    jobs = []
    if force or _stale(cuda_lib_path(), _deps_cuda()):
        jobs.append(("libisti.so", _cuda_cmd(cuda_lib_path())))
    if force or _stale(scene_lib_path(), [os.path.join(CSRC, "isti_scene.c")]):
        jobs.append(("libisti_scene.so", _scene_cmd(scene_lib_path())))
    procs = []
    for name, cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"building {name} failed:\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"))
    if errors:
        raise RuntimeError("\n".join(errors))
