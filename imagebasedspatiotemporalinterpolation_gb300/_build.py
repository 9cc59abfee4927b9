"""In-tree build of the native code (no CMake, no pip install).

  _lib/libisti.so        CUDA kernels + C ABI (include/isti.h, isti_io.h,
                         isti_dataset.h): renderer, image codecs, dataset loader
  _lib/splinter          the command-line frame loop (csrc/host/splinter.cpp),
                         linked statically against the same objects
  _lib/libisti_scene.so  procedural keyframe generator (host C, OpenMP)

Objects are compiled in parallel into _lib/obj/ and linked by nvcc (static
CUDA runtime).  The interpolation arithmetic is compiled twice: with
-fmad=false (no multiply-add contraction) and IEEE division / square root
(isti_render.cu, the default mode, bit-exact against the oracle), and with the
reference's -use_fast_math (isti_render_fm.cu, the reference GPU build's
arithmetic).  Host code uses -ffp-contract=off.
"""
from __future__ import annotations

import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
LIB_DIR = os.path.join(PKG_DIR, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
CSRC = os.path.join(PKG_DIR, "csrc")
HOST_SRC = os.path.join(CSRC, "host")
INCLUDE = os.path.join(REPO_DIR, "include")

CUDA_ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CUDA_SOURCES = ["isti_render.cu", "isti_render_fm.cu", "isti_metrics.cu", "isti_unet.cu", "isti_flownet.cu", "isti_scene_gpu.cu"]
# Translation units compiled with the reference's GPU arithmetic (-use_fast_math,
# the reference's CMakeLists.txt:36) instead of -fmad=false / IEEE division.
FAST_MATH_SOURCES = {"isti_render_fm.cu"}
# Translation units with the compiler's default contraction (the learned initialiser:
# tensor-core GEMMs with f32 accumulation, no bit-exactness contract).
DEFAULT_MATH_SOURCES = {"isti_unet.cu", "isti_flownet.cu", "isti_scene_gpu.cu"}
HOST_LIB_SOURCES = ["isti_io.cpp", "isti_dataset.cpp"]


def _cuda_home() -> str:
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc() -> str:
    cand = os.path.join(_cuda_home(), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def cuda_lib_path() -> str:
    return os.path.join(LIB_DIR, "libisti.so")


def splinter_path() -> str:
    return os.path.join(LIB_DIR, "splinter")


def scene_lib_path() -> str:
    return os.path.join(LIB_DIR, "libisti_scene.so")


def _obj(src: str) -> str:
    return os.path.join(OBJ_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")


def _cuda_obj_cmd(src: str) -> list[str]:
    base = os.path.basename(src)
    arith = ["-use_fast_math"] if base in FAST_MATH_SOURCES else ([] if base in DEFAULT_MATH_SOURCES else ["-fmad=false"])
    return [
        _nvcc(), "-std=c++20", "-O3", CUDA_ARCH, "-lineinfo", *arith,
        "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
        "-c", src, "-o", _obj(src),
    ]


def _host_obj_cmd(src: str) -> list[str]:
    return ["g++", "-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I", HOST_SRC,
            "-I", os.path.join(_cuda_home(), "include"), "-c", src, "-o", _obj(src)]


def _lib_objs() -> list[str]:
    return [_obj(os.path.join(CSRC, s)) for s in CUDA_SOURCES] + [_obj(os.path.join(HOST_SRC, s)) for s in HOST_LIB_SOURCES]


def _scene_cmd(out: str) -> list[str]:
    return ["gcc", "-std=c11", "-O2", "-fopenmp", "-fPIC", "-shared",
            os.path.join(CSRC, "isti_scene.c"), "-o", out, "-lm"]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out += [os.path.join(HOST_SRC, f) for f in os.listdir(HOST_SRC) if f.endswith((".hpp", ".h"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return out


def _run_parallel(jobs: list[tuple[str, list[str]]], verbose: bool) -> None:
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


def build_all(force: bool = False, verbose: bool = False) -> None:
    """Compile every native library and tool of the package (objects in parallel, then links)."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = _headers()
    jobs = []
    for s in CUDA_SOURCES:
        cu_src = os.path.join(CSRC, s)
        if force or _stale(_obj(cu_src), [cu_src] + headers):
            jobs.append((os.path.basename(_obj(cu_src)), _cuda_obj_cmd(cu_src)))
    for s in HOST_LIB_SOURCES + ["splinter.cpp"]:
        src = os.path.join(HOST_SRC, s)
        if force or _stale(_obj(src), [src] + headers):
            jobs.append((os.path.basename(_obj(src)), _host_obj_cmd(src)))
    if force or _stale(scene_lib_path(), [os.path.join(CSRC, "isti_scene.c")]):
        jobs.append(("libisti_scene.so", _scene_cmd(scene_lib_path())))
    _run_parallel(jobs, verbose)

    links = []
    lib_objs = _lib_objs()
    if force or _stale(cuda_lib_path(), lib_objs):
        links.append(("libisti.so", [_nvcc(), CUDA_ARCH, "-shared", *lib_objs, "-o", cuda_lib_path()]))
    exe_objs = lib_objs + [_obj(os.path.join(HOST_SRC, "splinter.cpp"))]
    if force or _stale(splinter_path(), exe_objs):
        links.append(("splinter", [_nvcc(), CUDA_ARCH, *exe_objs, "-o", splinter_path()]))
    _run_parallel(links, verbose)
