"""Recipe: compile the reference's own src/renderer.cu for the CPU and the GPU.

Test infrastructure.  The reference renderer is CUDA; there is no GPU in the
build container and the reference sources are not available where the GPU
runs.  So its translation unit is compiled by g++ against a host emulation of
the CUDA built-ins it uses (ref_host/isti_refhost.h, ref_host/ref_runtime.cpp)
and a glm subset (ref_host/glm), and executed on the CPU.  Its output pins the
C oracle (isti_oracle.c) and produces the golden fixtures in tests/golden.

The only change to the source is mechanical and made in a generated copy under
oracle/_ref/ (never committed): each kernel launch ``K<<<grid, block>>>(args)``
becomes ``isti_refhost::launch(grid, block, K)(args)``, which g++ can parse.
All other lines are compiled as they are.

GPU build (``stage_gpu`` + ``build_gpu``): unmodified copies of
src/renderer.cu and the headers it includes are staged under oracle/_ref/gpu/
(never committed; they travel with the working tree to the GPU host, where the
reference tree itself is absent), and ``build_gpu`` compiles them with
ref_gpu/ref_gpu_driver.cu by nvcc for sm_103a with the reference's own CUDA
flags (CMakeLists.txt:36 minus -keep) into oracle/_ref/libisti_ref_gpu.so.

Usage: python oracle/build_ref.py --reference <reference tree>
       (or ISTI_REFERENCE_DIR=<reference tree> python oracle/build_ref.py)
Writes oracle/_ref/libisti_ref.so, stages oracle/_ref/gpu/ and, where nvcc is
available, builds oracle/_ref/libisti_ref_gpu.so.
"""
import argparse
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LAUNCH_RE = re.compile(r"([A-Za-z_]\w*(?:\s*<[^<>;()]*>)?)\s*<<<(.*?)>>>")


def rewrite_launches(src: str) -> tuple[str, int]:
    return LAUNCH_RE.subn(lambda m: f"isti_refhost::launch({m.group(2)}, {m.group(1)})", src)


GPU_DIR = os.path.join(OUT_DIR, "gpu")
GPU_LIB = os.path.join(OUT_DIR, "libisti_ref_gpu.so")
# src/renderer.cu and everything it includes from the reference's include/ tree
GPU_SOURCES = ["src/renderer.cu", "include/renderer.h", "include/data.h", "include/util/image_buffer.h",
               "include/util/helper_common.h", "include/util/helper_math.h", "include/util/helper_math_ext.h",
               "include/util/cuda_helper_device.h", "include/util/cuda_helper_host.h"]


def stage_gpu(reference: str, verbose: bool = False) -> bool:
    """Copies the reference sources of the GPU build under oracle/_ref/gpu/, unmodified."""
    if not all(os.path.isfile(os.path.join(reference, f)) for f in GPU_SOURCES):
        return False
    for f in GPU_SOURCES:
        dst = os.path.join(GPU_DIR, "renderer.cu" if f == "src/renderer.cu" else f)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        src = os.path.join(reference, f)
        if not os.path.exists(dst) or open(src, "rb").read() != open(dst, "rb").read():
            shutil.copyfile(src, dst)
    if verbose:
        print(f"staged {len(GPU_SOURCES)} reference files under {GPU_DIR}")
    return True


def build_gpu(verbose: bool = False) -> str | None:
    """Compiles the staged reference renderer for sm_103a (no GPU needed to build)."""
    renderer = os.path.join(GPU_DIR, "renderer.cu")
    driver = os.path.join(HERE, "ref_gpu", "ref_gpu_driver.cu")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.isfile(renderer) or not os.path.isfile(nvcc):
        return None
    deps = [renderer, driver, os.path.join(HERE, "isti_oracle.h"), os.path.join(HERE, "ref_host", "glm", "glm.hpp")]
    if os.path.exists(GPU_LIB) and os.path.getmtime(GPU_LIB) > max(os.path.getmtime(d) for d in deps):
        return GPU_LIB
    cmd = [nvcc, "-std=c++20", "-O3", "-gencode=arch=compute_103a,code=sm_103a",
           # the reference's CUDA flags, CMakeLists.txt:36 (without -keep and --ptxas-options=-v)
           "-Xcompiler", "-D_FORCE_INLINES", "-DVERBOSE", "--expt-extended-lambda", "-use_fast_math",
           "--expt-relaxed-constexpr",
           "-Xcompiler", "-fPIC", "-shared", "-w",
           "-I", GPU_DIR, "-I", os.path.join(GPU_DIR, "include"), "-I", os.path.join(HERE, "ref_host"),
           driver, "-o", GPU_LIB]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return GPU_LIB


def build(reference: str, verbose: bool = False) -> str | None:
    src_path = os.path.join(reference, "src", "renderer.cu")
    if not os.path.isfile(src_path):
        if verbose:
            print(f"reference not found at {reference}; skipping oracle/_ref")
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(src_path) as f:
        src = f.read()
    out, n = rewrite_launches(src)
    if n != 3:
        raise RuntimeError(f"expected 3 kernel launch sites in renderer.cu, found {n}")
    gen = os.path.join(OUT_DIR, "renderer_host.cpp")
    with open(gen, "w") as f:
        f.write(f"// GENERATED by oracle/build_ref.py from {src_path}; do not commit.\n")
        f.write(out)
    lib = os.path.join(OUT_DIR, "libisti_ref.so")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cmd = [
        "g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
        "-Wno-attributes", "-Wno-deprecated-declarations", "-Wno-narrowing",
        "-D__host__=", "-D__device__=", "-D__global__=",
        "-include", os.path.join(HERE, "ref_host", "isti_refhost.h"),
        "-I", OUT_DIR, "-I", os.path.join(HERE, "ref_host"),
        "-I", os.path.join(reference, "include"), "-I", cuda_inc,
        os.path.join(HERE, "ref_host", "ref_driver.cpp"),
        os.path.join(HERE, "ref_host", "ref_runtime.cpp"),
        "-o", lib,
        # the emulated cudaMalloc & co. must bind inside this library even when a real CUDA
        # runtime is loaded globally into the process (torch loads one RTLD_GLOBAL)
        "-Wl,-Bsymbolic",
    ]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    build_io(reference, verbose)
    stage_gpu(reference, verbose)
    return lib


def build_io(reference: str, verbose: bool = False) -> str | None:
    """The reference's vendored image libraries (stb_image, stb_image_write,
    tinyexr; dependencies/) with the configuration of
    src/util/image_buffer.cu:8-17, wrapped by ref_host/ref_io.cpp."""
    deps = os.path.join(reference, "dependencies")
    if not os.path.isfile(os.path.join(deps, "tinyexr", "tinyexr.h")):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    lib = os.path.join(OUT_DIR, "libref_io.so")
    src = os.path.join(HERE, "ref_host", "ref_io.cpp")
    if os.path.exists(lib) and os.path.getmtime(lib) > os.path.getmtime(src):
        return lib
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w",
           "-I", os.path.join(deps, "stb_image"), "-I", os.path.join(deps, "tinyexr"),
           src, "-o", lib, "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return lib


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("ISTI_REFERENCE_DIR"))
    args = ap.parse_args()
    if not args.reference:
        ap.error("give --reference or set ISTI_REFERENCE_DIR")
    lib = build(args.reference, verbose=True)
    if lib:
        print(f"built {lib}")
    gpu = build_gpu(verbose=True)
    if gpu:
        print(f"built {gpu}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
