"""Recipe: compile the reference's own src/renderer.cu for the CPU.

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

Usage: python oracle/build_ref.py [--reference /root/reference]
Writes oracle/_ref/libisti_ref.so.  Exits 0 without building when the
reference tree is absent.
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LAUNCH_RE = re.compile(r"([A-Za-z_]\w*(?:\s*<[^<>;()]*>)?)\s*<<<(.*?)>>>")


def rewrite_launches(src: str) -> tuple[str, int]:
    return LAUNCH_RE.subn(lambda m: f"isti_refhost::launch({m.group(2)}, {m.group(1)})", src)


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
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    lib = build(args.reference, verbose=True)
    if lib:
        print(f"built {lib}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
