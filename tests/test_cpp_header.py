"""The C++ drop-in header (include/isti_renderer.hpp) over the C ABI.

tests/cpp/frame_loop_hpp.cpp is a frame loop written against the header with
the reference's names (FrameData, MotionZBufferImage, ImageBuffer, RenderInfo,
Renderer::render; src/main.cu's usage).  Here it is compiled and linked
against libisti.so (CPU), then run on keyframes written to files and its PNG
output compared with the oracle bit for bit (GPU).
"""
import dataclasses
import os
import subprocess

import numpy as np
import pytest

import oracle
from imagebasedspatiotemporalinterpolation_gb300 import _build, files
from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "frame_loop_hpp.cpp")


def compile_program(src: str, out_dir: str) -> str:
    exe = os.path.join(out_dir, os.path.splitext(os.path.basename(src))[0])
    cmd = [_build._nvcc(), "-std=c++20", "-O2", _build.CUDA_ARCH, "-I", _build.INCLUDE, src, "-o", exe,
           "-L", _build.LIB_DIR, "-listi", "-Xlinker", "-rpath," + _build.LIB_DIR,
           "-Xcompiler", "-Wall,-Wextra,-Werror"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.fixture(scope="module")
def frame_loop_exe(built, tmp_path_factory):
    return compile_program(SRC, str(tmp_path_factory.mktemp("hpp_build")))


def test_header_compiles_and_links(frame_loop_exe):
    assert os.access(frame_loop_exe, os.X_OK)


def test_header_error_behaviour(built, tmp_path):
    """Render failures are printed and execution continues (the reference's
    CUDA_CHECK_THROW); resize to another size and unreadable files throw."""
    exe = compile_program(os.path.join(ROOT, "tests", "cpp", "errors_hpp.cpp"), str(tmp_path))
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120, cwd=str(tmp_path))
    assert res.returncode == 0, res.stdout + res.stderr
    out = res.stdout
    assert "isti | Renderer::render failed with error:" in out
    assert "render status 0" not in out
    assert "resize threw: Resizing of ImageBuffer currently not supported" in out
    assert "read threw: Could not load image does_not_exist.png" in out
    assert "exr read threw: Error loading EXR file does_not_exist.exr" in out


def test_header_is_self_contained(tmp_path):
    """The header compiles on its own with the host compiler (no nvcc, no CUDA sources)."""
    src = tmp_path / "only_header.cpp"
    src.write_text('#include "isti_renderer.hpp"\nint main() { isti::RenderInfo i{}; return int(i.alpha); }\n')
    res = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Wextra", "-Wpedantic", "-Werror",
                          "-I", _build.INCLUDE, "-I", os.path.join(_build._cuda_home(), "include"), str(src)],
                         capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr


def _fmt(m) -> str:
    return " ".join("%.9g" % float(v) for v in np.asarray(m, np.float32).T.reshape(-1))  # column-major


def write_case(case_dir: str, pairs, fill=(0, 0, 0, 0)) -> None:
    """pairs: [(Frame, [Client, ...]), ...] -> case.txt + image files read by frame_loop_hpp."""
    first = pairs[0][0]
    lines = [f"{first.fwd.width} {first.fwd.height} {len(first.aux_curr)} {' '.join(map(str, fill))}"]
    for v, prio in zip(first.aux_curr, first.aux_priority):
        lines.append(f"{v.width} {v.height} {prio}")
    lines.append(str(len(pairs)))
    for p, (frame, clients) in enumerate(pairs):
        for k, view in enumerate(frame.views()):
            stem = os.path.join(case_dir, f"p{p}_v{k}_")
            files.write_png(stem + "color.png", view.color)
            files.write_exr(stem + "z.exr", view.z)
            has_motion = view.motion is not None
            has_shadows = view.shadow_a is not None
            if has_motion:
                files.write_exr(stem + "motion.exr", view.motion_f32x4(), zip_compression=False)
            if has_shadows:
                files.write_png(stem + "shadowA.png", view.shadow_a)
                files.write_png(stem + "shadowB.png", view.shadow_b)
                files.write_png(stem + "shadowInfo.png", view.shadow_info)
            lines.append(f"{int(has_motion)} {int(has_shadows)} {_fmt(view.viewproj)} {_fmt(view.inv_viewproj)}")
        lines.append(str(len(clients)))
        for c in clients:
            lines.append(f"{c.mode} {'%.9g' % c.alpha} {c.frames_per_anchor} {c.shadow_frames_per_anchor} "
                         f"{int(c.no_shadows)} {_fmt(c.viewproj)} {_fmt(c.inv_viewproj)}")
    with open(os.path.join(case_dir, "case.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")


def expected_frames(pairs, fill):
    first = pairs[0][0].fwd
    prev = np.empty((first.height, first.width, 4), np.uint8)
    prev[...] = np.asarray(fill, np.uint8)
    out = []
    for frame, clients in pairs:
        for c in clients:
            prev = oracle.run_oracle(frame, c, prev, with_intermediates=False)[0]
            out.append(prev.copy())
    return out


def run_case(exe, tmp_path, pairs, fill):
    case_dir, out_dir = tmp_path / "case", tmp_path / "out"
    case_dir.mkdir()
    out_dir.mkdir()
    write_case(str(case_dir), pairs, fill)
    res = subprocess.run([exe, str(case_dir), str(out_dir)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    want = expected_frames(pairs, fill)
    assert res.stdout.strip() == f"frames {len(want)}"
    for i, w in enumerate(want):
        got = files.read_png(str(out_dir / f"{i:04d}.png"))
        diff = (got != w).any(-1)
        assert not diff.any(), f"frame {i}: {int(diff.sum())} pixels differ"
    z = pairs[-1][0].fwd.z
    assert np.array_equal(files.read_exr(str(out_dir / "last_z.exr")), z)
    avg = float.fromhex(open(out_dir / "average_z.txt").read().strip())
    assert abs(avg - float(np.mean(z, dtype=np.float64))) <= 1e-6 * max(1.0, abs(avg))  # float32 result


@pytest.mark.gpu
def test_frame_loop_aux_shadows_two_pairs(cuda, frame_loop_exe, tmp_path):
    """Two keyframe pairs (FrameData::swap between them), two aux cameras, soft shadows, modes 0 and 1."""
    seq = Sequence(160, 90, 3, seed=91, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0, n_spheres=40)
    pairs = []
    for k in range(2):
        clients = [seq.client(k, b, mode=(b % 2)) for b in range(seq.fpa)]
        pairs.append((seq.frame(k), clients))
    run_case(frame_loop_exe, tmp_path, pairs, fill=(7, 8, 9, 255))


@pytest.mark.gpu
def test_frame_loop_optional_images_and_modes(cuda, frame_loop_exe, tmp_path):
    """Absent object motion / shadow images (std::nullopt), re-emplaced in the next pair; modes 2, 3 and 4."""
    seq = Sequence(132, 78, 3, seed=92, aux_offsets=(0.3,), aux_size=(66, 39), shadows=True, max_speed=2.0)
    f0 = seq.frame(0)
    f0 = dataclasses.replace(f0, fwd=dataclasses.replace(f0.fwd, motion=None),
                             aux_next=[dataclasses.replace(v, shadow_a=None, shadow_b=None, shadow_info=None)
                                       for v in f0.aux_next])
    pairs = [(f0, [seq.client(0, b, mode=m) for b, m in ((1, 2), (2, 3), (3, 4))]),
             (seq.frame(1), [seq.client(1, b, mode=m) for b, m in ((0, 3), (2, 2), (3, 4))])]
    run_case(frame_loop_exe, tmp_path, pairs, fill=(200, 0, 100, 50))
