"""The reprojection kernel keeps errors squared and compares them as their square roots
(csrc/isti_error_cmp.cuh).  Host build of the same header against sqrtf comparisons:
random and neighbouring bit patterns, squares of adjacent floats, +-0, +inf, NaN, the
marker of an unsearched direction (FLT_MAX in src/renderer.cu:204-215) and the EPS_1
thresholds."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "imagebasedspatiotemporalinterpolation_gb300", "csrc")


def test_squared_error_comparisons_match_square_roots(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "error_cmp_test")
    cmd = [gxx, "-std=c++20", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-I", CSRC,
           os.path.join(ROOT, "tests", "cpp", "error_cmp_test.cpp"), "-o", exe, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.startswith("ok "), res.stdout
