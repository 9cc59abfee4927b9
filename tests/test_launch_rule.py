"""The reprojection's fixed launch rule (csrc/isti_launch.cuh), built for the host with nvcc
and run without a device (the per-SM limits then default to the GB300's): the register cap
and row pairs of each shape class, including the classes where shared memory, not
registers, bounds the resident blocks."""
import os
import subprocess

import pytest

from imagebasedspatiotemporalinterpolation_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_launch_rule_per_shape_class(tmp_path):
    nvcc = _build._nvcc()
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "launch_rule_test")
    cmd = [nvcc, "-std=c++20", "-O1", _build.CUDA_ARCH, "-I", _build.INCLUDE, "-I", _build.CSRC,
           os.path.join(ROOT, "tests", "cpp", "launch_rule_test.cu"), "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")  # the GB300 defaults, also on a GPU host
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120, env=env)
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.startswith("ok "), res.stdout
