"""The C-ABI library (CPU checks: no kernel is launched).

libisti.so must load, export every function include/isti.h declares, agree
with the ctypes struct layouts, and reject bad arguments before any CUDA work.
"""
import ctypes as C
import os
import re
import subprocess

import pytest

from imagebasedspatiotemporalinterpolation_gb300 import _build, native

HEADER = os.path.join(_build.INCLUDE, "isti.h")
HEADERS = [os.path.join(_build.INCLUDE, h) for h in ("isti.h", "isti_io.h", "isti_dataset.h", "isti_metrics.h", "isti_unet.h",
                                                    "isti_train.h")]


def declared_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for m in re.finditer(r"\b(isti_[a-z_]+)\s*\(", text):
        names.add(m.group(1))
    return sorted(names)


def test_header_declares_expected_entry_points():
    names = declared_functions(HEADER)
    for n in ("isti_renderer_create", "isti_renderer_destroy", "isti_render", "isti_renderer_view_buffers"):
        assert n in names


@pytest.mark.parametrize("header", HEADERS, ids=os.path.basename)
def test_library_exports_every_declared_symbol(built, header):
    lib = C.CDLL(_build.cuda_lib_path())
    declared = declared_functions(header)
    assert declared
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert set(declared) <= set(native.ALL_SIGNATURES), "ctypes signatures incomplete"


def test_struct_layout_matches_header(built, tmp_path):
    prog = tmp_path / "layout.c"
    structs = {"isti_view": native.IstiView, "isti_frame_data": native.IstiFrameData,
               "isti_render_info": native.IstiRenderInfo, "isti_timing": native.IstiTiming,
               "isti_camera_info": native.IstiCameraInfo, "isti_camera_frame": native.IstiCameraFrame,
               "isti_quality": native.IstiQuality, "isti_tuning": native.IstiTuning,
               "isti_pair_frames": native.IstiPairFrames}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "isti.h"', '#include "isti_dataset.h"',
             '#include "isti_metrics.h"', "int main(void){"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    prog.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", _build.INCLUDE, str(prog), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"


def test_argument_validation_without_device(built):
    lib = native.load()
    assert lib.isti_abi_version() == 1
    assert lib.isti_status_string(native.ISTI_ERR_INVALID_ARG) == b"invalid argument"
    assert lib.isti_renderer_create(None) == native.ISTI_ERR_INVALID_ARG
    assert lib.isti_render(None, None, None, None, None) == native.ISTI_ERR_INVALID_ARG
    assert b"NULL" in lib.isti_last_error()
    assert lib.isti_renderer_destroy(None) == native.ISTI_OK
    assert lib.isti_renderer_view_buffers(None, 0, None, None, None, None, None) == native.ISTI_ERR_INVALID_ARG
    assert lib.isti_renderer_set_pair_units(None, 16, 64) == native.ISTI_ERR_INVALID_ARG
    assert lib.isti_renderer_set_autotune(None, 1) == native.ISTI_ERR_INVALID_ARG
    assert lib.isti_renderer_set_reproj_launch(None, 48, 1, 0) == native.ISTI_ERR_INVALID_ARG
    assert lib.isti_renderer_tuning_count(None, None) == native.ISTI_ERR_INVALID_ARG
    assert lib.isti_renderer_tuning(None, 0, None) == native.ISTI_ERR_INVALID_ARG


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="missing"):
        native.load(str(tmp_path / "libisti.so"))
