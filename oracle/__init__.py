"""Oracle for the interpolation path — TEST INFRASTRUCTURE ONLY.

Two CPU implementations of the reference renderer's per-frame path:

* ``run_oracle``: isti_oracle.c, a plain C restatement of src/renderer.cu
  (built into oracle/_build/ by ``build()``, here and on the GPU host);
* ``run_reference``: the reference's own src/renderer.cu compiled for the CPU
  by build_ref.py (oracle/_ref/, only where the reference tree exists);
* ``run_reference_gpu`` / ``time_reference_gpu``: the same renderer.cu compiled
  for the GPU with the reference's CUDA flags (-use_fast_math), from the copy
  build_ref.py stages under oracle/_ref/gpu/ (oracle/_ref/libisti_ref_gpu.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline/reference
legs use this package, as the checker or as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(BUILD_DIR, "libisti_oracle.so")
REF_LIB = os.path.join(REF_DIR, "libisti_ref.so")
REF_GPU_LIB = os.path.join(REF_DIR, "libisti_ref_gpu.so")

Mat16 = C.c_float * 16


class OracleView(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("color", C.c_void_p), ("z", C.c_void_p), ("motion", C.c_void_p),
        ("shadow_color_a", C.c_void_p), ("shadow_color_b", C.c_void_p), ("shadow_info", C.c_void_p),
        ("viewproj", Mat16), ("inv_viewproj", Mat16),
    ]


class OracleFrame(C.Structure):
    _fields_ = [("fwd", OracleView), ("bwd", OracleView), ("num_aux", C.c_int32),
                ("aux_curr", C.POINTER(OracleView)), ("aux_next", C.POINTER(OracleView)),
                ("aux_priority", C.POINTER(C.c_int32))]


class OracleRenderInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("alpha", C.c_float),
                ("viewproj", Mat16), ("inv_viewproj", Mat16),
                ("frames_per_anchor", C.c_int32), ("shadow_frames_per_anchor", C.c_int32),
                ("no_shadows", C.c_int32), ("mode", C.c_int32)]


class OracleViewOut(C.Structure):
    _fields_ = [("splat", C.c_void_p), ("cam_ff", C.c_void_p), ("full_ff", C.c_void_p)]


def build(verbose: bool = False) -> None:
    """Compile isti_oracle.c, and the reference's renderer when its tree is present."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "isti_oracle.c"), os.path.join(HERE, "isti_oracle_glm.c")]
    hdr = os.path.join(HERE, "isti_oracle.h")
    if not os.path.exists(ORACLE_LIB) or max(os.path.getmtime(p) for p in srcs + [hdr]) > os.path.getmtime(ORACLE_LIB):
        cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", *srcs, "-o", ORACLE_LIB, "-lm"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    from . import build_ref
    ref = os.environ.get("ISTI_REFERENCE_DIR")
    if ref:
        build_ref.build(ref, verbose=verbose)
    build_ref.build_gpu(verbose=verbose)


def mat16(m) -> Mat16:
    a = np.asarray(m, dtype=np.float32).reshape(4, 4)
    return Mat16(*a.T.reshape(-1).tolist())


def _p(a):
    return None if a is None else a.ctypes.data


class _Marshal:
    """Keeps the numpy buffers alive while a C call runs."""

    def __init__(self, frame, client):
        self.keep = []
        self.frame = OracleFrame()
        self.frame.fwd = self.view(frame.fwd)
        self.frame.bwd = self.view(frame.bwd)
        n = len(frame.aux_curr)
        self.frame.num_aux = n
        self.curr = (OracleView * max(1, n))(*[self.view(v) for v in frame.aux_curr])
        self.next = (OracleView * max(1, n))(*[self.view(v) for v in frame.aux_next])
        self.prio = (C.c_int32 * max(1, n))(*frame.aux_priority)
        self.frame.aux_curr = C.cast(self.curr, C.POINTER(OracleView))
        self.frame.aux_next = C.cast(self.next, C.POINTER(OracleView))
        self.frame.aux_priority = C.cast(self.prio, C.POINTER(C.c_int32))
        self.info = OracleRenderInfo(client.width, client.height, client.alpha, mat16(client.viewproj),
                                     mat16(client.inv_viewproj), client.frames_per_anchor,
                                     client.shadow_frames_per_anchor, int(client.no_shadows), client.mode)

    def view(self, v) -> OracleView:
        arrs = [np.ascontiguousarray(v.color), np.ascontiguousarray(v.z, dtype=np.float32), v.motion_f32x4(),
                None if v.shadow_a is None else np.ascontiguousarray(v.shadow_a),
                None if v.shadow_b is None else np.ascontiguousarray(v.shadow_b),
                None if v.shadow_info is None else np.ascontiguousarray(v.shadow_info)]
        self.keep += arrs
        return OracleView(v.width, v.height, *[_p(a) for a in arrs], mat16(v.viewproj), mat16(v.inv_viewproj))


def _outs(frame):
    views = frame.views()
    splats = [np.zeros((v.height, v.width), np.uint64) for v in views]
    cam = [np.zeros((v.height, v.width, 4), np.float32) for v in views]
    full = [np.zeros((v.height, v.width, 4), np.float32) for v in views]
    arr = (OracleViewOut * len(views))(*[OracleViewOut(_p(s), _p(c), _p(f)) for s, c, f in zip(splats, cam, full)])
    return arr, splats, cam, full


_libs: dict[str, C.CDLL] = {}


def _load(path: str, sym: str) -> C.CDLL:
    if path not in _libs:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} not built")
        lib = C.CDLL(path)
        fn = getattr(lib, sym)
        fn.restype = C.c_int
        _libs[path] = lib
    return _libs[path]


def reference_available() -> bool:
    return os.path.exists(REF_LIB)


def run_oracle(frame, client, prev_out=None, nthreads: int = 0, with_intermediates: bool = True):
    """C oracle.  Returns (out RGBA8 (H,W,4), splats, cam_ffs, full_ffs) — the
    last three are per-view lists (None when with_intermediates is False)."""
    lib = _load(ORACLE_LIB, "oracle_render")
    m = _Marshal(frame, client)
    out = np.zeros((client.height, client.width, 4), np.uint8) if prev_out is None else np.array(prev_out, np.uint8, copy=True)
    outs, splats, cam, full = _outs(frame) if with_intermediates else (None, None, None, None)
    rc = lib.oracle_render(C.byref(m.frame), C.byref(m.info), C.c_void_p(out.ctypes.data),
                           outs if outs is not None else None, C.c_int(nthreads))
    if rc != 0:
        raise ValueError("oracle_render rejected its arguments")
    return out, splats, cam, full


def prepared_call(frame, client, prev_out=None, nthreads: int = 0):
    """Marshals once and returns a zero-argument callable that runs only the C
    oracle on these inputs (for timing the CPU baseline)."""
    lib = _load(ORACLE_LIB, "oracle_render")
    m = _Marshal(frame, client)
    out = np.zeros((client.height, client.width, 4), np.uint8) if prev_out is None else np.array(prev_out, np.uint8, copy=True)

    def call():
        if lib.oracle_render(C.byref(m.frame), C.byref(m.info), C.c_void_p(out.ctypes.data), None, C.c_int(nthreads)) != 0:
            raise ValueError("oracle_render rejected its arguments")
        return out

    call.keep = (m, out)
    return call


def run_reference(frame, client, prev_out=None):
    """The reference's own renderer.cu, executed on the CPU (oracle/_ref)."""
    lib = _load(REF_LIB, "isti_ref_render")
    m = _Marshal(frame, client)
    out = np.zeros((client.height, client.width, 4), np.uint8) if prev_out is None else np.array(prev_out, np.uint8, copy=True)
    outs, splats, cam, full = _outs(frame)
    rc = lib.isti_ref_render(C.byref(m.frame), C.byref(m.info), C.c_void_p(out.ctypes.data), outs)
    if rc != 0:
        raise RuntimeError("reference renderer failed")
    return out, splats, cam, full


def reference_gpu_available() -> bool:
    return os.path.exists(REF_GPU_LIB)


def run_reference_gpu(frame, client, prev_out=None):
    """The reference's own renderer.cu built for the GPU with -use_fast_math, on the
    current CUDA device.  Returns (out, splats, cam_ffs, full_ffs) like run_reference."""
    lib = _load(REF_GPU_LIB, "isti_refgpu_render")
    m = _Marshal(frame, client)
    out = np.zeros((client.height, client.width, 4), np.uint8) if prev_out is None else np.array(prev_out, np.uint8, copy=True)
    outs, splats, cam, full = _outs(frame)
    rc = lib.isti_refgpu_render(C.byref(m.frame), C.byref(m.info), C.c_void_p(out.ctypes.data), outs)
    if rc != 0:
        raise RuntimeError("reference GPU renderer failed")
    return out, splats, cam, full


def time_reference_gpu(frame, clients, warmup: int = 3, repeats: int = 10) -> np.ndarray:
    """Per-call device milliseconds of the reference's Renderer::render on the GPU:
    one Renderer and FrameData kept alive, `warmup` untimed rounds, then `repeats`
    rounds over the client frames, each call bracketed by CUDA events on the legacy
    default stream.  Returns an array of repeats * len(clients) times."""
    lib = _load(REF_GPU_LIB, "isti_refgpu_time")
    lib.isti_refgpu_time.restype = C.c_int
    m = _Marshal(frame, clients[0])
    infos = (OracleRenderInfo * len(clients))(*[
        OracleRenderInfo(c.width, c.height, c.alpha, mat16(c.viewproj), mat16(c.inv_viewproj), c.frames_per_anchor,
                         c.shadow_frames_per_anchor, int(c.no_shadows), c.mode) for c in clients])
    ms = np.zeros(repeats * len(clients), np.float32)
    rc = lib.isti_refgpu_time(C.byref(m.frame), infos, C.c_int(len(clients)), C.c_int(warmup), C.c_int(repeats),
                              C.c_void_p(ms.ctypes.data))
    if rc != 0:
        raise RuntimeError("reference GPU timing failed")
    return ms
