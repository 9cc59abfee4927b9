"""ORACLE (test infrastructure only): the reference's client frame loop.

Restates src/main.cu:118-191 (the splinter loop: latency, hold-last,
holes-black, t > 1 before a late keyframe, keyframe reads at b == latency or
at the end of the interval), FrameFileReader's keyframe double buffer
(src/file_reader.cu:109-217, include/data.h:79-116: swap, then load unless
the sequence is exhausted) and the glm matrix steps of the loop through the C
restatement in isti_oracle_glm.c.  Every frame is rendered by the C oracle
(``run_oracle``).

Inputs are plain arrays, so the checker does not depend on any decoder: a
``Keyframes`` object holds, per camera and keyframe, what the dataset files
contain after loading (colour, z after convertDepthToZ, float4 motion of each
direction, shadow images, w2c and the raw projection).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import ORACLE_LIB, _load, run_oracle


def _glm():
    lib = _load(ORACLE_LIB, "oracle_render")
    f16 = C.POINTER(C.c_float)
    lib.oracle_mat4_mul.argtypes = [f16, f16, f16]
    lib.oracle_mat4_inverse.argtypes = [f16, f16]
    lib.oracle_mat4_interpolate.argtypes = [f16, f16, C.c_float, f16]
    lib.oracle_normalize_proj.argtypes = [f16, f16]
    for n in ("oracle_mat4_mul", "oracle_mat4_inverse", "oracle_mat4_interpolate", "oracle_normalize_proj"):
        getattr(lib, n).restype = None
    return lib


def _cm(m: np.ndarray):
    """row-major (4, 4) -> column-major float[16]"""
    return (C.c_float * 16)(*np.asarray(m, np.float32).T.reshape(-1).tolist())


def _rm(a) -> np.ndarray:
    return np.array(list(a), np.float32).reshape(4, 4).T.copy()


def mat_mul(a, b) -> np.ndarray:
    out = (C.c_float * 16)()
    _glm().oracle_mat4_mul(_cm(a), _cm(b), out)
    return _rm(out)


def mat_inverse(m) -> np.ndarray:
    out = (C.c_float * 16)()
    _glm().oracle_mat4_inverse(_cm(m), out)
    return _rm(out)


def mat_interpolate(m1, m2, t: float) -> np.ndarray:
    out = (C.c_float * 16)()
    _glm().oracle_mat4_interpolate(_cm(m1), _cm(m2), C.c_float(t), out)
    return _rm(out)


def normalize_proj(p) -> np.ndarray:
    out = (C.c_float * 16)()
    _glm().oracle_normalize_proj(_cm(p), out)
    return _rm(out)


@dataclass
class CamKeyframe:
    """One camera at one keyframe as loaded (MotionZBufferImage contents)."""
    color: np.ndarray
    z: np.ndarray                       # after convertDepthToZ
    w2c: np.ndarray                     # row-major float32
    proj_raw: np.ndarray                # as stored in cam.json
    motion_fwd: np.ndarray | None = None    # (H, W, 4) float32 to keyframe k + 1 (None: folder absent)
    motion_bwd: np.ndarray | None = None    # (H, W, 4) float32 to keyframe k - 1, stored under k - 1's name
    shadow_fwd: tuple | None = None
    shadow_bwd: tuple | None = None


@dataclass
class Keyframes:
    cams: list[list[CamKeyframe]]       # [camera][keyframe], camera 0 = main
    priorities: list[int] = field(default_factory=list)  # aux cameras
    server_fps: int = 30
    shadow_fps: int = 120


@dataclass
class _Slot:
    w: int
    h: int
    color: np.ndarray
    z: np.ndarray
    motion: np.ndarray | None
    shadows: tuple | None
    view: np.ndarray
    proj: np.ndarray
    vp: np.ndarray
    ivp: np.ndarray

    @staticmethod
    def empty(w, h):
        # buffers the reference leaves unwritten until the first read start as zeros
        z4 = np.zeros((h, w, 4), np.uint8)
        zero = np.zeros((4, 4), np.float32)
        return _Slot(w, h, z4.copy(), np.zeros((h, w), np.float32), np.zeros((h, w, 4), np.float32),
                     (z4.copy(), z4.copy(), z4.copy()), zero, zero, zero, zero)


class _View:
    """Duck-typed scene.View for run_oracle."""

    def __init__(self, s: _Slot):
        self.color, self.z = s.color, s.z
        self._m = s.motion
        self.motion = s.motion
        self.shadow_a, self.shadow_b, self.shadow_info = s.shadows if s.shadows else (None, None, None)
        if self.shadow_a is not None and self.shadow_info is None:
            self.shadow_a = self.shadow_b = None
        self.viewproj, self.inv_viewproj = s.vp, s.ivp
        self.width, self.height = s.w, s.h

    def motion_f32x4(self):
        return self._m


class _Frame:
    def __init__(self, fwd, bwd, aux_curr, aux_next, prio):
        self.fwd, self.bwd, self.aux_curr, self.aux_next, self.aux_priority = fwd, bwd, aux_curr, aux_next, prio

    def views(self):
        out = [self.fwd, self.bwd]
        for a, b in zip(self.aux_curr, self.aux_next):
            out += [a, b]
        return out


class Reader:
    """FrameFileReader + FrameData (src/file_reader.cu:109-217, include/data.h:79-116)."""

    def __init__(self, kf: Keyframes):
        self.kf = kf
        self.curr = []
        self.next = []
        for cam in kf.cams:
            h, w = cam[0].z.shape
            self.curr.append(_Slot.empty(w, h))
            self.next.append(_Slot.empty(w, h))
        self.index = 0
        for c in range(len(kf.cams)):
            self._color_depth(c, 0)

    def _color_depth(self, c, k):
        src = self.kf.cams[c][k]
        s = self.next[c]
        s.color, s.z = src.color, src.z
        s.view = np.asarray(src.w2c, np.float32)
        s.proj = normalize_proj(src.proj_raw)
        s.vp = mat_mul(s.proj, s.view)
        s.ivp = mat_inverse(s.vp)

    def read_next(self) -> bool:
        self.curr, self.next = self.next, self.curr
        n = len(self.kf.cams[0])
        if self.index >= n - 1:
            return False
        k = self.index
        for c in range(len(self.kf.cams)):
            self._color_depth(c, k + 1)
            a, b = self.kf.cams[c][k], self.kf.cams[c][k + 1]
            self.curr[c].motion = a.motion_fwd
            self.next[c].motion = b.motion_bwd
            self.curr[c].shadows = a.shadow_fwd
            self.next[c].shadows = b.shadow_bwd
        self.index += 1
        return True

    def frame(self) -> _Frame:
        n_aux = len(self.kf.cams) - 1
        return _Frame(_View(self.curr[0]), _View(self.next[0]), [_View(self.curr[c]) for c in range(1, n_aux + 1)],
                      [_View(self.next[c]) for c in range(1, n_aux + 1)], list(self.kf.priorities))


@dataclass
class _Client:
    width: int
    height: int
    alpha: float
    viewproj: np.ndarray
    inv_viewproj: np.ndarray
    frames_per_anchor: int
    shadow_frames_per_anchor: int
    no_shadows: bool
    mode: int


def splinter(kf: Keyframes, width: int, height: int, mode: int = 0, latency: int = 0, hold_last: bool = False,
             no_shadows: bool = False, holes_black: bool = False, camera_path: dict | None = None):
    """The frames src/main.cu writes with -w, as a list of RGBA8 arrays (index =
    file number).  camera_path: {"client_fps", "frames": [{"w2c", "proj"}]} as
    read from the client cam.json (-c), or None for the interpolated client view."""
    reader = Reader(kf)
    total = len(camera_path["frames"]) if camera_path else 120 * 15
    client_fps = camera_path["client_fps"] if camera_path else 120
    fpa = client_fps // kf.server_fps
    sfpa = kf.shadow_fps // kf.server_fps
    out = np.zeros((height, width, 4), np.uint8)
    frames = []
    for i in range(0, total, fpa):
        for b in range(fpa):
            if latency == b:
                reader.read_next()
            frame_number = i + b + 1
            if frame_number > total:
                break
            t = np.float32(fpa + b if latency > b else b) / np.float32(fpa)
            if camera_path:
                view = camera_path["frames"][i + b]["w2c"]
                proj = normalize_proj(camera_path["frames"][i + b]["proj"])
            else:
                view = mat_interpolate(reader.curr[0].view, reader.next[0].view, float(t))
                proj = reader.curr[0].proj
            vp = mat_mul(proj, view)
            if holes_black:
                out = np.zeros_like(out)
            if not (b < latency and hold_last):
                client = _Client(width, height, float(t), vp, mat_inverse(vp), fpa, sfpa, no_shadows, mode)
                out, _, _, _ = run_oracle(reader.frame(), client, prev_out=out, with_intermediates=False)
            frames.append(out.copy())
            if latency > b and b == fpa - 1:
                reader.read_next()
    return frames
