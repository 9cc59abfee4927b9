"""Seeded procedural keyframe sequences (synthetic stand-in for the reference's
Unity-recorded dataset, which is not available).

Scene: ground plane y = 0 plus ``n_spheres`` spheres (radius U[0.2, 1.5] m,
centre xz U[-10, 10]^2 at height r, albedo U[0, 1]^3, constant horizontal
velocity |v| <= max_speed), one directional light, Lambertian shading,
analytic soft shadows from a 2 deg sphere light.  Keyframes are ray-cast at
``keyframe_hz``; the camera follows a seeded path with at most ~1.5 deg
rotation and 5 cm translation per keyframe interval; the client camera is
the linear interpolation of that path at t = b / frames_per_anchor.

Buffers follow the conventions of the reference renderer's inputs: colour
RGBA8 (sRGB bytes), NDC z, object motion as an NDC delta to the other
keyframe under the view's own viewproj (stored as float16 xyz, the compact
form; ``View.motion_f32x4()`` widens it exactly to the reference's float4
layout), 2-bit soft-shadow levels packed in shadowInfo's RGB.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _build

MASK64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014): platform-independent seeded stream."""

    def __init__(self, seed: int):
        self.s = seed & MASK64

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, a: float, b: float) -> float:
        return a + (b - a) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


# ---------------------------------------------------------------- camera math

def perspective(fov_y_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """GL projection (NDC z in [-1, 1]) with image row 0 at the top (y flipped),
    the orientation the reference's loader produces for Unity captures."""
    f = 1.0 / math.tan(math.radians(fov_y_deg) / 2.0)
    return np.array([
        [f / aspect, 0.0, 0.0, 0.0],
        [0.0, -f, 0.0, 0.0],
        [0.0, 0.0, (far + near) / (near - far), 2.0 * far * near / (near - far)],
        [0.0, 0.0, -1.0, 0.0],
    ])


def look_dir(yaw: float, pitch: float) -> np.ndarray:
    return np.array([math.sin(yaw) * math.cos(pitch), math.sin(pitch), math.cos(yaw) * math.cos(pitch)])


def view_matrix(eye: np.ndarray, yaw: float, pitch: float) -> np.ndarray:
    f = look_dir(yaw, pitch)
    s = np.cross(f, [0.0, 1.0, 0.0])
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    return np.array([
        [s[0], s[1], s[2], -s @ eye],
        [u[0], u[1], u[2], -u @ eye],
        [-f[0], -f[1], -f[2], f @ eye],
        [0.0, 0.0, 0.0, 1.0],
    ])


def right_vector(yaw: float, pitch: float) -> np.ndarray:
    s = np.cross(look_dir(yaw, pitch), [0.0, 1.0, 0.0])
    return s / np.linalg.norm(s)


@dataclass
class Pose:
    eye: np.ndarray
    yaw: float
    pitch: float

    def lerp(self, o: "Pose", s: float) -> "Pose":
        return Pose(self.eye + (o.eye - self.eye) * s, self.yaw + (o.yaw - self.yaw) * s, self.pitch + (o.pitch - self.pitch) * s)


# ---------------------------------------------------------------- data model

@dataclass
class View:
    """One camera at one keyframe, as consumed for one direction of a pair
    (reference MotionZBufferImage, include/data.h:12-62)."""
    color: np.ndarray                  # (H, W, 4) uint8
    z: np.ndarray                      # (H, W) float32, NDC z
    motion: np.ndarray | None          # (H, W, 3) float16 NDC delta, or None
    shadow_a: np.ndarray | None = None     # (H, W, 4) uint8
    shadow_b: np.ndarray | None = None
    shadow_info: np.ndarray | None = None
    viewproj: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    inv_viewproj: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))

    @property
    def width(self) -> int:
        return int(self.z.shape[1])

    @property
    def height(self) -> int:
        return int(self.z.shape[0])

    def motion_f32x4(self) -> np.ndarray | None:
        if self.motion is None:
            return None
        m = np.zeros(self.z.shape + (4,), np.float32)
        m[..., :3] = self.motion.astype(np.float32)
        return m

    def nbytes(self) -> int:
        n = self.color.nbytes + self.z.nbytes + (self.motion.nbytes if self.motion is not None else 0)
        for a in (self.shadow_a, self.shadow_b, self.shadow_info):
            n += a.nbytes if a is not None else 0
        return n


@dataclass
class Frame:
    """Reference FrameData (include/data.h:79-116)."""
    fwd: View
    bwd: View
    aux_curr: list[View] = field(default_factory=list)
    aux_next: list[View] = field(default_factory=list)
    aux_priority: list[int] = field(default_factory=list)

    def views(self) -> list[View]:
        out = [self.fwd, self.bwd]
        for a, b in zip(self.aux_curr, self.aux_next):
            out += [a, b]
        return out


@dataclass
class Client:
    """Reference RenderInfo + AdditionalRenderInfo (include/renderer.h:18-35)."""
    width: int
    height: int
    alpha: float
    viewproj: np.ndarray
    inv_viewproj: np.ndarray
    frames_per_anchor: int = 4
    shadow_frames_per_anchor: int = 4
    no_shadows: bool = False
    mode: int = 0


# ---------------------------------------------------------------- generator binding

class _Sphere(C.Structure):
    _fields_ = [("cx", C.c_double), ("cz", C.c_double), ("r", C.c_double), ("vx", C.c_double), ("vz", C.c_double),
                ("albedo", C.c_double * 3)]


class _SceneDesc(C.Structure):
    _fields_ = [("n_spheres", C.c_int32), ("spheres", C.POINTER(_Sphere)), ("light_dir", C.c_double * 3),
                ("light_radius_deg", C.c_double)]


class _SceneCam(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("viewproj", C.c_double * 16),
                ("inv_viewproj", C.c_double * 16), ("t0", C.c_double), ("dt", C.c_double), ("sfpa", C.c_int32)]


class _SceneOut(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("color", "z", "motion_fwd", "motion_bwd", "shadow_a_fwd", "shadow_b_fwd",
                                          "shadow_info_fwd", "shadow_a_bwd", "shadow_b_bwd", "shadow_info_bwd")]


_scene_lib = None


def _lib():
    global _scene_lib
    if _scene_lib is None:
        p = _build.scene_lib_path()
        if not os.path.exists(p):
            _build.build_all()
        _scene_lib = C.CDLL(p)
        _scene_lib.isti_scene_render.argtypes = [C.POINTER(_SceneDesc), C.POINTER(_SceneCam), C.POINTER(_SceneOut)]
        _scene_lib.isti_scene_render.restype = C.c_int
    return _scene_lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _cm(m: np.ndarray):
    return (C.c_double * 16)(*np.asarray(m, np.float64).T.reshape(-1).tolist())


@dataclass
class Keyframe:
    """Raw ray-cast buffers of one camera at one keyframe (both directions)."""
    color: np.ndarray
    z: np.ndarray
    motion_fwd: np.ndarray
    motion_bwd: np.ndarray
    shadow_fwd: tuple | None
    shadow_bwd: tuple | None
    viewproj: np.ndarray      # float64
    pose: Pose


class Sequence:
    """Keyframes of a seeded scene for a main camera and optional aux cameras."""

    def __init__(self, width: int, height: int, n_keyframes: int, seed: int = 1, n_spheres: int = 64,
                 max_speed: float = 0.5, aux_offsets: tuple[float, ...] = (), aux_size: tuple[int, int] | None = None,
                 shadows: bool = False, frames_per_anchor: int = 4, shadow_frames_per_anchor: int = 4,
                 keyframe_hz: float = 30.0, fov_y_deg: float = 90.0, near: float = 0.1, far: float = 100.0,
                 max_rot_deg: float = 1.2, max_step_m: float = 0.05):
        self.width, self.height = width, height
        self.n_keyframes = n_keyframes
        self.seed = seed
        self.shadows = shadows
        self.fpa = frames_per_anchor
        self.sfpa = shadow_frames_per_anchor
        self.dt = 1.0 / keyframe_hz
        self.aux_offsets = tuple(aux_offsets)
        self.aux_size = aux_size or (width, height)
        rng = SplitMix64(seed)
        spheres = []
        for _ in range(n_spheres):
            r = rng.uniform(0.2, 1.5)
            cx, cz = rng.uniform(-10.0, 10.0), rng.uniform(-10.0, 10.0)
            sp = rng.uniform(0.0, max_speed)
            ang = rng.uniform(0.0, 2.0 * math.pi)
            alb = [rng.uniform(0.0, 1.0) for _ in range(3)]
            spheres.append((cx, cz, r, sp * math.cos(ang), sp * math.sin(ang), alb))
        self._spheres = (_Sphere * max(1, n_spheres))()
        for i, (cx, cz, r, vx, vz, alb) in enumerate(spheres):
            self._spheres[i] = _Sphere(cx, cz, r, vx, vz, (C.c_double * 3)(*alb))
        ld = np.array([0.45, 0.8, 0.35])
        ld /= np.linalg.norm(ld)
        self._desc = _SceneDesc(n_spheres, self._spheres, (C.c_double * 3)(*ld.tolist()), 2.0)
        self.proj_main = perspective(fov_y_deg, width / height, near, far)
        self.proj_aux = perspective(fov_y_deg, self.aux_size[0] / self.aux_size[1], near, far)
        # camera path
        poses = [Pose(np.array([0.0, 2.5, -15.0]), 0.0, math.radians(-8.0))]
        for _ in range(n_keyframes - 1):
            p = poses[-1]
            dyaw = math.radians(rng.uniform(-max_rot_deg, max_rot_deg))
            dpitch = math.radians(rng.uniform(-max_rot_deg, max_rot_deg)) * 0.5
            d = np.array([rng.uniform(-1, 1), rng.uniform(-0.3, 0.3), rng.uniform(-1, 1)])
            d = d / max(1e-9, np.linalg.norm(d)) * rng.uniform(0.0, max_step_m)
            poses.append(Pose(p.eye + d, p.yaw + dyaw, p.pitch + dpitch))
        self.poses = poses
        self._cache: dict[tuple[int, int], Keyframe] = {}

    # camera c = 0 main, c = 1.. aux
    def _cam_pose(self, pose: Pose, c: int) -> Pose:
        if c == 0:
            return pose
        off = self.aux_offsets[c - 1]
        return Pose(pose.eye + right_vector(pose.yaw, pose.pitch) * off, pose.yaw, pose.pitch)

    def keyframe(self, k: int, c: int) -> Keyframe:
        key = (k, c)
        if key in self._cache:
            return self._cache[key]
        pose = self._cam_pose(self.poses[k], c)
        w, h = (self.width, self.height) if c == 0 else self.aux_size
        proj = self.proj_main if c == 0 else self.proj_aux
        vp = proj @ view_matrix(pose.eye, pose.yaw, pose.pitch)
        ivp = np.linalg.inv(vp)
        cam = _SceneCam(w, h, _cm(vp), _cm(ivp), k * self.dt, self.dt, self.sfpa if self.shadows else 0)
        color = np.zeros((h, w, 4), np.uint8)
        z = np.zeros((h, w), np.float32)
        mf = np.zeros((h, w, 3), np.float32)
        mb = np.zeros((h, w, 3), np.float32)
        sh = [np.zeros((h, w, 4), np.uint8) for _ in range(6)] if self.shadows else [None] * 6
        out = _SceneOut(_ptr(color), _ptr(z), _ptr(mf), _ptr(mb), *[_ptr(a) for a in sh])
        _lib().isti_scene_render(C.byref(self._desc), C.byref(cam), C.byref(out))
        kf = Keyframe(color, z, mf.astype(np.float16), mb.astype(np.float16),
                      tuple(sh[:3]) if self.shadows else None, tuple(sh[3:]) if self.shadows else None, vp, pose)
        self._cache[key] = kf
        return kf

    def _view(self, kf: Keyframe, forward: bool) -> View:
        vp32 = kf.viewproj.astype(np.float32)
        ivp32 = np.linalg.inv(kf.viewproj).astype(np.float32)
        sh = kf.shadow_fwd if forward else kf.shadow_bwd
        return View(kf.color, kf.z, kf.motion_fwd if forward else kf.motion_bwd,
                    sh[0] if sh else None, sh[1] if sh else None, sh[2] if sh else None, vp32, ivp32)

    def frame(self, k: int) -> Frame:
        """FrameData for the keyframe pair (k, k + 1)."""
        fr = Frame(self._view(self.keyframe(k, 0), True), self._view(self.keyframe(k + 1, 0), False))
        prio = 2 + (1 if self.shadows else 0)  # objectMotion * 2 + shadowGradients, src/file_reader.cu:102-104
        for c in range(1, 1 + len(self.aux_offsets)):
            fr.aux_curr.append(self._view(self.keyframe(k, c), True))
            fr.aux_next.append(self._view(self.keyframe(k + 1, c), False))
            fr.aux_priority.append(prio)
        return fr

    def ground_truth(self, k: int, b: int) -> np.ndarray:
        """RGBA8 colour ray-cast for the client camera of (k, b) at its own time,
        (k + b / frames_per_anchor) keyframe intervals: the frame that
        interpolation approximates (the procedural scene makes it exact)."""
        t = b / self.fpa
        pose = self.poses[k].lerp(self.poses[min(k + 1, self.n_keyframes - 1)], t)
        vp = self.proj_main @ view_matrix(pose.eye, pose.yaw, pose.pitch)
        w, h = self.width, self.height
        cam = _SceneCam(w, h, _cm(vp), _cm(np.linalg.inv(vp)), (k + t) * self.dt, self.dt, 0)
        color = np.zeros((h, w, 4), np.uint8)
        z = np.zeros((h, w), np.float32)
        mf = np.zeros((h, w, 3), np.float32)
        mb = np.zeros((h, w, 3), np.float32)
        out = _SceneOut(_ptr(color), _ptr(z), _ptr(mf), _ptr(mb), *([None] * 6))
        _lib().isti_scene_render(C.byref(self._desc), C.byref(cam), C.byref(out))
        return color

    def client(self, k: int, b: int, mode: int = 0, no_shadows: bool = False, alpha: float | None = None) -> Client:
        """Client camera at t = b / frames_per_anchor between keyframes k and k + 1."""
        t = b / self.fpa if alpha is None else alpha
        pose = self.poses[k].lerp(self.poses[min(k + 1, self.n_keyframes - 1)], t)
        vp = self.proj_main @ view_matrix(pose.eye, pose.yaw, pose.pitch)
        return Client(self.width, self.height, float(np.float32(t)), vp.astype(np.float32),
                      np.linalg.inv(vp).astype(np.float32), self.fpa, self.sfpa,
                      no_shadows, mode)
