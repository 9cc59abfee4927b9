"""Dataset files through libisti (include/isti_io.h, include/isti_dataset.h).

Python mirror of the reference's file side: ``read_png`` / ``read_exr`` /
``write_png`` stand for ImageBuffer::readFromFile / writeToFile
(src/util/image_buffer.cu:103-200), ``read_camera_path`` for
FrameFileReader::initCamInfo (src/file_reader.cu:78-107) and ``Dataset`` for
FrameFileReader + FrameData (src/file_reader.cu:109-217, include/data.h).
Decoding runs in the native library; there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import native


def _lib():
    return native.load()


def read_png(path: str) -> np.ndarray:
    """RGBA8 image (H, W, 4) with stb_image's conversions for 4 channels."""
    lib = _lib()
    w, h, px = C.c_int32(), C.c_int32(), C.POINTER(C.c_uint8)()
    native.check(lib.isti_png_decode_file(os.fsencode(path), C.byref(w), C.byref(h), C.byref(px)))
    try:
        return np.ctypeslib.as_array(px, shape=(h.value, w.value, 4)).copy()
    finally:
        lib.isti_image_free(px)


def decode_png(data: bytes) -> np.ndarray:
    lib = _lib()
    w, h, px = C.c_int32(), C.c_int32(), C.POINTER(C.c_uint8)()
    buf = (C.c_uint8 * len(data)).from_buffer_copy(data)
    native.check(lib.isti_png_decode_memory(buf, len(data), C.byref(w), C.byref(h), C.byref(px)))
    try:
        return np.ctypeslib.as_array(px, shape=(h.value, w.value, 4)).copy()
    finally:
        lib.isti_image_free(px)


def read_exr(path: str) -> np.ndarray:
    """float32 (H, W) for a one-channel file, else (H, W, 4) RGBA (LoadEXR's mapping)."""
    lib = _lib()
    w, h, ch, px = C.c_int32(), C.c_int32(), C.c_int32(), C.POINTER(C.c_float)()
    native.check(lib.isti_exr_decode_file(os.fsencode(path), C.byref(w), C.byref(h), C.byref(ch), C.byref(px)))
    try:
        shape = (h.value, w.value) if ch.value == 1 else (h.value, w.value, 4)
        return np.ctypeslib.as_array(px, shape=shape).copy()
    finally:
        lib.isti_image_free(px)


def decode_exr(data: bytes) -> np.ndarray:
    lib = _lib()
    w, h, ch, px = C.c_int32(), C.c_int32(), C.c_int32(), C.POINTER(C.c_float)()
    buf = (C.c_uint8 * len(data)).from_buffer_copy(data)
    native.check(lib.isti_exr_decode_memory(buf, len(data), C.byref(w), C.byref(h), C.byref(ch), C.byref(px)))
    try:
        shape = (h.value, w.value) if ch.value == 1 else (h.value, w.value, 4)
        return np.ctypeslib.as_array(px, shape=shape).copy()
    finally:
        lib.isti_image_free(px)


def write_png(path: str, image: np.ndarray) -> None:
    """RGB8 / RGBA8 image (H, W, 3|4) to a PNG file."""
    img = np.ascontiguousarray(image, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] not in (3, 4):
        raise ValueError("write_png expects an (H, W, 3|4) uint8 image")
    native.check(_lib().isti_png_encode_file(os.fsencode(path), img.shape[1], img.shape[0], img.shape[2],
                                             img.ctypes.data))


def write_exr(path: str, image: np.ndarray, zip_compression: bool = True) -> None:
    """float32 (H, W) or (H, W, 4) image to a scan-line EXR file (FLOAT samples)."""
    img = np.ascontiguousarray(image, dtype=np.float32)
    if img.ndim == 2:
        ch = 1
    elif img.ndim == 3 and img.shape[2] == 4:
        ch = 4
    else:
        raise ValueError("write_exr expects (H, W) or (H, W, 4) float32")
    native.check(_lib().isti_exr_encode_file(os.fsencode(path), img.shape[1], img.shape[0], ch, img.ctypes.data,
                                             3 if zip_compression else 0))


def encode_png(image: np.ndarray) -> bytes:
    img = np.ascontiguousarray(image, dtype=np.uint8)
    lib = _lib()
    out, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    native.check(lib.isti_png_encode_memory(img.shape[1], img.shape[0], img.shape[2], img.ctypes.data,
                                            C.byref(out), C.byref(n)))
    try:
        return C.string_at(out, n.value)
    finally:
        lib.isti_image_free(out)


def zlib_decompress(data: bytes) -> bytes:
    lib = _lib()
    out, n = C.POINTER(C.c_uint8)(), C.c_size_t()
    buf = (C.c_uint8 * max(1, len(data))).from_buffer_copy(data if data else b"\0")
    native.check(lib.isti_zlib_decompress(buf, len(data), C.byref(out), C.byref(n)))
    try:
        return C.string_at(out, n.value)
    finally:
        lib.isti_image_free(out)


def _mat(m16) -> np.ndarray:
    """column-major float[16] -> row-major (4, 4) float32"""
    return np.array(list(m16), dtype=np.float32).reshape(4, 4).T.copy()


def read_camera_path(directory: str) -> dict:
    """cam.json of a camera folder: resolution, fps values, priority and frames
    (idx, w2c, proj as row-major 4x4 float32)."""
    lib = _lib()
    h = C.c_void_p()
    native.check(lib.isti_camera_path_open(os.fsencode(directory), C.byref(h)))
    try:
        info = native.IstiCameraInfo()
        native.check(lib.isti_camera_path_info(h, C.byref(info)))
        frames = []
        for i in range(info.n_frames):
            f = native.IstiCameraFrame()
            native.check(lib.isti_camera_path_frame(h, i, C.byref(f)))
            frames.append({"idx": f.idx, "w2c": _mat(f.w2c), "proj": _mat(f.proj)})
        return {"width": info.width, "height": info.height, "client_fps": info.client_fps,
                "server_fps": info.server_fps, "shadow_fps": info.shadow_fps, "priority": info.priority,
                "frames": frames}
    finally:
        lib.isti_camera_path_close(h)


def normalize_proj(proj: np.ndarray) -> np.ndarray:
    out = native.Mat16()
    native.check(_lib().isti_normalize_proj(native.mat16(proj), out))
    return _mat(out)


def unity_depth(z: np.ndarray) -> np.ndarray:
    """NDC z -> the reversed [0, 1] depth the dataset stores (the inverse of
    convertDepthToZ, src/file_reader.cu:17-37), float32."""
    z = np.asarray(z, np.float32)
    return np.float32(1.0) - (z + np.float32(1.0)) * np.float32(0.5)


def z_from_unity_depth(d: np.ndarray) -> np.ndarray:
    """convertDepthToZ's arithmetic on the host (float32, each step rounded): 2 (1 - d) - 1."""
    d = np.asarray(d, np.float32)
    return np.float32(2.0) * (np.float32(1.0) - d) - np.float32(1.0)


# FrameFileReader::normalizeProjMat's factors (include/file_reader.h:64-67) as row-major matrices
_REVERSE_Z = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, -1, 1], [0, 0, 0, 1]], np.float64)
_DEPTH_01_TO_11 = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 2, -1], [0, 0, 0, 1]], np.float64)
_UNITY_2022_3 = np.diag([1.0, -1.0, 1.0, 1.0])


def raw_projection(gl_proj: np.ndarray) -> np.ndarray:
    """The projection a Unity capture stores for a given OpenGL-convention
    projection: normalizeProjMat(raw) == gl_proj up to float rounding."""
    m = _UNITY_2022_3 @ _DEPTH_01_TO_11 @ _REVERSE_Z
    return (np.linalg.inv(m) @ np.asarray(gl_proj, np.float64)).astype(np.float32)


def _cam_json(path: str, frames, width: int, height: int, client_fps: int, server_fps: int, shadow_fps: int,
              object_motion: bool, shadow_gradients: bool) -> None:
    import json

    def mat(m):
        m = np.asarray(m, np.float32)
        return {f"e{r}{c}": float(m[r, c]) for r in range(4) for c in range(4)}

    doc = {"resolution": {"x": int(width), "y": int(height)}, "clientFps": client_fps, "serverFps": server_fps,
           "shadowFps": shadow_fps, "objectMotion": object_motion, "shadowGradients": shadow_gradients,
           "frames": [{"idx": int(i), "w2c": mat(w2c), "proj": mat(proj)} for i, w2c, proj in frames]}
    with open(path, "w") as f:
        json.dump(doc, f)


def export_sequence(seq, out_dir: str, aux_names=None, client_dir: str | None = "client",
                    client_fps: int | None = None, zip_exr: bool = True) -> dict:
    """Writes a procedural Sequence (scene.Sequence) as a dataset folder in the
    reference's format (cam.json, colour PNG, depth EXR, flow-field EXR and
    shadow PNG folders per camera; src/file_reader.cu), readable by Dataset and
    the splinter tool.  Cameras: "main" plus one folder per aux camera; with
    ``client_dir`` also a client camera path (cam.json only) at ``client_fps``
    following the sequence's client poses.  Returns the folder names."""
    from . import scene as _scene
    server_fps = int(round(1.0 / seq.dt))
    shadow_fps = seq.sfpa * server_fps
    client_fps = client_fps or seq.fpa * server_fps
    n_aux = len(seq.aux_offsets)
    if aux_names is None:
        aux_names = ["left", "right"][:n_aux] if n_aux <= 2 and (n_aux < 2 or seq.aux_offsets[0] < seq.aux_offsets[1]) \
            else [f"aux{i}" for i in range(n_aux)]
    cams = ["main"] + list(aux_names)
    shadow_dirs = [("forwardShadowColorA", "forwardShadowColorB", "forwardShadowInfo"),
                   ("backwardShadowColorA", "backwardShadowColorB", "backwardShadowInfo")]
    n = seq.n_keyframes
    for c, name in enumerate(cams):
        root = os.path.join(out_dir, name)
        subdirs = ["color", "depth", "forwardFlowField", "backwardFlowField"]
        if seq.shadows:
            subdirs += list(shadow_dirs[0]) + list(shadow_dirs[1])
        for s in subdirs:
            os.makedirs(os.path.join(root, s), exist_ok=True)
        proj = raw_projection(seq.proj_main if c == 0 else seq.proj_aux)
        frames = []
        w, h = (seq.width, seq.height) if c == 0 else seq.aux_size
        for k in range(n):
            kf = seq.keyframe(k, c)
            pose = seq._cam_pose(seq.poses[k], c)
            frames.append((k, _scene.view_matrix(pose.eye, pose.yaw, pose.pitch), proj))
            nm = f"{k:04d}"
            write_png(os.path.join(root, "color", nm + ".png"), kf.color)
            write_exr(os.path.join(root, "depth", nm + ".exr"), unity_depth(kf.z), zip_exr)
            if k + 1 < n:
                nxt = seq.keyframe(k + 1, c)
                for folder, motion in (("forwardFlowField", kf.motion_fwd), ("backwardFlowField", nxt.motion_bwd)):
                    m4 = np.zeros(motion.shape[:2] + (4,), np.float32)
                    m4[..., :3] = motion.astype(np.float32)
                    write_exr(os.path.join(root, folder, nm + ".exr"), m4, zip_exr)
                if seq.shadows:
                    for dirs, sh in ((shadow_dirs[0], kf.shadow_fwd), (shadow_dirs[1], nxt.shadow_bwd)):
                        for d, img in zip(dirs, sh):
                            write_png(os.path.join(root, d, nm + ".png"), img)
        _cam_json(os.path.join(root, "cam.json"), frames, w, h, client_fps, server_fps, shadow_fps, True, seq.shadows)
    if client_dir:
        root = os.path.join(out_dir, client_dir)
        os.makedirs(root, exist_ok=True)
        proj = raw_projection(seq.proj_main)
        frames = []
        for k in range(n - 1):
            for b in range(seq.fpa):
                t = b / seq.fpa
                pose = seq.poses[k].lerp(seq.poses[k + 1], t)
                frames.append((k * seq.fpa + b, _scene.view_matrix(pose.eye, pose.yaw, pose.pitch), proj))
        _cam_json(os.path.join(root, "cam.json"), frames, seq.width, seq.height, client_fps, server_fps, shadow_fps,
                  True, seq.shadows)
    return {"cameras": cams, "client": client_dir}


class Dataset:
    """Keyframes of a dataset folder on the device (FrameFileReader + FrameData).

    ``frame()`` returns the isti_frame_data of the current pair, ready for
    Renderer.render_raw / isti_render."""

    def __init__(self, input_dir: str, aux_dirs=(), stream=None):
        lib = _lib()
        self._h = C.c_void_p()
        aux = [os.fsencode(a) for a in aux_dirs]
        arr = (C.c_char_p * max(1, len(aux)))(*aux) if aux else None
        native.check(lib.isti_dataset_open(os.fsencode(input_dir), len(aux), arr, stream, C.byref(self._h)))

    def read_next(self) -> bool:
        adv = C.c_int32()
        native.check(_lib().isti_dataset_read_next(self._h, C.byref(adv)))
        return bool(adv.value)

    def frame(self) -> native.IstiFrameData:
        fd = native.IstiFrameData()
        native.check(_lib().isti_dataset_frame(self._h, C.byref(fd)))
        return fd

    def camera(self, index: int = -1) -> dict:
        info = native.IstiCameraInfo()
        native.check(_lib().isti_dataset_camera(self._h, index, C.byref(info)))
        return {f: getattr(info, f) for f, _ in info._fields_}

    def matrices(self, slot: int):
        view, proj = native.Mat16(), native.Mat16()
        native.check(_lib().isti_dataset_matrices(self._h, slot, view, proj))
        return _mat(view), _mat(proj)

    @property
    def keyframe(self) -> int:
        return _lib().isti_dataset_keyframe(self._h)

    def close(self) -> None:
        if self._h:
            _lib().isti_dataset_close(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
