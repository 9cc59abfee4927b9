"""ORACLE (test infrastructure only): the reference's vendored image libraries.

oracle/_ref/libref_io.so (built by build_ref.py where the reference tree
exists) wraps stb_image / stb_image_write / tinyexr with the configuration of
src/util/image_buffer.cu:8-17; ImageBuffer::readFromFile calls exactly
stbi_load(..., 4) and LoadEXR (:112-165).  Used to pin libisti's decoders and
to write the codec fixtures in tests/golden/io.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import REF_DIR

LIB = os.path.join(REF_DIR, "libref_io.so")
_lib = None


def available() -> bool:
    return os.path.exists(LIB)


def _l():
    global _lib
    if _lib is None:
        lib = C.CDLL(LIB)
        lib.ref_png_load.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.POINTER(C.c_uint8))]
        lib.ref_exr_load.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.POINTER(C.c_float)), C.c_char_p, C.c_int]
        lib.ref_exr_save.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_void_p]
        lib.ref_png_save.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.ref_png_failure.restype = C.c_char_p
        lib.ref_free.argtypes = [C.c_void_p]
        _lib = lib
    return _lib


def png_load(path: str):
    """stbi_load(path, 4): (H, W, 4) uint8, or the failure reason (str)."""
    lib = _l()
    w, h, px = C.c_int(), C.c_int(), C.POINTER(C.c_uint8)()
    if lib.ref_png_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(px)) != 0:
        return (lib.ref_png_failure() or b"").decode()
    a = np.ctypeslib.as_array(px, shape=(h.value, w.value, 4)).copy()
    lib.ref_free(px)
    return a


def exr_load(path: str):
    """LoadEXR(path): (H, W) or (H, W, 4) float32, or the error message (str)."""
    lib = _l()
    w, h, ch, px = C.c_int(), C.c_int(), C.c_int(), C.POINTER(C.c_float)()
    err = C.create_string_buffer(512)
    if lib.ref_exr_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(ch), C.byref(px), err, 512) != 0:
        return err.value.decode()
    shape = (h.value, w.value) if ch.value == 1 else (h.value, w.value, 4)
    a = np.ctypeslib.as_array(px, shape=shape).copy()
    lib.ref_free(px)
    return a


def exr_save(path: str, planes: np.ndarray, names: list[str], pixel_type: int, compression: int) -> None:
    """tinyexr SaveEXRImageToFile: planes (C, H, W) float32, pixel_type 1 HALF / 2 FLOAT,
    compression 0 NONE, 1 RLE, 2 ZIPS, 3 ZIP, 4 PIZ."""
    p = np.ascontiguousarray(planes, np.float32)
    rc = _l().ref_exr_save(os.fsencode(path), p.shape[2], p.shape[1], p.shape[0], ",".join(names).encode(),
                           pixel_type, compression, p.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"SaveEXRImageToFile failed ({rc})")


def png_save(path: str, img: np.ndarray) -> None:
    a = np.ascontiguousarray(img, np.uint8)
    comp = 1 if a.ndim == 2 else a.shape[2]
    if _l().ref_png_save(os.fsencode(path), a.shape[1], a.shape[0], comp, a.ctypes.data) != 0:
        raise RuntimeError("stbi_write_png failed")
