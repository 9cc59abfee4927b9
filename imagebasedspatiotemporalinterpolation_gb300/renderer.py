"""Python mirror of the reference's renderer interface over the C ABI.

  DeviceView   <- MotionZBufferImage (include/data.h:12-62), device-resident
  DeviceFrame  <- FrameData (include/data.h:79-116), incl. swap()
  Renderer     <- Renderer::render(ImageBuffer<uchar4,4>&, RenderInfo, FrameData&)
                  (include/renderer.h:52-56)

Device memory and streams come from PyTorch (plumbing only); every pixel is
computed by libisti.so.  There is no CPU fallback: a missing library or a
non-CUDA tensor raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native
from .native import IstiFrameData, IstiRenderInfo, IstiView, check, mat16


def _torch():
    import torch
    return torch


def _dptr(t) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("isti buffers must be CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("isti buffers must be contiguous")
    return t.data_ptr()


@dataclass
class DeviceView:
    """One camera at one keyframe in device memory."""
    color: object                     # (H, W, 4) uint8
    z: object                         # (H, W) float32
    motion: object | None             # (H, W, 3) float16 or (H, W, 4) float32
    shadow_a: object | None = None
    shadow_b: object | None = None
    shadow_info: object | None = None
    viewproj: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    inv_viewproj: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))

    @property
    def width(self) -> int:
        return int(self.z.shape[1])

    @property
    def height(self) -> int:
        return int(self.z.shape[0])

    @staticmethod
    def from_host(v, device="cuda", motion_format: str = "f16x3", non_blocking: bool = False) -> "DeviceView":
        torch = _torch()

        def up(a, dtype=None):
            if a is None:
                return None
            t = torch.from_numpy(np.ascontiguousarray(a if dtype is None else a.astype(dtype)))
            return t.to(device, non_blocking=non_blocking)

        if v.motion is None:
            mot = None
        elif motion_format == "f16x3":
            mot = up(v.motion, np.float16)
        elif motion_format == "f32x4":
            mot = up(v.motion_f32x4())
        else:
            raise ValueError(f"unknown motion format {motion_format}")
        return DeviceView(up(v.color), up(v.z, np.float32), mot, up(v.shadow_a), up(v.shadow_b), up(v.shadow_info),
                          np.asarray(v.viewproj, np.float32), np.asarray(v.inv_viewproj, np.float32))

    def to_c(self) -> IstiView:
        if self.motion is None:
            fmt = native.MOTION_NONE
        elif self.motion.shape[-1] == 3:
            fmt = native.MOTION_F16X3
        else:
            fmt = native.MOTION_F32X4
        return IstiView(self.width, self.height, _dptr(self.color), _dptr(self.z), _dptr(self.motion), fmt,
                        _dptr(self.shadow_a), _dptr(self.shadow_b), _dptr(self.shadow_info),
                        mat16(self.viewproj), mat16(self.inv_viewproj))


@dataclass
class DeviceFrame:
    """FrameData in device memory: fwd/bwd main keyframes plus aux cameras."""
    fwd: DeviceView
    bwd: DeviceView
    aux_curr: list = field(default_factory=list)
    aux_next: list = field(default_factory=list)
    aux_priority: list = field(default_factory=list)
    _c: object = None

    @staticmethod
    def from_host(frame, device="cuda", motion_format: str = "f16x3", non_blocking: bool = False) -> "DeviceFrame":
        up = lambda v: DeviceView.from_host(v, device, motion_format, non_blocking)
        return DeviceFrame(up(frame.fwd), up(frame.bwd), [up(v) for v in frame.aux_curr], [up(v) for v in frame.aux_next],
                           list(frame.aux_priority))

    def swap(self) -> None:
        """FrameData::swap (include/data.h:110-115): the later keyframe becomes the earlier one."""
        self.fwd, self.bwd = self.bwd, self.fwd
        self.aux_curr, self.aux_next = self.aux_next, self.aux_curr
        self._c = None

    def views(self) -> list:
        out = [self.fwd, self.bwd]
        for a, b in zip(self.aux_curr, self.aux_next):
            out += [a, b]
        return out

    def to_c(self):
        """Marshalled isti_frame_data (cached until swap())."""
        if self._c is None:
            n = len(self.aux_curr)
            curr = (IstiView * max(1, n))(*[v.to_c() for v in self.aux_curr])
            nxt = (IstiView * max(1, n))(*[v.to_c() for v in self.aux_next])
            prio = (C.c_int32 * max(1, n))(*(self.aux_priority or [0] * n))
            fd = IstiFrameData(self.fwd.to_c(), self.bwd.to_c(), n, C.cast(curr, C.POINTER(IstiView)),
                               C.cast(nxt, C.POINTER(IstiView)), C.cast(prio, C.POINTER(C.c_int32)))
            self._c = (fd, curr, nxt, prio)
        return self._c[0]


def render_info(client) -> IstiRenderInfo:
    """RenderInfo from a scene.Client-like object."""
    return IstiRenderInfo(int(client.width), int(client.height), float(client.alpha), mat16(client.viewproj),
                          mat16(client.inv_viewproj), int(client.frames_per_anchor),
                          int(client.shadow_frames_per_anchor), int(bool(client.no_shadows)), int(client.mode))


class _CudaArray:
    """__cuda_array_interface__ view of a raw device pointer (read back only)."""

    def __init__(self, ptr: int, shape: tuple, typestr: str):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


class Renderer:
    """Reference Renderer (include/renderer.h:52-93) on libisti.so."""

    def __init__(self):
        self._lib = native.load()
        h = C.c_void_p()
        check(self._lib.isti_renderer_create(C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            check(self._lib.isti_renderer_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, render_buffer, info, frame_data: DeviceFrame, stream=None) -> None:
        """Render one interpolated client frame into render_buffer ((H, W, 4)
        uint8 CUDA tensor).  Pixels without a valid result keep their content."""
        torch = _torch()
        ri = info if isinstance(info, IstiRenderInfo) else render_info(info)
        if tuple(render_buffer.shape) != (ri.height, ri.width, 4) or render_buffer.dtype != torch.uint8:
            raise ValueError("render_buffer must be a (H, W, 4) uint8 tensor of the render resolution")
        s = (stream or torch.cuda.current_stream()).cuda_stream
        check(self._lib.isti_render(self._h, _dptr(render_buffer), C.byref(ri), C.byref(frame_data.to_c()), C.c_void_p(s)))

    def render_batch(self, render_buffers, infos, frame_data: DeviceFrame, chain: bool = True, stream=None) -> None:
        """Render len(infos) client frames of one keyframe pair in one launch pair
        (isti_render_batch).  With chain=True the result equals rendering the
        frames in order into one persistent buffer that starts as
        render_buffers[0] and is copied to render_buffers[k] after frame k."""
        torch = _torch()
        n = len(infos)
        if n != len(render_buffers) or not 1 <= n <= native.MAX_BATCH_FRAMES:
            raise ValueError(f"need 1..{native.MAX_BATCH_FRAMES} frames and one buffer per frame")
        ris = (IstiRenderInfo * n)(*[i if isinstance(i, IstiRenderInfo) else render_info(i) for i in infos])
        for b in render_buffers:
            if tuple(b.shape) != (ris[0].height, ris[0].width, 4) or b.dtype != torch.uint8:
                raise ValueError("render buffers must be (H, W, 4) uint8 tensors of the render resolution")
        outs = (C.c_void_p * n)(*[_dptr(b) for b in render_buffers])
        s = (stream or torch.cuda.current_stream()).cuda_stream
        check(self._lib.isti_render_batch(self._h, n, outs, ris, C.byref(frame_data.to_c()), int(chain), C.c_void_p(s)))

    def render_pairs(self, jobs, chain: bool = False, stream=None) -> None:
        """isti_render_pairs: jobs = [(render_buffers, infos, frame_data), ...], the frames of
        several keyframe pairs in one persistent launch; each job's result equals
        render_batch(render_buffers, infos, frame_data, chain)."""
        torch = _torch()
        if not 1 <= len(jobs) <= native.MAX_PAIRS:
            raise ValueError(f"need 1..{native.MAX_PAIRS} keyframe pairs")
        keep = []
        arr = (native.IstiPairFrames * len(jobs))()
        for i, (bufs, infos, fd) in enumerate(jobs):
            n = len(infos)
            if n != len(bufs) or not 1 <= n <= native.MAX_BATCH_FRAMES:
                raise ValueError(f"need 1..{native.MAX_BATCH_FRAMES} frames and one buffer per frame")
            ris = (IstiRenderInfo * n)(*[x if isinstance(x, IstiRenderInfo) else render_info(x) for x in infos])
            outs = (C.c_void_p * n)(*[_dptr(b) for b in bufs])
            fdc = fd.to_c()
            keep += [ris, outs, fdc]
            arr[i] = native.IstiPairFrames(C.pointer(fdc), n, C.cast(outs, C.POINTER(C.c_void_p)), C.cast(ris, C.POINTER(IstiRenderInfo)),
                                           int(chain))
        s = (stream or torch.cuda.current_stream()).cuda_stream
        self._keep_pairs = (arr, keep)  # the structs must outlive the call
        check(self._lib.isti_render_pairs(self._h, len(jobs), arr, C.c_void_p(s)))

    def test_stall_pair(self, pair: int, spin_limit: int = 0) -> None:
        """isti_renderer_test_stall_pair: the failure-detection test hook of render_pairs
        (pair < 0: off)."""
        check(self._lib.isti_renderer_test_stall_pair(self._h, int(pair), int(spin_limit)))

    def set_pair_units(self, splat_rows: int = 0, init_unit_kib: int = 0) -> None:
        """isti_renderer_set_pair_units: render_pairs' splat-unit rows and init-unit KiB (0: default)."""
        check(self._lib.isti_renderer_set_pair_units(self._h, int(splat_rows), int(init_unit_kib)))

    def render_learned(self, render_buffers, infos, frame_data: DeviceFrame, net=None, iterations: int = 1, chain: bool = False,
                       stream=None) -> None:
        """isti_render_learned: the frames of one keyframe pair (main camera only) with the
        search started from the learned initialiser `net` (a flownet.FlowNet; None = at the
        output pixel) and `iterations` search steps; tiles left unresolved are rendered by
        the plain method.  chain: as render_batch's (one persistent buffer across the frames);
        otherwise each buffer is updated in place like isti_render."""
        torch = _torch()
        n = len(infos)
        if n != len(render_buffers) or not 1 <= n <= native.MAX_BATCH_FRAMES:
            raise ValueError(f"need 1..{native.MAX_BATCH_FRAMES} frames and one buffer per frame")
        ris = (IstiRenderInfo * n)(*[i if isinstance(i, IstiRenderInfo) else render_info(i) for i in infos])
        outs = (C.c_void_p * n)(*[_dptr(b) for b in render_buffers])
        s = (stream or torch.cuda.current_stream()).cuda_stream
        check(self._lib.isti_render_learned(self._h, net.handle if net is not None else None, n, outs, ris,
                                            C.byref(frame_data.to_c()), int(iterations), int(chain), C.c_void_p(s)))

    def learned_stats(self) -> tuple[int, int]:
        """(tiles rendered by the plain method, all tiles) of the last learned call (waits)."""
        a, b = C.c_int32(), C.c_int32()
        check(self._lib.isti_renderer_learned_stats(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def device_status(self) -> int:
        """Waits for the device; 0, or ISTI_ERR_TIMEOUT when a kernel's bounded wait gave up."""
        s = C.c_int32()
        check(self._lib.isti_renderer_device_status(self._h, C.byref(s)))
        return s.value

    def set_arithmetic(self, arith: int) -> None:
        """isti_renderer_set_arithmetic: native.ARITH_IEEE (default, bit-exact against the
        oracle) or native.ARITH_REFERENCE_GPU (the reference GPU build's -use_fast_math)."""
        check(self._lib.isti_renderer_set_arithmetic(self._h, int(arith)))

    def test_withhold_tile(self, x: int, y: int, wait_limit: int = 0) -> None:
        """Failure-detection hook (isti_renderer_test_withhold_tile): the reprojection block
        covering output pixel (x, y) issues no tile copy, so its bounded wait runs out and
        the device status turns ISTI_ERR_TIMEOUT.  x < 0 switches it off."""
        check(self._lib.isti_renderer_test_withhold_tile(self._h, int(x), int(y), int(wait_limit)))

    def enable_timing(self, on: bool = True) -> None:
        check(self._lib.isti_renderer_enable_timing(self._h, int(on)))

    def timing(self) -> dict:
        """Summed per-stage device time of the renders since the last call (waits for them)."""
        t = native.IstiTiming()
        check(self._lib.isti_renderer_timing(self._h, C.byref(t)))
        return {"frames": t.frames, "kernel_launches": t.kernel_launches, "init_ms": t.init_ms,
                "splat_ms": t.splat_ms, "reproj_ms": t.reproj_ms}

    def set_autotune(self, on: bool = True) -> None:
        """isti_renderer_set_autotune: the first uncaptured render of each shape class times
        the reprojection's candidate launches and later renders use the fastest."""
        check(self._lib.isti_renderer_set_autotune(self._h, int(on)))

    def set_reproj_launch(self, regs: int = 0, row_pairs: int = 0, plain_tiles: int = 0) -> None:
        """isti_renderer_set_reproj_launch: pin the reprojection launch of later renders
        (register cap, output row pairs per block, key tiles by plain loads); 0: the rule's."""
        check(self._lib.isti_renderer_set_reproj_launch(self._h, int(regs), int(row_pairs), int(plain_tiles)))

    def tuning(self) -> list:
        """The tuned shape classes and their chosen launches (isti_renderer_tuning)."""
        n = C.c_int32()
        check(self._lib.isti_renderer_tuning_count(self._h, C.byref(n)))
        out = []
        for i in range(n.value):
            t = native.IstiTuning()
            check(self._lib.isti_renderer_tuning(self._h, i, C.byref(t)))
            out.append({k: getattr(t, k) for k, _ in native.IstiTuning._fields_})
        return out

    def view_buffers(self, view: int):
        """(splat keys as int64 bit patterns (H, W), client flow (x, y) f32 (H, W, 2), full_ff f32
        (H, W, 4)) of the last render, as copies."""
        torch = _torch()
        sp, cf, ff = C.c_void_p(), C.c_void_p(), C.c_void_p()
        w, h = C.c_uint32(), C.c_uint32()
        check(self._lib.isti_renderer_view_buffers(self._h, view, C.byref(sp), C.byref(cf), C.byref(ff), C.byref(w), C.byref(h)))
        H, W = h.value, w.value
        out = []
        for ptr, shape, ts in ((sp, (H, W), "<i8"), (cf, (H, W, 2), "<f4"), (ff, (H, W, 4), "<f4")):
            out.append(None if not ptr.value else torch.as_tensor(_CudaArray(ptr.value, shape, ts), device="cuda").clone())
        return tuple(out)

    def view_depth(self, view: int):
        """(client-flow depth z_to_depth(z + dz) f32 (H, W), visible_in_main uint8 (H, W)) of the
        last render, as copies (isti_renderer_view_depth)."""
        torch = _torch()
        dp, vs = C.c_void_p(), C.c_void_p()
        w, h = C.c_uint32(), C.c_uint32()
        check(self._lib.isti_renderer_view_buffers(self._h, view, None, None, None, C.byref(w), C.byref(h)))
        check(self._lib.isti_renderer_view_depth(self._h, view, C.byref(dp), C.byref(vs)))
        H, W = h.value, w.value
        return tuple(None if not ptr.value else torch.as_tensor(_CudaArray(ptr.value, (H, W), ts), device="cuda").clone()
                     for ptr, ts in ((dp, "<f4"), (vs, "|u1")))


def render_noalloc(render_buffer, info, frame_data: DeviceFrame, stream=None) -> None:
    """isti_render_noalloc: render one frame without any device allocation.

    For callers that cannot allocate device memory while they run (their
    device budget is reserved up front by their own pool, or cudaMalloc's
    possible device synchronisation would break a per-frame deadline).  The
    scratch is a fixed 64 MiB array inside libisti.so, so frames are limited to
    sum(width * height * 40 bytes) over the source views (640x360 with two aux
    cameras fits).  The first call on a device looks up that array's address:
    make it before any stream capture.  All calls share the array; do not let
    calls overlap on the GPU."""
    torch = _torch()
    lib = native.load()
    ri = info if isinstance(info, IstiRenderInfo) else render_info(info)
    if tuple(render_buffer.shape) != (ri.height, ri.width, 4) or render_buffer.dtype != torch.uint8:
        raise ValueError("render_buffer must be a (H, W, 4) uint8 tensor of the render resolution")
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(lib.isti_render_noalloc(_dptr(render_buffer), C.byref(ri), C.byref(frame_data.to_c()), C.c_void_p(s)))


def rgb8_to_rgba8(dst, src, stream=None) -> None:
    """isti_rgb8_to_rgba8: a packed RGB8 device tensor (..., 3) uint8 -> the RGBA8 tensor
    (..., 4) uint8 the renderer reads, alpha 255.  For images whose alpha the renderer
    never reads (shadow colour A/B, shadow info): uploading them as RGB moves 3/4 of the
    bytes over the host link."""
    torch = _torch()
    if src.dtype != torch.uint8 or dst.dtype != torch.uint8 or src.shape[-1] != 3 or dst.shape[-1] != 4 \
            or src.shape[:-1] != dst.shape[:-1] or not src.is_contiguous() or not dst.is_contiguous():
        raise ValueError("rgb8_to_rgba8 expects contiguous uint8 (..., 3) -> (..., 4) tensors of the same pixel count")
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(native.load().isti_rgb8_to_rgba8(_dptr(dst), _dptr(src), C.c_size_t(src.numel() // 3), C.c_void_p(s)))


SHADOW_ENTRY_BYTES = 16  # ISTI_SHADOW_ENTRY_BYTES


def pack_shadow_entries(info, a, b):
    """Host side of isti_unpack_shadows: the sparse form of one view's shadow info, colour A
    and colour B images ((H, W, 3 or 4) uint8 numpy arrays).  One 16-byte entry per pixel
    whose info field (R, G, B) is non-zero -- the only pixels where the renderer reads any of
    the three images: pixel index (uint32 little-endian), info RGB, A RGB, B RGB, 3 zero
    bytes.  Returns an (n, 16) uint8 array."""
    import numpy as np
    info, a, b = (np.asarray(x) for x in (info, a, b))
    if not (info.shape[:2] == a.shape[:2] == b.shape[:2]) or info.dtype != np.uint8 or a.dtype != np.uint8 or b.dtype != np.uint8:
        raise ValueError("shadow images must be uint8 arrays of one size")
    n_px = info.shape[0] * info.shape[1]
    if n_px >= 1 << 32:
        raise ValueError("too many pixels for 32-bit indices")
    rgb = lambda x: x.reshape(n_px, x.shape[-1])[:, :3]
    idx = np.flatnonzero(rgb(info).any(axis=1))
    out = np.zeros((len(idx), SHADOW_ENTRY_BYTES), np.uint8)
    out[:, 0:4] = idx.astype("<u4").view(np.uint8).reshape(-1, 4)
    out[:, 4:7] = rgb(info)[idx]
    out[:, 7:10] = rgb(a)[idx]
    out[:, 10:13] = rgb(b)[idx]
    return out


def unpack_shadows(info, a, b, entries, n_entries=None, clear_entries=None, n_clear=None, stream=None) -> None:
    """isti_unpack_shadows: device RGBA8 tensors info, a, b ((H, W, 4) uint8, 16-byte aligned)
    <- zero, then the listed pixels of `entries` (a device uint8 tensor of n x 16 bytes, as
    pack_shadow_entries makes them).  clear_entries: the entries of the previous unpack into
    the same images, whose pixels alone are then cleared."""
    torch = _torch()
    for t in (info, a, b):
        if t.dtype != torch.uint8 or t.shape[-1] != 4 or not t.is_contiguous() or t.shape != info.shape:
            raise ValueError("unpack_shadows expects three contiguous uint8 (..., 4) tensors of one shape")
    n = entries.numel() // SHADOW_ENTRY_BYTES if n_entries is None else int(n_entries)
    nc = 0 if clear_entries is None else (clear_entries.numel() // SHADOW_ENTRY_BYTES if n_clear is None else int(n_clear))
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(native.load().isti_unpack_shadows(_dptr(info), _dptr(a), _dptr(b), C.c_size_t(info.numel() // 4),
                                            C.c_void_p(_dptr(entries) if n else None), C.c_size_t(n),
                                            C.c_void_p(_dptr(clear_entries) if clear_entries is not None else None), C.c_size_t(nc),
                                            C.c_void_p(s)))
