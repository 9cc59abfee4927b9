"""Python side of the learned flow initialiser (include/isti_unet.h).

``FlowNet`` owns a network in libisti.so: parameters, gradients and Adam state in
device memory, forward pass and training step on the tcgen05 kernels.  Tensors are
torch CUDA tensors (plumbing only: every operation runs in libisti.so; a CPU tensor
or a missing library raises).
"""
from __future__ import annotations

import ctypes as C

from . import native
from .native import check


def _torch():
    import torch
    return torch


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("flownet buffers must be contiguous CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _stream(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def layers() -> list[tuple[int, int, int, int]]:
    """(taps, cin, cout, relu) of the 11 layers (10 tensor-core convolutions + head)."""
    lib = native.load()
    out = []
    for i in range(lib.isti_flownet_num_layers()):
        v = [C.c_int32() for _ in range(4)]
        check(lib.isti_flownet_layer(i, *[C.byref(x) for x in v]))
        out.append(tuple(x.value for x in v))
    return out


class FlowNet:
    """isti_flownet: the quarter-resolution U-Net (16 input channels, 4 output channels)."""

    IN_CH = 16
    OUT_CH = 4

    def __init__(self, seed: int = 0):
        self._lib = native.load()
        self._h = C.c_void_p()
        check(self._lib.isti_flownet_create(C.byref(self._h), C.c_uint64(seed)))
        p, g, n = C.c_void_p(), C.c_void_p(), C.c_size_t()
        check(self._lib.isti_flownet_tensors(self._h, C.byref(p), C.byref(g), C.byref(n)))
        self._params, self._grads, self.n_params = p.value, g.value, n.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            check(self._lib.isti_flownet_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def params(self):
        """Copy of the f32 parameter array (torch CUDA tensor)."""
        return self._read(self._params)

    def grads(self):
        return self._read(self._grads)

    def _read(self, addr: int):
        torch = _torch()
        out = torch.empty(self.n_params, dtype=torch.float32, device="cuda")
        _memcpy_d2d(out.data_ptr(), addr, self.n_params * 4)
        return out

    def set_params(self, values) -> None:
        """Overwrite the f32 parameters (and repack the bf16 operand images)."""
        torch = _torch()
        v = values.to(device="cuda", dtype=torch.float32).contiguous()
        if v.numel() != self.n_params:
            raise ValueError("wrong parameter count")
        _memcpy_d2d(self._params, v.data_ptr(), self.n_params * 4)
        check(self._lib.isti_flownet_sync_params(self._h, _stream()))

    def offsets(self, layer: int) -> tuple[int, int]:
        w, b = C.c_size_t(), C.c_size_t()
        check(self._lib.isti_flownet_param_offsets(self._h, layer, C.byref(w), C.byref(b)))
        return w.value, b.value

    def forward(self, x, flow=None, flow16=None, stream=None):
        """x: (n, h, w, 16) bf16 -> writes flow (n, h, w, 4) f32 and/or flow16 (f16)."""
        n, h, w, c = x.shape
        if c != self.IN_CH:
            raise ValueError("flownet input needs 16 channels")
        torch = _torch()
        if flow is None and flow16 is None:
            flow = torch.empty((n, h, w, self.OUT_CH), dtype=torch.float32, device=x.device)
        check(self._lib.isti_flownet_forward(self._h, _ptr(x), n, h, w, _ptr(flow), _ptr(flow16), _stream(stream)))
        return flow if flow is not None else flow16

    def backward(self, x, label, stream=None) -> None:
        n, h, w, _ = x.shape
        check(self._lib.isti_flownet_backward(self._h, _ptr(x), _ptr(label), n, h, w, _stream(stream)))

    def adam(self, lr: float, stream=None) -> None:
        check(self._lib.isti_flownet_adam(self._h, C.c_float(lr), _stream(stream)))

    def loss(self) -> float:
        torch = _torch()
        p = C.c_void_p()
        check(self._lib.isti_flownet_loss(self._h, C.byref(p)))
        out = torch.empty(1, dtype=torch.float32, device="cuda")
        _memcpy_d2d(out.data_ptr(), p.value, 4)
        return float(out.item())

    def device_status(self) -> int:
        s = C.c_int32()
        check(self._lib.isti_flownet_device_status(self._h, C.byref(s)))
        return s.value


def _memcpy_d2d(dst: int, src: int, nbytes: int) -> None:
    """Device-to-device copy of raw device memory on the current torch stream."""
    _wrap(dst, nbytes).copy_(_wrap(src, nbytes))


class _CudaArray:
    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (ptr, False), "version": 3}


def _wrap(addr: int, nbytes: int):
    """A uint8 CUDA tensor viewing raw device memory (no ownership)."""
    return _torch().as_tensor(_CudaArray(addr, nbytes), device="cuda")
