"""GPU image quality (include/isti_metrics.h): the PSNR / SSIM of the
reference's evaluation script (scripts/eval.py:66-132, scripts/loss_utils.py)
for RGBA8 frames resident on the device."""
from __future__ import annotations

import ctypes as C

from . import native


class Quality:
    """Reusable scratch + result buffers for one image size."""

    def __init__(self, width: int, height: int, device=None):
        import torch

        self.width, self.height = int(width), int(height)
        self._lib = native.load()
        n = self._lib.isti_quality_scratch_bytes(self.width, self.height)
        dev = device or torch.device("cuda", torch.cuda.current_device())
        self._scratch = torch.empty(max(8, n), dtype=torch.uint8, device=dev)
        self._out = torch.zeros(3, dtype=torch.float64, device=dev)

    def launch(self, a, b, stream=None):
        """Enqueue the metric kernels for two (H, W, 4) uint8 CUDA tensors; returns
        the device tensor [mse, psnr, ssim] (valid once the stream reaches it)."""
        import torch

        for t in (a, b):
            if t.device.type != "cuda" or t.dtype != torch.uint8 or tuple(t.shape) != (self.height, self.width, 4) \
                    or not t.is_contiguous():
                raise ValueError("expected contiguous (H, W, 4) uint8 CUDA tensors of the configured size")
        s = stream if stream is not None else torch.cuda.current_stream()
        native.check(self._lib.isti_quality_rgba8(a.data_ptr(), b.data_ptr(), self.width, self.height,
                                                  self._scratch.data_ptr(), self._out.data_ptr(), s.cuda_stream))
        return self._out

    def __call__(self, a, b, stream=None) -> dict:
        out = self.launch(a, b, stream).cpu().tolist()
        return {"mse": out[0], "psnr": out[1], "ssim": out[2]}

    def flip(self, test, reference, pixels_per_degree: float = native.FLIP_DEFAULT_PPD, stream=None, with_map: bool = False):
        """LDR-FLIP of a rendered frame against its reference (scripts/flip_loss.py; eval.py's
        flip_fn(render, ground_truth)).  Returns the mean, or (mean, per-pixel map tensor)."""
        import torch

        for t in (test, reference):
            if t.device.type != "cuda" or t.dtype != torch.uint8 or tuple(t.shape) != (self.height, self.width, 4) \
                    or not t.is_contiguous():
                raise ValueError("expected contiguous (H, W, 4) uint8 CUDA tensors of the configured size")
        if not hasattr(self, "_flip_scratch"):
            n = self._lib.isti_flip_scratch_bytes(self.width, self.height)
            self._flip_scratch = torch.empty(max(8, n), dtype=torch.uint8, device=test.device)
            self._flip_out = torch.zeros(1, dtype=torch.float64, device=test.device)
        fmap = torch.empty((self.height, self.width), dtype=torch.float32, device=test.device) if with_map else None
        s = stream if stream is not None else torch.cuda.current_stream()
        native.check(self._lib.isti_flip_rgba8(test.data_ptr(), reference.data_ptr(), self.width, self.height,
                                               float(pixels_per_degree), self._flip_scratch.data_ptr(),
                                               self._flip_out.data_ptr(), None if fmap is None else fmap.data_ptr(),
                                               s.cuda_stream))
        mean = float(self._flip_out.item())
        return (mean, fmap) if with_map else mean


def quality(a, b) -> dict:
    """PSNR / SSIM of two (H, W, 4) uint8 CUDA tensors (waits for the result)."""
    return Quality(a.shape[1], a.shape[0], a.device)(a, b)
