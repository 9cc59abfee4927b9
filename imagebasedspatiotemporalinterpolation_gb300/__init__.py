"""GB300-native per-frame image-based spatio-temporal interpolation.

Drop-in for the interpolation path of the reference renderer
(DerThomy/ImageBasedSpatioTemporalInterpolation, src/renderer.cu): depth-keyed
64-bit atomic splatting, bidirectional reprojection with the iterative
flow-field search, hole filling and soft-shadow blending, as hand-written
sm_103a CUDA kernels behind the C ABI in include/isti.h (libisti.so).
"""
from .native import (MODE_BACKWARD_BIDIRECTIONAL, MODE_BACKWARD_UNIDIRECTIONAL, MODE_OURS, MODE_SPLATTING,
                     MODE_TIMEWARP, IstiError)

__all__ = ["MODE_OURS", "MODE_BACKWARD_BIDIRECTIONAL", "MODE_BACKWARD_UNIDIRECTIONAL", "MODE_SPLATTING",
           "MODE_TIMEWARP", "IstiError", "Renderer", "DeviceFrame", "DeviceView"]


def __getattr__(name):
    if name in ("Renderer", "DeviceFrame", "DeviceView"):
        from . import renderer
        return getattr(renderer, name)
    raise AttributeError(name)
