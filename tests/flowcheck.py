"""Comparison of the renderer's client-camera flow with a reference-layout one.

The reference keeps the client flow of each source pixel as f32x4 (x, y, dz, visible)
(src/renderer.cu:117) and derives the reprojection depth z_to_depth(z + dz) after the search
(src/renderer.cu:339).  The renderer stores (x, y), that depth and the visibility byte; these
helpers derive the same three from a reference-layout flow and the view's z.
"""
import numpy as np


def expected_client_flow(cam_ff, z):
    """The same parts from a reference-layout f32x4 flow (x, y, dz, visible) and the view's z:
    depth = z_to_depth(z + dz) = (f32(z + dz) + 1) * 0.5, each step rounded to f32."""
    s = (z.astype(np.float32) + cam_ff[..., 2]).astype(np.float32)
    depth = ((s + np.float32(1.0)).astype(np.float32) * np.float32(0.5)).astype(np.float32)
    return cam_ff[..., :2], depth, (cam_ff[..., 3] > 0).astype(np.uint8)


def assert_client_flow_equal(k, got, cam_ff, z):
    exp = expected_client_flow(cam_ff, z)
    for name, a, b in zip(("flow x, y", "flow depth", "visibility"), got, exp):
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), \
            f"view {k}: client {name} differs"
