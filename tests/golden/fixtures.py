"""Golden fixture format: one compressed .npz per case, holding the inputs
(views, client camera, previous output image) and the reference renderer's
outputs (output image, per-view 64-bit splat keys and f32x4 flow fields).

Written by make_golden.py from the reference's own src/renderer.cu (compiled
for the CPU by oracle/build_ref.py); read by the tests.
"""
from __future__ import annotations

import glob
import os

import numpy as np

from imagebasedspatiotemporalinterpolation_gb300.scene import Client, Frame, View

GOLDEN_DIR = os.path.dirname(os.path.abspath(__file__))
VIEW_KEYS = ("color", "z", "motion", "shadow_a", "shadow_b", "shadow_info", "viewproj", "inv_viewproj")


def save(path, frame: Frame, client: Client, prev, out, splats, cams=None, fulls=None, meta: str = "") -> None:
    """cams / fulls (per-view flow fields) may be None to keep a fixture small."""
    d = {}
    for k, v in enumerate(frame.views()):
        for key in VIEW_KEYS:
            a = getattr(v, key)
            if a is not None:
                d[f"v{k}_{key}"] = np.asarray(a)
        d[f"v{k}_splat"] = splats[k]
        if cams is not None:
            d[f"v{k}_cam_ff"] = cams[k]
        if fulls is not None:
            d[f"v{k}_full_ff"] = fulls[k]
    d["n_aux"] = np.int32(len(frame.aux_curr))
    d["aux_priority"] = np.asarray(frame.aux_priority, np.int32)
    d["client_ints"] = np.asarray([client.width, client.height, client.frames_per_anchor,
                                   client.shadow_frames_per_anchor, int(client.no_shadows), client.mode], np.int32)
    d["client_alpha"] = np.float32(client.alpha)
    d["client_vp"] = np.asarray(client.viewproj, np.float32)
    d["client_ivp"] = np.asarray(client.inv_viewproj, np.float32)
    d["prev"] = prev
    d["out"] = out
    d["meta"] = np.asarray(meta)
    np.savez_compressed(path, **d)


def load(path):
    z = np.load(path)
    n_aux = int(z["n_aux"])

    def view(k):
        kw = {key: (z[f"v{k}_{key}"] if f"v{k}_{key}" in z else None) for key in VIEW_KEYS}
        return View(**kw)

    views = [view(k) for k in range(2 + 2 * n_aux)]
    frame = Frame(views[0], views[1], views[2::2], views[3::2], [int(p) for p in z["aux_priority"]])
    ci = z["client_ints"]
    client = Client(int(ci[0]), int(ci[1]), float(z["client_alpha"]), z["client_vp"], z["client_ivp"], int(ci[2]),
                    int(ci[3]), bool(ci[4]), int(ci[5]))
    expected = {
        "out": z["out"],
        "splat": [z[f"v{k}_splat"] for k in range(len(views))],
        "cam_ff": [z[f"v{k}_cam_ff"] if f"v{k}_cam_ff" in z else None for k in range(len(views))],
        "full_ff": [z[f"v{k}_full_ff"] if f"v{k}_full_ff" in z else None for k in range(len(views))],
        "meta": str(z["meta"]),
    }
    return frame, client, z["prev"], expected


def cases() -> list[str]:
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))
