"""Generates the golden fixtures of tests/golden from the reference renderer.

Runs the reference's own src/renderer.cu (compiled for the CPU by
oracle/build_ref.py, so it needs the reference tree) on small seeded
procedural scenes and stores inputs and outputs with fixtures.save().

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence  # noqa: E402
from tests.golden import fixtures  # noqa: E402


def pattern(h, w):
    y, x = np.mgrid[0:h, 0:w]
    return np.stack([(x * 7) % 256, (y * 13) % 256, (x + y) % 256, np.full_like(x, 255)], -1).astype(np.uint8)


def case(name, seq, k, b, mode=0, no_shadows=False, patch=None, drop_motion=False, meta=""):
    frame = seq.frame(k)
    if drop_motion:
        for v in frame.views():
            v.motion = None
    if patch:
        patch(frame)
    client = seq.client(k, b, mode=mode, no_shadows=no_shadows)
    prev = pattern(client.height, client.width)
    out, splats, cams, fulls = oracle.run_reference(frame, client, prev)
    if client.width * client.height > 10000:  # keep large fixtures small: keys + image only
        cams = fulls = None
    fixtures.save(os.path.join(fixtures.GOLDEN_DIR, name + ".npz"), frame, client, prev, out, splats, cams, fulls, meta)
    valid = int((out != prev).any(-1).sum())
    print(f"{name}: {client.width}x{client.height} views={len(frame.views())} mode={mode} t={client.alpha} changed={valid}")


def nan_levels(frame):
    # constant non-zero shadow levels (0b01 in all four sub-frames): the reference's
    # (my - min) / (max - min) is 0 / 0 there (src/renderer.cu:256)
    for v in frame.views():
        if v.shadow_info is not None:
            v.shadow_info = v.shadow_info.copy()
            v.shadow_info[10:20, :, 0] = 0
            v.shadow_info[10:20, :, 1] = 0
            v.shadow_info[10:20, :, 2] = 0x55


def timewarp_cases():
    tw = Sequence(160, 90, 2, seed=15, aux_offsets=(0.3,), aux_size=(80, 45))
    case("tw_aux_half_res_t025_mode4", tw, 0, 1, mode=4, meta="timewarp with an aux fallback camera")
    tw_main = Sequence(128, 72, 2, seed=16)
    case("tw_main_t075_mode4", tw_main, 0, 3, mode=4, meta="timewarp, main camera only")


def main():
    oracle.build()
    if not oracle.reference_available():
        raise SystemExit("reference renderer not built (needs the reference tree)")
    if sys.argv[1:] == ["timewarp"]:
        timewarp_cases()
        return
    timewarp_cases()
    c1 = Sequence(320, 180, 3, seed=11)
    case("c1_t050_mode0", c1, 0, 2, meta="main only, no shadows")
    case("c1_t025_mode3", c1, 1, 1, mode=3, meta="splatting only")
    case("c1_t075_mode1", c1, 0, 3, mode=1, meta="backward bidirectional, 7x7 window, 5 iterations")
    # faster spheres than the benchmark scene so that more pixels carry shadow gradients
    c2 = Sequence(96, 54, 3, seed=12, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=4.0)
    case("c2_aux_shadow_t025_mode0", c2, 0, 1, meta="two aux cameras, soft shadows")
    case("c2_aux_shadow_t050_mode2", c2, 1, 2, mode=2, meta="backward unidirectional (same code as mode 0)")
    case("c2_aux_shadow_t075_mode1", c2, 0, 3, mode=1, meta="mode 1 with aux cameras")
    case("c2_noshadow_flag_t050", c2, 0, 2, no_shadows=True, meta="shadow buffers present, -ns set")
    case("c2_nan_levels_t025", c2, 0, 1, patch=nan_levels, meta="constant non-zero shadow levels")
    odd = Sequence(37, 23, 2, seed=13)
    case("odd_nomotion_t050_mode2", odd, 0, 2, mode=2, drop_motion=True, meta="odd size, no object motion")
    low = Sequence(128, 72, 2, seed=14, aux_offsets=(0.3,), aux_size=(64, 36), shadows=True, max_speed=4.0)
    case("aux_half_res_t050", low, 0, 2, meta="one aux camera at half resolution")


if __name__ == "__main__":
    main()
