"""isti_render_noalloc: rendering without any device allocation.

Some callers cannot allocate device memory while they run: their device
budget is reserved up front by their own memory pool, or they run a
real-time loop in which cudaMalloc/cudaFree may synchronise the device and
miss the frame deadline.  For them the library renders with a fixed scratch
array it owns.  This file checks, through the C ABI, that the result is the
same as isti_render's (bit-exact, the tolerance every parity test here uses)
on two calls in a row, and that frames larger than the scratch are refused.
It is collected last so that a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest

from imagebasedspatiotemporalinterpolation_gb300 import native
from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer, render_info
from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence

pytestmark = pytest.mark.gpu


def _noalloc(out, client, frame):
    import torch
    lib = native.load()
    ri = render_info(client)
    return lib.isti_render_noalloc(C.c_void_p(out.data_ptr()), C.byref(ri), C.byref(frame.to_c()),
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_matches_isti_render_twice(cuda):
    import torch
    seq = Sequence(320, 180, 3, seed=77, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0)
    r = Renderer()
    for k, b in ((0, 1), (1, 3)):  # two calls in a row, different frames
        frame = DeviceFrame.from_host(seq.frame(k))
        client = seq.client(k, b)
        prev = torch.full((180, 320, 4), 5, dtype=torch.uint8, device="cuda")
        want = prev.clone()
        got = prev.clone()
        r.render(want, client, frame)
        assert _noalloc(got, client, frame) == native.ISTI_OK, native.load().isti_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"frame {k}: {int((got != want).any(-1).sum())} pixels differ"
        assert bool((want != prev).any())
    r.close()


def test_noalloc_rejects_frames_beyond_scratch(cuda):
    import torch
    seq = Sequence(1280, 720, 2, seed=78, aux_offsets=(-0.3, 0.3))
    frame = DeviceFrame.from_host(seq.frame(0))
    out = torch.zeros((720, 1280, 4), dtype=torch.uint8, device="cuda")
    assert _noalloc(out, seq.client(0, 2), frame) == native.ISTI_ERR_INVALID_ARG
    msg = native.load().isti_last_error().decode()
    assert "scratch" in msg and str(native.NOALLOC_SCRATCH_BYTES) in msg
