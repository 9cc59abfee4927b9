"""isti_render_noalloc: rendering without any device allocation.

Some callers cannot allocate device memory while they run: their device
budget is reserved up front by their own memory pool, or they run a
real-time loop in which cudaMalloc/cudaFree may synchronise the device and
miss the frame deadline.  For them the library renders with a fixed scratch
array it owns.  This file checks, through the C ABI, that the result is the
same as isti_render's (bit-exact, the tolerance every parity test here uses)
on two calls in a row (also in timewarp mode, whose scratch layout and kernels
differ), that its device status word reads ISTI_OK afterwards, that a
warmed-up call leaves the device's free memory unchanged, and that frames
larger than the scratch are refused.  It is collected last so that a failure
here leaves every other test run.
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


def _status():
    s = C.c_int32(-1)
    assert native.load().isti_noalloc_device_status(C.byref(s)) == native.ISTI_OK
    return s.value


def test_noalloc_status_word_reads_ok_after_calls(cuda):
    import torch
    seq = Sequence(160, 96, 2, seed=79)
    frame = DeviceFrame.from_host(seq.frame(0))
    out = torch.zeros((96, 160, 4), dtype=torch.uint8, device="cuda")
    for b in (1, 2):
        assert _noalloc(out, seq.client(0, b), frame) == native.ISTI_OK
        assert _status() == native.ISTI_OK


def test_noalloc_timewarp_matches_isti_render_twice(cuda):
    import torch
    seq = Sequence(320, 180, 3, seed=80, aux_offsets=(0.3,))
    r = Renderer()
    for k, b in ((0, 1), (1, 2)):
        frame = DeviceFrame.from_host(seq.frame(k))
        client = seq.client(k, b, mode=native.MODE_TIMEWARP)
        prev = torch.full((180, 320, 4), 9, dtype=torch.uint8, device="cuda")
        want, got = prev.clone(), prev.clone()
        r.render(want, client, frame)
        assert _noalloc(got, client, frame) == native.ISTI_OK, native.load().isti_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"frame {k}: {int((got != want).any(-1).sum())} pixels differ"
        assert _status() == native.ISTI_OK
    r.close()


def test_noalloc_allocates_no_device_memory(cuda):
    """Free device memory is the same before and after a warmed-up call (the torch
    allocator is idle in between, so any change would be the call's own)."""
    import torch
    seq = Sequence(320, 180, 2, seed=81, aux_offsets=(0.3,), shadows=True)
    frame = DeviceFrame.from_host(seq.frame(0))
    out = torch.zeros((180, 320, 4), dtype=torch.uint8, device="cuda")
    clients = [seq.client(0, 2), seq.client(0, 2, mode=native.MODE_TIMEWARP)]
    for c in clients:  # warm-up: modules of both modes loaded
        assert _noalloc(out, c, frame) == native.ISTI_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for c in clients:
        assert _noalloc(out, c, frame) == native.ISTI_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"


def test_noalloc_rejects_frames_beyond_scratch(cuda):
    import torch
    seq = Sequence(1280, 720, 2, seed=78, aux_offsets=(-0.3, 0.3))
    frame = DeviceFrame.from_host(seq.frame(0))
    out = torch.zeros((720, 1280, 4), dtype=torch.uint8, device="cuda")
    assert _noalloc(out, seq.client(0, 2), frame) == native.ISTI_ERR_INVALID_ARG
    msg = native.load().isti_last_error().decode()
    assert "scratch" in msg and str(native.NOALLOC_SCRATCH_BYTES) in msg
