"""The tcgen05 convolution operators against a plain PyTorch fp32 reference.

isti_unet_conv (forward, and the data gradient through transposed packed weights)
and isti_unet_wgrad (weight gradient) run on bf16 operands with f32 accumulation in
TMEM.  The reference convolves the same bf16-rounded inputs and weights in fp32, so
the bound is the bf16 rounding of the stored output (half an ulp, |y| * 2^-8) plus
accumulation-order noise: |got - ref| <= |ref| * 2^-7 + 1e-3 for bf16 outputs, and
1e-4 of the output scale for the f32 weight gradient.
"""
import ctypes as C

import pytest

from imagebasedspatiotemporalinterpolation_gb300 import native

pytestmark = pytest.mark.gpu

SHAPES = [(9, 16, 32), (9, 32, 64), (9, 64, 96), (9, 96, 128), (1, 128, 96), (9, 96, 96), (1, 96, 64), (9, 64, 64), (1, 64, 32),
          (9, 32, 32)]


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _w4d(w, taps, cin, cout):
    k = 3 if taps == 9 else 1
    return w.view(cout, k, k, cin).permute(0, 3, 1, 2)


def _pack(lib, w, taps, cin, cout, transpose):
    import torch
    out = torch.empty(taps * cin * cout, dtype=torch.bfloat16, device="cuda")
    assert lib.isti_unet_pack(taps, _p(w), cin, cout, transpose, _p(out), None) == native.ISTI_OK
    return out


@pytest.mark.parametrize("taps,cin,cout", SHAPES, ids=lambda v: str(v))
def test_conv_dgrad_wgrad_match_torch(cuda, taps, cin, cout):
    import torch
    import torch.nn.functional as F
    lib = native.load()
    torch.manual_seed(taps * 1000 + cin * 10 + cout)
    n, h, w = 2, 24, 40  # not a multiple of the 16 x 8 tile: ragged edge tiles
    pad = 1 if taps == 9 else 0
    status = torch.zeros(64, dtype=torch.int32, device="cuda")
    x = torch.randn(n, h, w, cin, device="cuda").bfloat16()
    wt = torch.randn(cout, taps, cin, device="cuda") * (2.0 / (taps * cin)) ** 0.5
    wb = wt.bfloat16().float()
    bias = torch.randn(cout, device="cuda") * 0.1
    mask = torch.randn(n, h, w, cout, device="cuda").bfloat16()

    # forward with bias, ReLU and a gradient mask
    out = torch.empty(n, h, w, cout, dtype=torch.bfloat16, device="cuda")
    wp = _pack(lib, wt, taps, cin, cout, 0)
    assert lib.isti_unet_conv(taps, _p(x), n, h, w, cin, _p(wp), _p(bias), _p(mask), 1, _p(out), cout, _p(status), None) == 0
    ref = F.conv2d(x.float().permute(0, 3, 1, 2), _w4d(wb, taps, cin, cout), bias, padding=pad).relu().permute(0, 2, 3, 1)
    ref = ref * (mask.float() > 0)
    torch.cuda.synchronize()
    assert ((out.float() - ref).abs() <= ref.abs() * 2 ** -7 + 1e-3).all()

    # data gradient: the packed transposed convolution
    dy = torch.randn(n, h, w, cout, device="cuda").bfloat16()
    dx = torch.empty(n, h, w, cin, dtype=torch.bfloat16, device="cuda")
    wpt = _pack(lib, wt, taps, cin, cout, 1)
    assert lib.isti_unet_conv(taps, _p(dy), n, h, w, cout, _p(wpt), None, None, 0, _p(dx), cin, _p(status), None) == 0
    refdx = torch.nn.grad.conv2d_input((n, cin, h, w), _w4d(wb, taps, cin, cout), dy.float().permute(0, 3, 1, 2), padding=pad)
    refdx = refdx.permute(0, 2, 3, 1)
    torch.cuda.synchronize()
    assert ((dx.float() - refdx).abs() <= refdx.abs() * 2 ** -7 + 1e-3).all()

    # weight gradient, also accumulated onto an existing gradient
    k = 3 if taps == 9 else 1
    refdw = torch.nn.grad.conv2d_weight(x.float().permute(0, 3, 1, 2), (cout, cin, k, k), dy.float().permute(0, 3, 1, 2), padding=pad)
    refdw = refdw.permute(0, 2, 3, 1).reshape(cout, taps, cin)
    nbytes = lib.isti_unet_wgrad_scratch_bytes(taps, n, h, w, cin, cout)
    scratch = torch.empty(nbytes // 4 + 1, dtype=torch.float32, device="cuda")
    dw = torch.full((cout, taps, cin), 0.5, device="cuda")
    assert lib.isti_unet_wgrad(taps, _p(dy), _p(x), n, h, w, cin, cout, _p(dw), 0, _p(scratch), nbytes, _p(status), None) == 0
    torch.cuda.synchronize()
    scale = refdw.abs().max().item()
    assert (dw - refdw).abs().max().item() <= 1e-4 * scale
    assert lib.isti_unet_wgrad(taps, _p(dy), _p(x), n, h, w, cin, cout, _p(dw), 1, _p(scratch), nbytes, _p(status), None) == 0
    torch.cuda.synchronize()
    assert (dw - 2 * refdw).abs().max().item() <= 2e-4 * scale
    assert int(status[0].item()) == native.ISTI_OK


def test_conv_rejects_bad_shapes(cuda):
    import torch
    lib = native.load()
    x = torch.zeros(1, 8, 16, 24, dtype=torch.bfloat16, device="cuda")  # 24 channels: not a multiple of 16
    wp = torch.zeros(9 * 24 * 32, dtype=torch.bfloat16, device="cuda")
    out = torch.zeros(1, 8, 16, 32, dtype=torch.bfloat16, device="cuda")
    assert lib.isti_unet_conv(9, _p(x), 1, 8, 16, 24, _p(wp), None, None, 0, _p(out), 32, None, None) == native.ISTI_ERR_INVALID_ARG
