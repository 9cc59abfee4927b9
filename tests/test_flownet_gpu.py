"""The learned flow initialiser's network on the GPU against its float64 oracle.

oracle/flownet.py restates the architecture, the loss and every gradient in
numpy (its gradients are pinned to finite differences in test_flownet_oracle.py).
With bf16 emulation it rounds what the GPU stores in bf16, so the GPU's forward
flow must match within 1 % of the flow scale, the loss within 1e-3 relative, and
each layer's weight and bias gradient within 3 % (relative L2) with cosine
similarity >= 0.999.  A short training run on a fixed batch must reduce the loss.
"""
import numpy as np
import pytest

import oracle.flownet as OF
from imagebasedspatiotemporalinterpolation_gb300.flownet import FlowNet

pytestmark = pytest.mark.gpu


def _batch(seed, n=2, h=24, w=48):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn(n, h, w, 16, generator=g).bfloat16()
    label = torch.randn(n, h, w, 4, generator=g) * 0.5
    label[0, :3, :5, 1] = float("nan")  # unlabelled entries
    return x.cuda(), label.cuda()


def test_forward_and_gradients_match_oracle(cuda):
    import torch
    net = FlowNet(seed=3)
    x, label = _batch(11)
    flow = net.forward(x)
    torch.cuda.synchronize()
    params = net.params().cpu().numpy().astype(np.float64)
    xn = x.float().cpu().numpy().astype(np.float64)
    loss_ref, grad_ref, acts = OF.loss_and_grads(params, xn, label.cpu().numpy().astype(np.float64), bf16=True)
    got = flow.cpu().numpy()
    assert np.abs(got - acts["flow"]).max() <= 1e-2 * np.abs(acts["flow"]).max()

    net.backward(x, label)
    loss = net.loss()
    grads = net.grads().cpu().numpy().astype(np.float64)
    assert net.device_status() == 0
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref)
    offs, _ = OF.offsets()
    for li, ((taps, cin, cout, _), (wo, bo)) in enumerate(zip(OF.LAYERS, offs)):
        for name, lo, hi in (("w", wo, wo + taps * cin * cout), ("b", bo, bo + cout)):
            a, b = grads[lo:hi], grad_ref[lo:hi]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            cos = float(a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))
            assert rel <= 3e-2 and cos >= 0.999, f"layer {li} {name}: rel {rel:.3g} cos {cos:.5f}"
    net.close()


def test_training_reduces_loss(cuda):
    """Labels that are a learnable function of the input (a per-pixel linear map of the
    first channels) must be fitted: the loss halves within 60 Adam steps."""
    import torch
    net = FlowNet(seed=4)
    x, _ = _batch(12)
    mix = torch.tensor([[0.8, -0.3, 0.0, 0.5], [0.2, 0.6, -0.4, 0.0], [0.0, 0.1, 0.9, -0.2], [-0.5, 0.0, 0.3, 0.7]], device="cuda")
    label = (x.float()[..., :4] @ mix).contiguous()
    net.backward(x, label)
    first = net.loss()
    for _ in range(60):
        net.backward(x, label)
        net.adam(3e-3)
    net.backward(x, label)
    torch.cuda.synchronize()
    assert net.device_status() == 0
    assert net.loss() < 0.5 * first, (first, net.loss())
    net.close()


def test_forward_with_fused_head_matches_oracle(cuda):
    """Rows of 128 pixels or more run the last 3x3 layer on the row-tile kernel, whose
    epilogue also computes the 1x1 head (the layer's own output is then not stored): the
    flow matches the oracle like the separate head's, and the f16 copy is the f32 flow
    rounded."""
    import torch
    net = FlowNet(seed=4)
    x, _ = _batch(12, n=1, h=16, w=160)
    f32 = torch.empty((1, 16, 160, 4), dtype=torch.float32, device="cuda")
    f16 = torch.empty((1, 16, 160, 4), dtype=torch.float16, device="cuda")
    net.forward(x, flow=f32, flow16=f16)
    torch.cuda.synchronize()
    assert net.device_status() == 0
    params = net.params().cpu().numpy().astype(np.float64)
    acts = OF.forward(params, x.float().cpu().numpy().astype(np.float64), True)
    got = f32.cpu().numpy()
    assert np.abs(got - acts["flow"]).max() <= 1e-2 * np.abs(acts["flow"]).max()
    assert torch.equal(f16, f32.half())
    net.close()
