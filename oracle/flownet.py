"""Float64 restatement of the learned flow initialiser -- TEST INFRASTRUCTURE ONLY.

The checker of the tensor-core network in libisti.so (include/isti_unet.h,
csrc/isti_flownet.cu): forward pass, loss and every parameter gradient, written
directly from the architecture with numpy (no autograd).  The network has no
counterpart in the reference (whose renderer starts its search from splatting,
src/renderer.cu:148-202), so there is nothing of the reference to pin it to; the
tests compare the GPU against this restatement, and the restatement's gradients
against finite differences of its own loss.

With ``bf16=True`` every tensor the GPU stores in bf16 (activations, activation
gradients, the packed convolution weights) is rounded to bf16 here too, so the
remaining difference is the f32 accumulation order of the GPU.
"""
from __future__ import annotations

import numpy as np

# (taps, cin, cout, relu) of layers 0..9 (e1 e2 e3 e4 p3 d3 p2 d2 p1 d1) and the head
LAYERS = [(9, 16, 32, 1), (9, 32, 64, 1), (9, 64, 96, 1), (9, 96, 128, 1), (1, 128, 96, 0),
          (9, 96, 96, 1), (1, 96, 64, 0), (9, 64, 64, 1), (1, 64, 32, 0), (9, 32, 32, 1), (1, 32, 4, 0)]


def offsets():
    """(w_off, b_off) per layer in the flat parameter array (tensors 16-byte aligned)."""
    out, off = [], 0
    for taps, cin, cout, _ in LAYERS:
        w = off
        off += taps * cin * cout
        b = off
        off += cout
        off = (off + 3) // 4 * 4
        out.append((w, b))
    return out, off


def bf16_round(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, bf16=False):
    """Per layer (W [cout, taps, cin], b [cout]) from the flat f32 array."""
    offs, _ = offsets()
    out = []
    for li, ((taps, cin, cout, _), (wo, bo)) in enumerate(zip(LAYERS, offs)):
        w = np.asarray(params[wo:wo + taps * cin * cout], np.float64).reshape(cout, taps, cin)
        if bf16 and li < 10:  # the tensor-core layers use bf16 weights; the head keeps f32
            w = bf16_round(w)
        out.append((w, np.asarray(params[bo:bo + cout], np.float64)))
    return out


def conv(x, w, b=None):
    """NHWC convolution, stride 1, zero padding 1 for 3x3 (tap = 3 (dy+1) + (dx+1))."""
    taps = w.shape[1]
    if taps == 1:
        y = x @ w[:, 0, :].T
    else:
        n, h, wd, _ = x.shape
        xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
        y = np.zeros((n, h, wd, w.shape[0]))
        for t in range(9):
            dy, dx = t // 3 - 1, t % 3 - 1
            y += xp[:, 1 + dy:1 + dy + h, 1 + dx:1 + dx + wd, :] @ w[:, t, :].T
    return y if b is None else y + b


def conv_dgrad(g, w):
    """Gradient of conv's input: the convolution with transposed, mirrored taps."""
    wt = np.transpose(w, (2, 1, 0))[:, ::-1, :] if w.shape[1] == 9 else np.transpose(w, (2, 1, 0))
    return conv(g, np.ascontiguousarray(wt))


def conv_wgrad(g, x, taps):
    """dW[co, tap, ci] = sum over pixels of g[p, co] x[p + offset(tap), ci]."""
    if taps == 1:
        return np.einsum("nhwc,nhwd->cd", g, x)[:, None, :]
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((g.shape[-1], 9, x.shape[-1]))
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        out[:, t, :] = np.einsum("nhwc,nhwd->cd", g, xp[:, 1 + dy:1 + dy + h, 1 + dx:1 + dx + wd, :])
    return out


def pool(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def downsum(g):
    n, h, w, c = g.shape
    return g.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def forward(params, x, bf16=False):
    """Activations of every layer and the f64 flow (n, h, w, 4)."""
    L = unpack(params, bf16)
    r = bf16_round if bf16 else (lambda a: a)
    relu = lambda a: np.maximum(a, 0.0)
    a = {"x": np.asarray(x, np.float64)}
    a["e1"] = r(relu(conv(a["x"], *L[0])))
    a["q1"] = r(pool(a["e1"]))
    a["e2"] = r(relu(conv(a["q1"], *L[1])))
    a["q2"] = r(pool(a["e2"]))
    a["e3"] = r(relu(conv(a["q2"], *L[2])))
    a["q3"] = r(pool(a["e3"]))
    a["e4"] = r(relu(conv(a["q3"], *L[3])))
    a["p3"] = r(conv(a["e4"], *L[4]))
    a["s3"] = r(up(a["p3"]) + a["e3"])
    a["d3"] = r(relu(conv(a["s3"], *L[5])))
    a["p2"] = r(conv(a["d3"], *L[6]))
    a["s2"] = r(up(a["p2"]) + a["e2"])
    a["d2"] = r(relu(conv(a["s2"], *L[7])))
    a["p1"] = r(conv(a["d2"], *L[8]))
    a["s1"] = r(up(a["p1"]) + a["e1"])
    a["d1"] = r(relu(conv(a["s1"], *L[9])))
    a["flow"] = conv(a["d1"], *L[10])
    return a


def loss_and_grads(params, x, label, bf16=False):
    """Huber loss (delta 1, NaN labels skipped, divided by n*h*w) and the flat gradient."""
    L = unpack(params, bf16)
    r = bf16_round if bf16 else (lambda v: v)
    a = forward(params, x, bf16)
    n, h, w, _ = a["flow"].shape
    norm = n * h * w
    lab = np.asarray(label, np.float64)
    valid = ~np.isnan(lab)
    d = np.where(valid, a["flow"] - np.nan_to_num(lab), 0.0)
    ad = np.abs(d)
    loss = float(np.where(ad < 1, 0.5 * d * d, ad - 0.5).sum() / norm)
    gflow = np.clip(d, -1, 1) / norm
    grads = [None] * len(LAYERS)

    def wb(li, g, xin):
        grads[li] = (conv_wgrad(g, xin, LAYERS[li][0]), g.sum(axis=(0, 1, 2)))

    grads[10] = (np.einsum("nhwc,nhwd->cd", gflow, a["d1"])[:, None, :], gflow.sum(axis=(0, 1, 2)))
    g_d1 = r((gflow @ L[10][0][:, 0, :]) * (a["d1"] > 0))
    wb(9, g_d1, a["s1"])
    g_s1 = r(conv_dgrad(g_d1, L[9][0]))
    g_p1 = r(downsum(g_s1))
    wb(8, g_p1, a["d2"])
    g_d2 = r(conv_dgrad(g_p1, L[8][0]) * (a["d2"] > 0))
    wb(7, g_d2, a["s2"])
    g_s2 = r(conv_dgrad(g_d2, L[7][0]))
    g_p2 = r(downsum(g_s2))
    wb(6, g_p2, a["d3"])
    g_d3 = r(conv_dgrad(g_p2, L[6][0]) * (a["d3"] > 0))
    wb(5, g_d3, a["s3"])
    g_s3 = r(conv_dgrad(g_d3, L[5][0]))
    g_p3 = r(downsum(g_s3))
    wb(4, g_p3, a["e4"])
    g_e4 = r(conv_dgrad(g_p3, L[4][0]) * (a["e4"] > 0))
    wb(3, g_e4, a["q3"])
    g_q3 = r(conv_dgrad(g_e4, L[3][0]))
    g_e3 = r((g_s3 + 0.25 * up(g_q3)) * (a["e3"] > 0))
    wb(2, g_e3, a["q2"])
    g_q2 = r(conv_dgrad(g_e3, L[2][0]))
    g_e2 = r((g_s2 + 0.25 * up(g_q2)) * (a["e2"] > 0))
    wb(1, g_e2, a["q1"])
    g_q1 = r(conv_dgrad(g_e2, L[1][0]))
    g_e1 = r((g_s1 + 0.25 * up(g_q1)) * (a["e1"] > 0))
    wb(0, g_e1, a["x"])
    offs, total = offsets()
    flat = np.zeros(total)
    for (gw, gb), (wo, bo) in zip(grads, offs):
        flat[wo:wo + gw.size] = gw.reshape(-1)
        flat[bo:bo + gb.size] = gb
    return loss, flat, a
