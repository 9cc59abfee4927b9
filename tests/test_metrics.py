"""Image quality metrics (include/isti_metrics.h) against the reference's own
evaluation code.

tests/golden/metrics/pairs.npz holds seeded image pairs with the PSNR and SSIM that
scripts/eval.py's psnr_fn and scripts/loss_utils.ssim compute for them (torch,
CPU; tests/golden/make_golden.py metrics).  The numpy oracle (oracle/metrics.py)
is pinned to those values on the CPU; the GPU kernels are compared with both.
Tolerances: SSIM 1e-5, PSNR 1e-4 dB (the reference computes in float32).
"""
import os

import numpy as np
import pytest

from oracle import metrics as om

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "metrics", "pairs.npz")
NAMES = ("noise", "odd", "tiny", "tall", "smooth", "identical")
SSIM_TOL, PSNR_TOL = 1e-5, 1e-4


def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def close_psnr(a, b):
    return (np.isinf(a) and np.isinf(b)) or abs(a - b) <= PSNR_TOL


def test_oracle_matches_reference_metrics():
    g = golden()
    for n in NAMES:
        a, b = g[n + "_a"], g[n + "_b"]
        assert abs(om.ssim(a, b) - float(g[n + "_ssim"])) <= SSIM_TOL, n
        assert close_psnr(om.psnr(a, b), float(g[n + "_psnr"])), n


@pytest.mark.gpu
def test_gpu_metrics_match_reference_and_oracle(cuda):
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.metrics import quality

    g = golden()
    for n in NAMES:
        a, b = g[n + "_a"], g[n + "_b"]
        q = quality(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda))
        assert abs(q["ssim"] - float(g[n + "_ssim"])) <= SSIM_TOL, (n, q)
        assert close_psnr(q["psnr"], float(g[n + "_psnr"])), (n, q)
        assert abs(q["ssim"] - om.ssim(a, b)) <= SSIM_TOL, (n, q)
        assert abs(q["mse"] - om.mse(a, b)) <= 1e-12, (n, q)
    q = quality(torch.from_numpy(g["identical_a"]).to(cuda), torch.from_numpy(g["identical_b"]).to(cuda))
    assert q["mse"] == 0.0 and np.isinf(q["psnr"]) and q["ssim"] == 1.0


@pytest.mark.gpu
def test_gpu_metrics_interpolated_1080p_frame(cuda):
    """The use the metrics serve: an interpolated 1080p frame against the
    keyframe it approaches; deterministic across runs."""
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.metrics import Quality
    from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer
    from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence

    seq = Sequence(1920, 1080, 2, seed=5, aux_offsets=(-0.3, 0.3), shadows=True)
    client = seq.client(0, 3)
    frame = DeviceFrame.from_host(seq.frame(0), cuda)
    out = torch.zeros((1080, 1920, 4), dtype=torch.uint8, device=cuda)
    r = Renderer()
    r.render(out, client, frame)
    truth = torch.from_numpy(seq.keyframe(1, 0).color).to(cuda)
    q = Quality(1920, 1080)
    first = q(out, truth)
    for _ in range(3):
        assert q(out, truth) == first  # fixed-order reductions: bitwise identical
    host_out = out.cpu().numpy()
    assert abs(first["ssim"] - om.ssim(host_out, seq.keyframe(1, 0).color)) <= SSIM_TOL
    assert close_psnr(first["psnr"], om.psnr(host_out, seq.keyframe(1, 0).color))
    assert 10.0 < first["psnr"] < 60.0 and 0.3 < first["ssim"] < 1.0
    r.close()


@pytest.mark.gpu
def test_gpu_metrics_reject_bad_arguments(cuda):
    import torch
    from imagebasedspatiotemporalinterpolation_gb300 import native
    from imagebasedspatiotemporalinterpolation_gb300.metrics import Quality

    lib = native.load()
    assert lib.isti_quality_rgba8(None, None, 4, 4, None, None, None) == native.ISTI_ERR_INVALID_ARG
    q = Quality(8, 8)
    with pytest.raises(ValueError):
        q(torch.zeros((8, 8, 3), dtype=torch.uint8, device=cuda), torch.zeros((8, 8, 3), dtype=torch.uint8, device=cuda))


FLIP_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "metrics", "flip.npz")
FLIP_NAMES = ("noise", "odd", "tiny", "tall", "smooth", "identical", "render")
FLIP_MEAN_TOL, FLIP_PIXEL_TOL = 1e-4, 2e-3


def flip_golden():
    with np.load(FLIP_GOLDEN) as z:
        return {k: z[k] for k in z.files}


def test_flip_oracle_matches_reference():
    """oracle/flip.py against the reference's scripts/flip_loss.py (LDRFLIPLoss), run by
    tests/golden/make_golden.py flip: means within 1e-6, maps within 1e-4."""
    from oracle import flip as of

    g = flip_golden()
    for n in FLIP_NAMES:
        assert abs(of.flip(g[n + "_a"], g[n + "_b"]) - float(g[n + "_flip"])) <= 1e-6, n
    for n in ("odd", "render"):
        assert np.abs(of.flip_map(g[n + "_a"], g[n + "_b"]) - g[n + "_map"]).max() <= 1e-4, n


@pytest.mark.gpu
def test_gpu_flip_matches_reference(cuda):
    """GPU LDR-FLIP (separable float32 filters) against the reference's values: mean within
    1e-4, per pixel within 2e-3 (float32 power functions near zero)."""
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.metrics import Quality

    g = flip_golden()
    for n in FLIP_NAMES:
        a, b = g[n + "_a"], g[n + "_b"]
        q = Quality(a.shape[1], a.shape[0])
        mean, fmap = q.flip(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), with_map=True)
        assert abs(mean - float(g[n + "_flip"])) <= FLIP_MEAN_TOL, (n, mean, float(g[n + "_flip"]))
        if n + "_map" in g:
            assert np.abs(fmap.cpu().numpy() - g[n + "_map"]).max() <= FLIP_PIXEL_TOL, n
        assert abs(mean - float(fmap.double().mean())) <= 1e-9


@pytest.mark.gpu
def test_gpu_flip_1080p_matches_oracle(cuda):
    """A 1080p interpolated frame against its ground truth: GPU vs the float64 oracle, and
    bitwise-identical repeated runs."""
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.metrics import Quality
    from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer
    from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence
    from oracle import flip as of

    seq = Sequence(1920, 1080, 2, seed=7, aux_offsets=(-0.3, 0.3), shadows=True)
    frame = DeviceFrame.from_host(seq.frame(0), cuda)
    out = torch.zeros((1080, 1920, 4), dtype=torch.uint8, device=cuda)
    r = Renderer()
    r.render(out, seq.client(0, 2), frame)
    truth = seq.ground_truth(0, 2)
    q = Quality(1920, 1080)
    got = q.flip(out, torch.from_numpy(truth).to(cuda))
    assert q.flip(out, torch.from_numpy(truth).to(cuda)) == got
    assert abs(got - of.flip(out.cpu().numpy(), truth)) <= FLIP_MEAN_TOL
    r.close()


@pytest.mark.gpu
def test_gpu_flip_rejects_large_radius(cuda):
    import torch
    from imagebasedspatiotemporalinterpolation_gb300 import native
    from imagebasedspatiotemporalinterpolation_gb300.metrics import Quality

    q = Quality(16, 16)
    img = torch.zeros((16, 16, 4), dtype=torch.uint8, device=cuda)
    with pytest.raises(native.IstiError):
        q.flip(img, img, pixels_per_degree=500.0)
