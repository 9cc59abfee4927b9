"""Generates the golden fixtures of tests/golden from the reference renderer.

Runs the reference's own src/renderer.cu (compiled for the CPU by
oracle/build_ref.py, so it needs the reference tree) on small seeded
procedural scenes and stores inputs and outputs with fixtures.save().

    python tests/golden/make_golden.py            (everything)
    python tests/golden/make_golden.py io         (codec fixtures only)
    python tests/golden/make_golden.py timewarp   (timewarp fixtures only)
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


def reference_dir() -> str:
    """The reference tree, named by the ISTI_REFERENCE_DIR environment variable."""
    ref = os.environ.get("ISTI_REFERENCE_DIR")
    if not ref or not os.path.isdir(ref):
        raise SystemExit("set ISTI_REFERENCE_DIR to the reference tree")
    return ref


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


IO_DIR = os.path.join(fixtures.GOLDEN_DIR, "io")


def io_cases():
    """Codec fixtures: PNG files of every colour type / depth / tRNS form /
    interlacing (tests/golden/png_writer.py) and from stb_image_write, EXR files
    from tinyexr in every compression it writes; expected decodes from the
    reference's own stb_image / LoadEXR (oracle/ref_io.py) in io/expected.npz."""
    from oracle import ref_io
    from tests.golden.png_writer import make_png

    os.makedirs(IO_DIR, exist_ok=True)
    rng = np.random.default_rng(2024)
    expected = {}

    def png(name, data):
        path = os.path.join(IO_DIR, name + ".png")
        with open(path, "wb") as f:
            f.write(data)
        expected[name + ".png"] = ref_io.png_load(path)

    h, w = 11, 19
    for depth in (1, 2, 4, 8, 16):
        s = rng.integers(0, 1 << depth, (h, w))
        png(f"grey{depth}", make_png(s, depth, 0))
        png(f"grey{depth}_trns", make_png(s, depth, 0, trns=int(s[3, 4]).to_bytes(2, "big")))
        png(f"grey{depth}_adam7", make_png(s, depth, 0, interlace=1))
        if depth <= 8:
            n = min(1 << depth, 200)
            sp = rng.integers(0, n, (h, w))
            pal = rng.integers(0, 256, 3 * n, dtype=np.uint8).tobytes()
            png(f"palette{depth}", make_png(sp, depth, 3, palette=pal))
            png(f"palette{depth}_trns", make_png(sp, depth, 3, palette=pal,
                                                 trns=rng.integers(0, 256, n // 2 + 1, dtype=np.uint8).tobytes()))
            png(f"palette{depth}_adam7", make_png(sp, depth, 3, palette=pal, interlace=1))
    for depth in (8, 16):
        for color in (2, 4, 6):
            ch = {2: 3, 4: 2, 6: 4}[color]
            s = rng.integers(0, 1 << depth, (13, 9, ch))
            s[5:8] = s[0:1, 0:1]
            png(f"color{color}_depth{depth}", make_png(s, depth, color))
            png(f"color{color}_depth{depth}_adam7", make_png(s, depth, color, interlace=1))
            if color == 2:
                key = b"".join(int(k).to_bytes(2, "big") for k in s[0, 0])
                png(f"color2_depth{depth}_trns", make_png(s, depth, color, trns=key))
    for comp in (1, 2, 3, 4):
        img = rng.integers(0, 256, (17, 23, comp), dtype=np.uint8)
        path = os.path.join(IO_DIR, f"stb_{comp}ch.png")
        ref_io.png_save(path, img)
        expected[f"stb_{comp}ch.png"] = ref_io.png_load(path)

    for comp_name, comp in (("none", 0), ("rle", 1), ("zips", 2), ("zip", 3), ("piz", 4)):
        for pt_name, pt in (("half", 1), ("float", 2)):
            for names in (["Y"], ["B", "G", "R"], ["A", "B", "G", "R", "Z"], ["G", "R"]):
                planes = (rng.standard_normal((len(names), 11, 17)) * 50).astype(np.float32)
                planes[:, 3:6] = 0.75  # runs for RLE
                name = f"{comp_name}_{pt_name}_{''.join(names)}.exr"
                path = os.path.join(IO_DIR, name)
                ref_io.exr_save(path, planes, names, pt, comp)
                expected[name] = ref_io.exr_load(path)
    # PIZ over three 32-line blocks (the last one partial), smooth and noisy planes
    prng = np.random.default_rng(4242)  # own stream: the files above do not change
    yy, xx = np.mgrid[0:70, 0:45].astype(np.float32)
    for pt_name, pt in (("half", 1), ("float", 2)):
        planes = np.stack([xx * 0.37 - yy, np.sin(xx * 0.2) * 40 + yy, prng.standard_normal((70, 45)) * 3000,
                           prng.integers(0, 4, (70, 45)).astype(np.float32)]).astype(np.float32)
        name = f"piz_blocks_{pt_name}_ABGR.exr"
        path = os.path.join(IO_DIR, name)
        ref_io.exr_save(path, planes, ["A", "B", "G", "R"], pt, 4)
        expected[name] = ref_io.exr_load(path)
    np.savez_compressed(os.path.join(IO_DIR, "expected.npz"),
                        **{k: (np.array(v) if isinstance(v, str) else v) for k, v in expected.items()})
    print(f"io: {len(expected)} files")


def metrics_cases(reference=None):
    """PSNR / SSIM of seeded image pairs by the reference's own evaluation code:
    scripts/loss_utils.ssim and eval.py's psnr_fn (torch, CPU), on (1, 3, H, W)
    float tensors of the RGB bytes / 255 as eval.py's loader makes them."""
    import torch
    import torch.nn.functional as F

    sys.path.insert(0, os.path.join(reference or reference_dir(), "scripts"))
    from loss_utils import ssim  # the reference's implementation

    rng = np.random.default_rng(77)
    pairs = {}
    for name, (h, w) in (("noise", (30, 40)), ("odd", (45, 67)), ("tiny", (5, 8)), ("tall", (70, 12))):
        a = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        b = np.clip(a.astype(int) + rng.integers(-40, 41, (h, w, 4)), 0, 255).astype(np.uint8)
        pairs[name] = (a, b)
    yy, xx = np.mgrid[0:48, 0:64]
    smooth = np.stack([(xx * 4) % 256, (yy * 5) % 256, (xx + yy) % 256, np.full_like(xx, 255)], -1).astype(np.uint8)
    pairs["smooth"] = (smooth, np.roll(smooth, 1, axis=1))
    pairs["identical"] = (smooth, smooth.copy())
    out = {}
    for name, (a, b) in pairs.items():
        ta = torch.from_numpy(np.ascontiguousarray(np.moveaxis(a[..., :3], -1, 0))).float().unsqueeze(0) / 255.0
        tb = torch.from_numpy(np.ascontiguousarray(np.moveaxis(b[..., :3], -1, 0))).float().unsqueeze(0) / 255.0
        s = ssim(ta, tb).mean().item()
        p = (-10.0 * torch.log(F.mse_loss(ta, tb)) / np.log(10.0)).item()
        out[f"{name}_a"], out[f"{name}_b"] = a, b
        out[f"{name}_ssim"], out[f"{name}_psnr"] = np.float64(s), np.float64(p)
    os.makedirs(os.path.join(fixtures.GOLDEN_DIR, "metrics"), exist_ok=True)
    np.savez_compressed(os.path.join(fixtures.GOLDEN_DIR, "metrics", "pairs.npz"), **out)
    print(f"metrics: {len(pairs)} pairs")


def flip_cases(reference=None):
    """LDR-FLIP (eval.py's flip_fn(render, ground_truth)) of the metric pairs plus an
    interpolated frame against its analytic ground truth, computed by the
    reference's scripts/flip_loss.py.  That file places every tensor on 'cuda';
    here it runs on the CPU with torch.Tensor.cuda and the device argument of
    torch.zeros redirected for the duration of the call."""
    import torch

    sys.path.insert(0, os.path.join(reference or reference_dir(), "scripts"))
    pairs = dict(np.load(os.path.join(fixtures.GOLDEN_DIR, "metrics", "pairs.npz")))
    names = [k[:-2] for k in pairs if k.endswith("_a")]
    seq = Sequence(96, 54, 2, seed=21, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=2.0)
    render, _, _, _ = oracle.run_oracle(seq.frame(0), seq.client(0, 2), with_intermediates=False)
    pairs["render_a"], pairs["render_b"] = render, seq.ground_truth(0, 2)
    names.append("render")

    orig_cuda, orig_zeros = torch.Tensor.cuda, torch.zeros
    torch.Tensor.cuda = lambda self, *a, **k: self
    torch.zeros = lambda *a, **k: orig_zeros(*a, **{kk: v for kk, v in k.items() if kk != "device"})
    try:
        from flip_loss import LDRFLIPLoss  # the reference's implementation
        flip = LDRFLIPLoss()
        out = {}
        for n in names:
            a, b = pairs[n + "_a"], pairs[n + "_b"]
            ta = torch.from_numpy(np.ascontiguousarray(np.moveaxis(a[..., :3], -1, 0))).float().unsqueeze(0) / 255.0
            tb = torch.from_numpy(np.ascontiguousarray(np.moveaxis(b[..., :3], -1, 0))).float().unsqueeze(0) / 255.0
            m = flip(ta, tb)  # test = a (render), reference = b (ground truth)
            out[f"{n}_a"], out[f"{n}_b"] = a, b
            out[f"{n}_flip"] = np.float64(m.mean().item())
            if n in ("odd", "render"):
                out[f"{n}_map"] = m.squeeze().numpy().astype(np.float32)
    finally:
        torch.Tensor.cuda, torch.zeros = orig_cuda, orig_zeros
    np.savez_compressed(os.path.join(fixtures.GOLDEN_DIR, "metrics", "flip.npz"), **out)
    print(f"flip: {len(names)} pairs")


def main():
    if sys.argv[1:] == ["metrics"]:
        metrics_cases()
        return
    if sys.argv[1:] == ["flip"]:
        oracle.build()
        flip_cases()
        return
    oracle.build()
    if not oracle.reference_available():
        raise SystemExit("reference renderer not built (needs the reference tree)")
    if sys.argv[1:] == ["timewarp"]:
        timewarp_cases()
        return
    if sys.argv[1:] == ["io"]:
        io_cases()
        return
    io_cases()
    metrics_cases()
    flip_cases()
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
