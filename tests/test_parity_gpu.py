"""CUDA path (libisti.so through the C ABI) against the reference and the oracle.

Bar: bit-exact.  The output image, every 64-bit splat key and every flow-field
float must equal the reference renderer's (golden fixtures) and the C oracle's
(live, seeded scenes at the benchmark sizes).  The parity tolerance (colour
within 1/255 per channel, >= 60 dB PSNR) is implied and asserted as well.
"""
import numpy as np
import pytest

import oracle
from imagebasedspatiotemporalinterpolation_gb300 import native
from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer
from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence
from tests.flowcheck import assert_client_flow_equal
from tests.golden import fixtures

pytestmark = pytest.mark.gpu

TOL_PER_CHANNEL = 1      # 1/255 per channel (the parity bound; the kernels are bit-exact)
TOL_PSNR_DB = 60.0


def psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


def render_gpu(frame, client, prev, motion_format="f16x3", renderer=None):
    import torch
    dev = DeviceFrame.from_host(frame, motion_format=motion_format)
    out = torch.from_numpy(np.ascontiguousarray(prev)).cuda()
    r = renderer or Renderer()
    r.render(out, client, dev)
    torch.cuda.synchronize()
    assert r.device_status() == 0
    nv = len(dev.views())
    bufs = [r.view_buffers(k) for k in range(nv)]
    deps = [r.view_depth(k) for k in range(nv)]
    npy = lambda t, view=None: None if t is None else (t.cpu().numpy().view(view) if view else t.cpu().numpy())
    cams = [None if b[1] is None else client_flow(b[1], d[0], d[1]) for b, d in zip(bufs, deps)]
    res = (out.cpu().numpy(), [npy(b[0], np.uint64) for b in bufs], cams, [npy(b[2]) for b in bufs],
           [v.z.cpu().numpy() for v in dev.views()])
    if renderer is None:
        r.close()
    return res


def client_flow(xy, depth, vis):
    """The renderer's client-flow parts as numpy: (x, y) (H, W, 2), depth (H, W), visible (H, W)."""
    return xy.cpu().numpy(), depth.cpu().numpy(), vis.cpu().numpy()


def assert_bit_exact(got, exp_out, exp_splat, exp_cam=None, exp_full=None):
    out, splats, cams, fulls, zs = got
    diff = np.abs(out.astype(np.int32) - exp_out.astype(np.int32))
    assert diff.max() <= TOL_PER_CHANNEL and psnr(out, exp_out) >= TOL_PSNR_DB
    assert np.array_equal(out, exp_out), f"{int((out != exp_out).any(-1).sum())} output pixels differ"
    for k, (a, b) in enumerate(zip(splats, exp_splat)):
        assert np.array_equal(a, b), f"view {k}: {int((a != b).sum())} splat keys differ"
    if exp_cam is not None:
        for k, (a, b) in enumerate(zip(cams, exp_cam)):
            if b is not None:
                assert_client_flow_equal(k, a, b, zs[k])
    if exp_full is not None:
        for k, (a, b) in enumerate(zip(fulls, exp_full)):
            if b is not None:
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"view {k}: full_ff differs"


@pytest.mark.parametrize("motion_format", ["f16x3", "f32x4"])
@pytest.mark.parametrize("path", fixtures.cases(), ids=lambda p: p.split("/")[-1][:-4])
def test_golden_bit_exact(cuda, path, motion_format):
    frame, client, prev, exp = fixtures.load(path)
    got = render_gpu(frame, client, prev, motion_format)
    if client.mode == native.MODE_TIMEWARP:  # no splat intermediates in this mode
        assert np.array_equal(got[0], exp["out"]), f"{int((got[0] != exp['out']).any(-1).sum())} output pixels differ"
        return
    assert_bit_exact(got, exp["out"], exp["splat"], exp["cam_ff"], exp["full_ff"])


@pytest.mark.parametrize("aux", [(), (-0.3, 0.3)])
def test_timewarp_matches_oracle_1080p(cuda, aux):
    """Mode 4 (planar timewarp at the forward keyframe's mean depth, src/renderer.cu:467-522)."""
    import torch
    seq = Sequence(1920, 1080, 2, seed=707, aux_offsets=aux)
    frame = seq.frame(0)
    dev = DeviceFrame.from_host(frame)
    r = Renderer()
    for b in (1, 3):
        client = seq.client(0, b, mode=native.MODE_TIMEWARP)
        prev = np.full((1080, 1920, 4), 11, np.uint8)
        out = torch.from_numpy(prev.copy()).cuda()
        r.render(out, client, dev)
        exp = oracle.run_oracle(frame, client, prev, with_intermediates=False)[0]
        assert np.array_equal(out.cpu().numpy(), exp)
    r.close()


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
@pytest.mark.parametrize("b", [1, 2, 3])
def test_oracle_parity_640x360_main_only(cuda, mode, b):
    """Plain method at 640x360, main camera only, shadows off."""
    seq = Sequence(640, 360, 2, seed=101)
    frame, client = seq.frame(0), seq.client(0, b, mode=mode)
    prev = np.zeros((360, 640, 4), np.uint8)
    exp = oracle.run_oracle(frame, client, prev)
    assert_bit_exact(render_gpu(frame, client, prev), *exp)


@pytest.mark.parametrize("b", [1, 2, 3])
def test_oracle_parity_1080p_aux_shadows(cuda, b):
    """1920x1080, left/right aux cameras at +-0.3 m (6 source views), soft shadows."""
    seq = Sequence(1920, 1080, 2, seed=202, aux_offsets=(-0.3, 0.3), shadows=True)
    frame, client = seq.frame(0), seq.client(0, b)
    prev = np.zeros((1080, 1920, 4), np.uint8)
    exp = oracle.run_oracle(frame, client, prev)
    assert_bit_exact(render_gpu(frame, client, prev), *exp)


def test_oracle_parity_fast_motion_shadows_modes(cuda):
    seq = Sequence(480, 270, 2, seed=303, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=4.0)
    frame = seq.frame(0)
    for mode in (0, 1, 3):
        for alpha in (0.0, 0.25, 0.6, 1.0, 1.25):
            client = seq.client(0, 0, mode=mode, alpha=alpha)
            prev = np.full((270, 480, 4), 9, np.uint8)
            exp = oracle.run_oracle(frame, client, prev)
            assert_bit_exact(render_gpu(frame, client, prev), *exp)


def test_oracle_parity_odd_sizes_and_half_res_aux(cuda):
    for (w, h, aux_size) in ((333, 197, None), (250, 140, (125, 70)), (31, 17, None)):
        seq = Sequence(w, h, 2, seed=w, aux_offsets=(0.3,), aux_size=aux_size, shadows=True, max_speed=3.0)
        frame, client = seq.frame(0), seq.client(0, 1)
        prev = np.full((h, w, 4), 200, np.uint8)
        exp = oracle.run_oracle(frame, client, prev)
        assert_bit_exact(render_gpu(frame, client, prev), *exp)


@pytest.mark.parametrize("mode", [0, 1, 3])
def test_row_pair_blocks_partial_last_block(cuda, mode):
    """Single frames of 6 views run 3 row pairs per block (4 views: 2): heights that leave a
    partial last block, full- and half-resolution aux cameras."""
    for (w, h, aux_size) in ((250, 139, None), (250, 140, (125, 70)), (96, 7, None), (130, 4, (65, 2))):
        seq = Sequence(w, h, 2, seed=w + h + mode, aux_offsets=(-0.3, 0.3), aux_size=aux_size, shadows=True,
                       max_speed=3.0, n_spheres=40)
        frame, client = seq.frame(0), seq.client(0, 1, mode=mode)
        prev = np.full((h, w, 4), 31, np.uint8)
        assert_bit_exact(render_gpu(frame, client, prev), *oracle.run_oracle(frame, client, prev))
    seq = Sequence(161, 43, 2, seed=5, aux_offsets=(0.3,), shadows=True, max_speed=3.0)  # 4 views
    frame, client = seq.frame(0), seq.client(0, 2, mode=mode)
    prev = np.full((43, 161, 4), 3, np.uint8)
    assert_bit_exact(render_gpu(frame, client, prev), *oracle.run_oracle(frame, client, prev))


def test_repeated_runs_bit_identical(cuda):
    """atomicMin is order-independent: 10 renders give identical keys and images."""
    seq = Sequence(640, 360, 2, seed=404, aux_offsets=(-0.3, 0.3), shadows=True)
    frame, client = seq.frame(0), seq.client(0, 2)
    prev = np.zeros((360, 640, 4), np.uint8)
    r = Renderer()
    first = render_gpu(frame, client, prev, renderer=r)
    for _ in range(9):
        again = render_gpu(frame, client, prev, renderer=r)
        assert np.array_equal(first[0], again[0])
        assert all(np.array_equal(a, b) for a, b in zip(first[1], again[1]))
    r.close()


def test_one_renderer_across_shapes_and_modes(cuda):
    """One renderer, calls whose view sizes, aux cameras and modes change from call to call
    (the arena is reused or regrown, timewarp uses it differently): every call matches the
    oracle, keys included."""
    import torch
    seq_a = Sequence(320, 180, 2, seed=4101, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0)
    seq_b = Sequence(320, 180, 2, seed=4102, aux_offsets=(0.3,), aux_size=(160, 90), shadows=True, max_speed=3.0)
    seq_c = Sequence(200, 120, 2, seed=4103)
    frames = {"a": seq_a.frame(0), "b": seq_b.frame(0), "c": seq_c.frame(0)}
    seqs = {"a": seq_a, "b": seq_b, "c": seq_c}
    devs = {k: DeviceFrame.from_host(f) for k, f in frames.items()}
    r = Renderer()
    plan = [("c", 1, 0), ("a", 2, 0), ("a", 3, 1), ("b", 1, 0), ("b", 2, 3), ("a", 2, 0), ("a", 2, 4), ("a", 1, 0),
            ("a", 3, 2), ("c", 2, 0), ("c", 1, 4), ("a", 0, 0)]
    for i, (name, b, mode) in enumerate(plan):
        frame, client = frames[name], seqs[name].client(0, b, mode=mode)
        h, w = client.height, client.width
        prev = np.full((h, w, 4), i, np.uint8)
        out = torch.from_numpy(prev.copy()).cuda()
        r.render(out, client, devs[name])
        torch.cuda.synchronize()
        assert r.device_status() == 0
        exp = oracle.run_oracle(frame, client, prev, with_intermediates=mode != native.MODE_TIMEWARP)
        assert np.array_equal(out.cpu().numpy(), exp[0]), f"call {i} ({name}, mode {mode}) differs"
        if mode != native.MODE_TIMEWARP:
            for v in range(len(frame.views())):
                keys = r.view_buffers(v)[0].cpu().numpy().view(np.uint64)
                assert np.array_equal(keys, exp[1][v]), f"call {i} view {v} keys differ"
    r.close()


def test_temporal_hole_filling_keeps_previous_output(cuda):
    seq = Sequence(320, 180, 2, seed=505)
    frame, client = seq.frame(0), seq.client(0, 2)
    prev = np.random.default_rng(0).integers(0, 256, (180, 320, 4), dtype=np.uint8)
    out = render_gpu(frame, client, prev)[0]
    exp = oracle.run_oracle(frame, client, prev)[0]
    assert np.array_equal(out, exp)
    kept = (out == prev).all(-1)
    assert kept.any() and (~kept).any()


def test_render_on_side_stream(cuda):
    import torch
    seq = Sequence(320, 180, 2, seed=606, aux_offsets=(0.3,), shadows=True)
    frame, client = seq.frame(0), seq.client(0, 1)
    dev = DeviceFrame.from_host(frame)
    s = torch.cuda.Stream()
    out = torch.zeros((180, 320, 4), dtype=torch.uint8, device="cuda")
    r = Renderer()
    with torch.cuda.stream(s):
        r.render(out, client, dev, stream=s)
    s.synchronize()
    exp = oracle.run_oracle(frame, client, np.zeros((180, 320, 4), np.uint8), with_intermediates=False)[0]
    assert np.array_equal(out.cpu().numpy(), exp)
    r.close()


def test_invalid_arguments_are_rejected(cuda):
    import torch
    seq = Sequence(64, 36, 2, seed=7, aux_offsets=(0.3,))
    frame = seq.frame(0)
    dev = DeviceFrame.from_host(frame)
    out = torch.zeros((36, 64, 4), dtype=torch.uint8, device="cuda")
    r = Renderer()
    bad = seq.client(0, 1)
    bad.shadow_frames_per_anchor = 17
    with pytest.raises(native.IstiError) as e:
        r.render(out, bad, dev)
    assert e.value.status == native.ISTI_ERR_INVALID_ARG
    bad = seq.client(0, 1, mode=9)
    with pytest.raises(native.IstiError):
        r.render(out, bad, dev)
    # aux camera larger than the render resolution (the reference divides by zero, src/renderer.cu:425)
    big = Sequence(64, 36, 2, seed=7, aux_offsets=(0.3,), aux_size=(96, 54))
    with pytest.raises(native.IstiError):
        r.render(out, big.client(0, 1), DeviceFrame.from_host(big.frame(0)))
    r.close()


@pytest.mark.parametrize("mode", [0, 1, 3, 4])
def test_batch_equals_sequential_renders(cuda, mode):
    """isti_render_batch == isti_render frame by frame (chained: one persistent buffer)."""
    import torch
    seq = Sequence(480, 270, 2, seed=909 + mode, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0)
    frame = DeviceFrame.from_host(seq.frame(0))
    clients = [seq.client(0, b, mode=mode) for b in (0, 1, 2, 3)] + [seq.client(0, 0, mode=mode, alpha=a) for a in (0.6, 1.0)]
    g = torch.Generator().manual_seed(mode)
    prev = torch.randint(0, 256, (270, 480, 4), dtype=torch.uint8, generator=g).cuda()
    nv = len(frame.views())
    r = Renderer()
    buf, snaps, keys = prev.clone(), [], []
    for c in clients:
        r.render(buf, c, frame)
        snaps.append(buf.clone())
        keys.append([r.view_buffers(v)[0] for v in range(nv)])
    outs = [prev.clone()] + [torch.zeros_like(prev) for _ in clients[1:]]
    r.render_batch(outs, clients, frame, chain=True)
    torch.cuda.synchronize()
    for k in range(len(clients)):
        assert torch.equal(outs[k], snaps[k]), f"chained frame {k} differs"
        if mode == native.MODE_TIMEWARP:
            continue  # no splat keys in this mode
        for v in range(nv):
            assert torch.equal(r.view_buffers(k * nv + v)[0], keys[k][v]), f"frame {k} view {v} keys differ"
    outs = [prev.clone() for _ in clients]
    r.render_batch(outs, clients, frame, chain=False)
    for k, c in enumerate(clients):
        single = prev.clone()
        r.render(single, c, frame)
        assert torch.equal(outs[k], single), f"unchained frame {k} differs"
    r.close()


def test_batch_limits(cuda):
    import torch
    seq = Sequence(64, 36, 2, seed=11)
    frame = DeviceFrame.from_host(seq.frame(0))
    r = Renderer()
    bufs = [torch.zeros((36, 64, 4), dtype=torch.uint8, device="cuda") for _ in range(9)]
    clients = [seq.client(0, b % 4, alpha=(b + 1) / 9) for b in range(9)]
    # the largest batch equals frame-by-frame renders, outputs and splat keys
    singles, keys = [], []
    for c in clients[:8]:
        single = torch.zeros((36, 64, 4), dtype=torch.uint8, device="cuda")
        r.render(single, c, frame)
        singles.append(single)
        keys.append(r.view_buffers(0)[0].clone())
    r.render_batch(bufs[:8], clients[:8], frame, chain=False)
    torch.cuda.synchronize()
    for k in range(8):
        assert torch.equal(bufs[k], singles[k]), f"frame {k} of 8 differs"
        assert torch.equal(r.view_buffers(k * len(frame.views()))[0], keys[k]), f"frame {k} of 8: keys differ"
    with pytest.raises(ValueError):
        r.render_batch(bufs, clients, frame)
    mixed = [seq.client(0, 1), seq.client(0, 2, mode=3)]
    with pytest.raises(native.IstiError):
        r.render_batch(bufs[:2], mixed, frame)
    r.close()


@pytest.mark.parametrize("mode", [0, 1, 3])
@pytest.mark.parametrize("size", [(1, 1), (1, 9), (9, 1), (2, 3), (36, 4), (37, 5), (38, 5), (40, 8), (4097, 3), (65535, 2)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
def test_extreme_shapes_match_oracle(cuda, size, mode):
    """Degenerate and extreme image shapes: single pixels, single rows/columns, exactly the
    key-tile box (36x4, 40x8), widths whose row pitch forbids the TMA tile path (37), the
    16-bit key field's largest width (65535)."""
    w, h = size
    seq = Sequence(w, h, 2, seed=w * 7 + h, n_spheres=24, max_speed=2.0)
    frame, client = seq.frame(0), seq.client(0, 2, mode=mode)
    prev = np.full((h, w, 4), 77, np.uint8)
    assert_bit_exact(render_gpu(frame, client, prev), *oracle.run_oracle(frame, client, prev))


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_nonfinite_inputs_render_without_fault(cuda, mode):
    """NaN / +-inf depth and motion (outside the parity claim: NaN bit patterns differ
    between CPU and GPU) must neither fault nor stop the renderer: every splat key and
    search step stays inside its view."""
    import torch
    seq = Sequence(160, 90, 2, seed=808, aux_offsets=(0.3,), shadows=True)
    frame = seq.frame(0)
    for v in frame.views():
        v.z = v.z.copy()
        v.z[10:20, 10:40] = np.nan
        v.z[30:35, :] = np.inf
        v.z[40:42, 50:90] = -np.inf
        m = v.motion.astype(np.float32)
        m[50:60, 0:30] = np.nan
        m[60:62, :, 0] = np.inf
        v.motion = m.astype(np.float16)
    client = seq.client(0, 2, mode=mode)
    dev = DeviceFrame.from_host(frame)
    out = torch.zeros((90, 160, 4), dtype=torch.uint8, device="cuda")
    r = Renderer()
    for _ in range(2):
        r.render(out, client, dev)
    torch.cuda.synchronize()
    assert r.device_status() == 0
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(160, 90, (-0.3, 0.3), True, 0, 1), (160, 90, (), False, 0, 6), (128, 72, (0.3,), True, 1, 3),
                                  (96, 54, (), False, 3, 2)], ids=["6v-shadows-1f", "2v-6f", "mode1-4v-3f", "mode3-2v-2f"])
def test_autotuned_renders_equal_the_rule_and_the_oracle(cuda, case):
    """With autotuning on, the first render of a shape class also times every candidate
    reprojection launch (register cap x row pairs); that render and the later ones, with
    the chosen launch, equal the fixed-rule renderer and the oracle bit for bit."""
    import torch
    w, h, aux, sh, mode, nf = case
    seq = Sequence(w, h, 2, seed=4100 + w + nf, aux_offsets=aux, shadows=sh, max_speed=2.0)
    frame = seq.frame(0)
    dev = DeviceFrame.from_host(frame)
    clients = [seq.client(0, b % 4, mode=mode, alpha=(b + 1) / (nf + 1)) for b in range(nf)]
    g = torch.Generator().manual_seed(w * nf)
    prev = torch.randint(0, 256, (h, w, 4), dtype=torch.uint8, generator=g).cuda()
    tuned, rule = Renderer(), Renderer()
    tuned.set_autotune(True)
    for rep in range(2):   # the tuning call, then a call with the chosen launch
        a = [prev.clone()] + [torch.zeros_like(prev) for _ in clients[1:]]
        b = [prev.clone()] + [torch.zeros_like(prev) for _ in clients[1:]]
        tuned.render_batch(a, clients, dev, chain=True)
        rule.render_batch(b, clients, dev, chain=True)
        torch.cuda.synchronize()
        for k in range(nf):
            assert torch.equal(a[k], b[k]), f"call {rep}, frame {k}: the tuned launch differs from the rule"
        for v in range(len(dev.views())):
            assert torch.equal(tuned.view_buffers(v)[0], rule.view_buffers(v)[0])
    t = tuned.tuning()
    assert len(t) == 1
    t = t[0]
    assert (t["mode"], t["n_views"], t["n_frames"], t["shadows"], t["width"], t["height"]) == (mode, len(dev.views()), nf, int(sh), w, h)
    assert t["regs"] in ((40, 48) if mode != 1 else (56,)) and 1 <= t["row_pairs"] <= 3
    assert 0 < t["best_ms"] <= t["rule_ms"]
    # the first frame against the oracle
    exp = oracle.run_oracle(frame, clients[0], prev.cpu().numpy(), with_intermediates=False)[0]
    np.testing.assert_array_equal(a[0].cpu().numpy(), exp)
    tuned.close()
    rule.close()


def test_autotuned_unchained_batch_of_eight(cuda):
    """Autotuning on an unchained batch of the largest size (8 frames, 4 views, shadows):
    the tuning call and the next one equal the fixed rule frame by frame."""
    import torch
    seq = Sequence(144, 80, 2, seed=8080, aux_offsets=(0.3,), shadows=True, max_speed=2.0)
    dev = DeviceFrame.from_host(seq.frame(0))
    clients = [seq.client(0, b % 4, alpha=(b + 1) / 9) for b in range(8)]
    g = torch.Generator().manual_seed(88)
    prevs = [torch.randint(0, 256, (80, 144, 4), dtype=torch.uint8, generator=g).cuda() for _ in clients]
    tuned, rule = Renderer(), Renderer()
    tuned.set_autotune(True)
    for rep in range(2):
        a = [p.clone() for p in prevs]
        b = [p.clone() for p in prevs]
        tuned.render_batch(a, clients, dev, chain=False)
        rule.render_batch(b, clients, dev, chain=False)
        torch.cuda.synchronize()
        for k in range(8):
            assert torch.equal(a[k], b[k]), f"call {rep}, frame {k} differs"
    assert len(tuned.tuning()) == 1 and tuned.tuning()[0]["n_frames"] == 8
    tuned.close()
    rule.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(160, 90, (), False, 0, 2, True), (128, 72, (0.3,), True, 0, 3, True),
                                  (96, 54, (), False, 0, 1, True), (160, 90, (-0.3, 0.3), True, 0, 1, False),
                                  (96, 54, (0.3,), False, 1, 2, True)],
                         ids=["2v-2f-chained", "4v-3f-chained-shadows", "2v-1f-chained", "6v-1f", "mode1-4v-2f-chained"])
def test_every_pinned_reprojection_launch_equals_the_rule(cuda, case):
    """Every reprojection launch a renderer can be pinned to (register cap x output row
    pairs x key tiles by TMA or plain loads) renders the rule's frames bit for bit, chained
    batches of several frames included (their blocks keep at most one row per view)."""
    import torch
    w, h, aux, sh, mode, nf, chain = case
    seq = Sequence(w, h, 2, seed=6200 + w + nf, aux_offsets=aux, shadows=sh, max_speed=2.0)
    dev = DeviceFrame.from_host(seq.frame(0))
    clients = [seq.client(0, b % 4, mode=mode, alpha=(b + 1) / (nf + 1)) for b in range(nf)]
    g = torch.Generator().manual_seed(w + 7 * nf)
    prevs = [torch.randint(0, 256, (h, w, 4), dtype=torch.uint8, generator=g).cuda() for _ in clients]
    rule = Renderer()
    want = [p.clone() for p in prevs]
    rule.render_batch(want, clients, dev, chain=chain)
    pinned = Renderer()
    with pytest.raises(native.IstiError):
        pinned.set_reproj_launch(44, 1, 0)
    with pytest.raises(native.IstiError):
        pinned.set_reproj_launch(48, 4, 0)
    for regs in ((56,) if mode == 1 else (40, 48)):
        for rp in (1, 2, 3):
            for plain in (0, 1):
                pinned.set_reproj_launch(regs, rp, plain)
                got = [p.clone() for p in prevs]
                pinned.render_batch(got, clients, dev, chain=chain)
                torch.cuda.synchronize()
                for k in range(nf):
                    assert torch.equal(got[k], want[k]), f"regs {regs}, row pairs {rp}, plain tiles {plain}: frame {k} differs"
    assert pinned.device_status() == 0 and rule.device_status() == 0
    pinned.close()
    rule.close()
