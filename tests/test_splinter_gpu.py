"""The caller side of the path on the GPU: the dataset loader (include/isti_dataset.h)
and the splinter frame loop (csrc/host/splinter.cpp) against the oracle.

A seeded procedural sequence is written in the reference's dataset format
(files.export_sequence); the expected frames come from oracle/frame_loop.py,
which restates src/main.cu's loop and FrameFileReader's double buffer over
the sequence's own arrays (no decoder involved) and renders every frame with
the C oracle.  The CLI's PNG output must match bit for bit.
"""
import os
import subprocess

import numpy as np
import pytest

from imagebasedspatiotemporalinterpolation_gb300 import _build, files, scene
from oracle import frame_loop as fl

pytestmark = pytest.mark.gpu


def keyframes_of(seq) -> fl.Keyframes:
    """What the dataset folder of export_sequence(seq) holds after loading."""
    cams = []
    n = seq.n_keyframes
    for c in range(1 + len(seq.aux_offsets)):
        proj_raw = files.raw_projection(seq.proj_main if c == 0 else seq.proj_aux)
        lst = []
        for k in range(n):
            kf = seq.keyframe(k, c)
            pose = seq._cam_pose(seq.poses[k], c)
            w2c = scene.view_matrix(pose.eye, pose.yaw, pose.pitch).astype(np.float32)

            def widen(m):
                out = np.zeros(m.shape[:2] + (4,), np.float32)
                out[..., :3] = m.astype(np.float32)
                return out

            lst.append(fl.CamKeyframe(
                color=kf.color, z=files.z_from_unity_depth(files.unity_depth(kf.z)), w2c=w2c, proj_raw=proj_raw,
                motion_fwd=widen(kf.motion_fwd) if k + 1 < n else None,
                motion_bwd=widen(kf.motion_bwd) if k > 0 else None,
                shadow_fwd=kf.shadow_fwd if seq.shadows else None, shadow_bwd=kf.shadow_bwd if seq.shadows else None))
        cams.append(lst)
    prio = 2 + (1 if seq.shadows else 0)
    server = int(round(1.0 / seq.dt))
    return fl.Keyframes(cams, [prio] * len(seq.aux_offsets), server, seq.sfpa * server)


def camera_path_of(seq) -> dict:
    frames = []
    proj = files.raw_projection(seq.proj_main)
    for k in range(seq.n_keyframes - 1):
        for b in range(seq.fpa):
            pose = seq.poses[k].lerp(seq.poses[k + 1], b / seq.fpa)
            frames.append({"w2c": scene.view_matrix(pose.eye, pose.yaw, pose.pitch).astype(np.float32), "proj": proj})
    return {"client_fps": seq.fpa * int(round(1.0 / seq.dt)), "frames": frames}


@pytest.fixture(scope="module")
def aux_dataset(tmp_path_factory, cuda):
    seq = scene.Sequence(96, 54, 3, seed=41, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0, n_spheres=48)
    root = str(tmp_path_factory.mktemp("ds_aux"))
    files.export_sequence(seq, root)
    return seq, root


def run_splinter(args, cwd=None):
    return subprocess.run([_build.splinter_path(), *args], capture_output=True, text=True, timeout=600, cwd=cwd)


def read_frames(out_dir, n):
    return [files.read_png(os.path.join(out_dir, f"{i:04d}.png")) for i in range(n)]


def assert_frames_equal(got, want, first=0):
    assert len(got) == len(want)
    for i in range(first, len(want)):
        diff = (got[i] != want[i]).any(-1)
        assert not diff.any(), f"frame {i}: {int(diff.sum())} pixels differ"


CASES = {
    "mode0": dict(mode=0),
    "mode1": dict(mode=1),
    "mode3": dict(mode=3),
    "mode4": dict(mode=4),
    "no_shadows": dict(mode=0, no_shadows=True),
    "latency2_hold_last": dict(mode=0, latency=2, hold_last=True),
    "holes_black": dict(mode=0, holes_black=True),
}


def cli_flags(o):
    f = ["-m", str(o.get("mode", 0))]
    if o.get("latency"):
        f += ["-l", str(o["latency"])]
    if o.get("hold_last"):
        f.append("-lh")
    if o.get("no_shadows"):
        f.append("-ns")
    if o.get("holes_black"):
        f.append("-hb")
    return f


@pytest.mark.parametrize("case", list(CASES))
def test_splinter_matches_frame_loop_oracle(aux_dataset, tmp_path, case):
    seq, root = aux_dataset
    opts = CASES[case]
    out = str(tmp_path / "out")
    aux = ["left"] if opts.get("mode") == 4 else ["left", "right"]
    r = run_splinter([root, out, "-w", "-r", str(seq.width), str(seq.height), "-c", os.path.join(root, "client"),
                      *cli_flags(opts), "-a", *aux])
    assert r.returncode == 0, r.stdout + r.stderr
    kf = keyframes_of(seq)
    if len(aux) == 1:
        kf = fl.Keyframes(kf.cams[:2], kf.priorities[:1], kf.server_fps, kf.shadow_fps)
    want = fl.splinter(kf, seq.width, seq.height, camera_path=camera_path_of(seq), **opts)
    assert_frames_equal(read_frames(out, len(want)), want)


def test_splinter_latency_extrapolation(aux_dataset, tmp_path):
    """-l 2 without hold-last: frames b < 2 of each interval extrapolate the old
    pair to t = 1, 1.25.  The first interval reads the never-loaded "fwd" slot
    (zero matrices: NaN positions, whose bit patterns differ between CPU and
    GPU), so frames are compared from the second interval on, with -hb making
    each frame independent of the previous one."""
    seq, root = aux_dataset
    out = str(tmp_path / "out")
    r = run_splinter([root, out, "-w", "-r", str(seq.width), str(seq.height), "-c", os.path.join(root, "client"),
                      "-l", "2", "-hb", "-a", "left", "right"])
    assert r.returncode == 0, r.stdout + r.stderr
    want = fl.splinter(keyframes_of(seq), seq.width, seq.height, latency=2, holes_black=True,
                       camera_path=camera_path_of(seq))
    assert_frames_equal(read_frames(out, len(want)), want, first=seq.fpa)


def test_splinter_interpolated_client_view(tmp_path, cuda):
    """Without -c: 1800 client frames at 120 Hz along glm::interpolate of the
    keyframe views (src/main.cu:139-161); after the last keyframe the reader
    keeps swapping the pair, as the reference does."""
    seq = scene.Sequence(64, 36, 3, seed=43, max_speed=2.0, n_spheres=24)
    root = str(tmp_path / "ds")
    files.export_sequence(seq, root, client_dir=None, zip_exr=False)
    out = str(tmp_path / "out")
    r = run_splinter([root, out, "-w", "-r", "64", "36"])
    assert r.returncode == 0, r.stdout + r.stderr
    want = fl.splinter(keyframes_of(seq), 64, 36)
    assert len(want) == 1800
    assert_frames_equal(read_frames(out, 1800), want)


def test_splinter_errors(aux_dataset, tmp_path):
    seq, root = aux_dataset
    r = run_splinter([root, str(tmp_path / "o")])  # default -r 2560 1440 != 96x54 keyframes
    assert r.returncode == 1 and "Error" in r.stdout
    r = run_splinter([root, str(tmp_path / "o"), "-r", "96", "54", "-a", "missing_cam"])
    assert r.returncode == 1 and "cam.json" in r.stdout


def test_dataset_loader_buffers(aux_dataset):
    """isti_dataset: device buffers and matrices after open and each read_next."""
    import torch
    from imagebasedspatiotemporalinterpolation_gb300 import native

    seq, root = aux_dataset
    kf = keyframes_of(seq)
    ds = files.Dataset(root, ["left", "right"])
    ref = fl.Reader(kf)

    def dev(ptr, shape, dtype):
        from imagebasedspatiotemporalinterpolation_gb300.renderer import _CudaArray
        typestr = {np.uint8: "|u1", np.float32: "<f4"}[dtype]
        torch.cuda.synchronize()
        return torch.as_tensor(_CudaArray(int(ptr), tuple(shape), typestr), device="cuda").cpu().numpy()

    def check_pair():
        fd = ds.frame()
        want = ref.frame()
        pairs = [(fd.fwd, want.fwd), (fd.bwd, want.bwd)]
        for i in range(fd.num_aux):
            pairs += [(fd.aux_curr[i], want.aux_curr[i]), (fd.aux_next[i], want.aux_next[i])]
        for got, w in pairs:
            h, wd = w.z.shape
            assert (dev(got.color, (h, wd, 4), np.uint8) == w.color).all()
            assert (dev(got.z, (h, wd), np.float32).view(np.uint32) == w.z.view(np.uint32)).all()
            m = w.motion_f32x4()
            assert (got.motion is None) == (m is None)
            if m is not None:
                assert got.motion_format == native.MOTION_F32X4
                assert (dev(got.motion, (h, wd, 4), np.float32) == m).all()
            assert (got.shadow_color_a is None) == (w.shadow_a is None)
            if w.shadow_a is not None:
                for p, a in ((got.shadow_color_a, w.shadow_a), (got.shadow_info, w.shadow_info)):
                    assert (dev(p, (h, wd, 4), np.uint8) == a).all()
            got_vp = np.array(list(got.viewproj), np.float32).reshape(4, 4).T
            assert (got_vp.view(np.uint32) == w.viewproj.view(np.uint32)).all()

    check_pair()
    assert ds.keyframe == 0
    for step in range(4):  # two real reads, then swaps of an exhausted sequence
        advanced = ds.read_next()
        assert advanced == ref.read_next() == (step < 2)
        check_pair()
    info = ds.camera(-1)
    assert (info["width"], info["height"], info["server_fps"], info["n_frames"]) == (96, 54, 30, 3)
    ds.close()


def test_rgb8_to_rgba8_upload_format(cuda):
    """isti_rgb8_to_rgba8: packed RGB8 -> RGBA8 with alpha 255, on the vector path (aligned
    buffers, 4 pixels per thread) and the byte path (unaligned), any pixel count."""
    import torch

    from imagebasedspatiotemporalinterpolation_gb300 import native
    from imagebasedspatiotemporalinterpolation_gb300.renderer import rgb8_to_rgba8

    rng = np.random.default_rng(5)
    lib = native.load()
    for n in (0, 1, 3, 4, 5, 7, 1023, 1920 * 1080 + 3):
        rgb = rng.integers(0, 256, (n, 3), dtype=np.uint8)
        want = np.concatenate([rgb, np.full((n, 1), 255, np.uint8)], 1)
        for src_off, dst_off in ((0, 0), (1, 0), (0, 1), (3, 2)):
            src_buf = torch.zeros(3 * n + 16, dtype=torch.uint8, device="cuda")
            dst_buf = torch.zeros(4 * n + 64, dtype=torch.uint8, device="cuda")
            src = src_buf[src_off:src_off + 3 * n]
            src.copy_(torch.from_numpy(rgb.reshape(-1)))
            dst = dst_buf[4 * dst_off:4 * dst_off + 4 * n]
            native.check(lib.isti_rgb8_to_rgba8(dst.data_ptr(), src.data_ptr(), n, None))
            torch.cuda.synchronize()
            assert np.array_equal(dst.cpu().numpy().reshape(n, 4), want), (n, src_off, dst_off)
            assert not dst_buf[:4 * dst_off].any() and not dst_buf[4 * dst_off + 4 * n:].any()  # nothing outside
    img = torch.from_numpy(rng.integers(0, 256, (37, 53, 3), dtype=np.uint8)).cuda()
    out = torch.empty((37, 53, 4), dtype=torch.uint8, device="cuda")
    rgb8_to_rgba8(out, img)
    assert torch.equal(out[..., :3], img) and bool((out[..., 3] == 255).all())
    buf = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    with pytest.raises(native.IstiError):   # overlapping buffers
        native.check(lib.isti_rgb8_to_rgba8(buf.data_ptr(), buf.data_ptr() + 8, 100, None))
    with pytest.raises(native.IstiError):   # destination not 4-byte aligned
        native.check(lib.isti_rgb8_to_rgba8(buf.data_ptr() + 2, buf.data_ptr() + 2048, 10, None))
