"""Sparse shadow images (isti_unpack_shadows, renderer.pack_shadow_entries).

CPU: the entry format -- one 16-byte entry per pixel whose shadow-info RGB is non-zero:
index (uint32 LE), info RGB, colour A RGB, colour B RGB, zero padding.
GPU: the device expansion equals the dense images wherever the renderer reads them (zero
elsewhere), entries past the image are skipped, and frames rendered from unpacked shadow
images equal the frames rendered from the dense ones, bit for bit."""
import numpy as np
import pytest

from imagebasedspatiotemporalinterpolation_gb300.renderer import SHADOW_ENTRY_BYTES, pack_shadow_entries


def _images(seed, h=6, w=7):
    rng = np.random.default_rng(seed)
    info = np.zeros((h, w, 4), np.uint8)
    mask = rng.random((h, w)) < 0.3
    info[mask, :3] = rng.integers(0, 256, (int(mask.sum()), 3), dtype=np.uint8)
    info[..., 3] = 255
    a = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    b = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    return info, a, b


def test_entry_format():
    info, a, b = _images(1)
    e = pack_shadow_entries(info, a, b)
    nz = np.flatnonzero(info[..., :3].reshape(-1, 3).any(1))
    assert e.shape == (len(nz), SHADOW_ENTRY_BYTES) and e.dtype == np.uint8
    assert np.array_equal(e[:, :4].copy().view("<u4").ravel(), nz)
    assert np.array_equal(e[:, 4:7], info.reshape(-1, 4)[nz, :3])
    assert np.array_equal(e[:, 7:10], a.reshape(-1, 4)[nz, :3])
    assert np.array_equal(e[:, 10:13], b.reshape(-1, 3)[nz])
    assert not e[:, 13:].any()
    assert pack_shadow_entries(np.zeros((3, 3, 3), np.uint8), np.ones((3, 3, 3), np.uint8), np.ones((3, 3, 3), np.uint8)).shape == (0, 16)
    with pytest.raises(ValueError):
        pack_shadow_entries(info, a[:2], b)


@pytest.mark.gpu
def test_unpack_equals_dense_where_read(cuda):
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.renderer import unpack_shadows
    info, a, b = _images(2, 37, 53)
    e = pack_shadow_entries(info, a, b)
    bad = np.zeros((2, SHADOW_ENTRY_BYTES), np.uint8)
    bad[:, :4] = np.array([37 * 53, 0xFFFFFFFF], "<u4").view(np.uint8).reshape(2, 4)   # past the image: skipped
    bad[:, 4:13] = 9
    ent = torch.from_numpy(np.concatenate([e, bad])).cuda()
    imgs = [torch.full((37, 53, 4), 77, dtype=torch.uint8, device="cuda") for _ in range(3)]
    unpack_shadows(*imgs, ent)
    torch.cuda.synchronize()
    got = [x.cpu().numpy() for x in imgs]
    m = info[..., :3].any(-1)
    for g, dense in zip(got, (info, a, np.concatenate([b, np.full(b.shape[:2] + (1,), 255, np.uint8)], -1))):
        assert np.array_equal(g[m, :3], dense[m, :3])
        assert (g[m, 3] == 255).all()
        assert not g[~m].any()


@pytest.mark.gpu
def test_unpack_clearing_the_previous_entries_equals_a_fresh_unpack(cuda):
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.renderer import unpack_shadows
    e1 = torch.from_numpy(pack_shadow_entries(*_images(3, 29, 31))).cuda()
    e2 = torch.from_numpy(pack_shadow_entries(*_images(4, 29, 31))).cuda()
    imgs = [torch.full((29, 31, 4), 77, dtype=torch.uint8, device="cuda") for _ in range(3)]
    unpack_shadows(*imgs, e1)                      # whole images cleared
    unpack_shadows(*imgs, e2, clear_entries=e1)    # only e1's pixels cleared
    fresh = [torch.full((29, 31, 4), 99, dtype=torch.uint8, device="cuda") for _ in range(3)]
    unpack_shadows(*fresh, e2)
    torch.cuda.synchronize()
    for a, b in zip(imgs, fresh):
        assert torch.equal(a, b)


@pytest.mark.gpu
def test_frames_from_unpacked_shadows_equal_dense(cuda):
    import torch
    from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, DeviceView, Renderer, unpack_shadows
    from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence
    seq = Sequence(320, 180, 2, seed=77, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=2.0)
    frame = seq.frame(0)
    dense = DeviceFrame.from_host(frame)
    sparse_views = []
    for v, dv in zip(frame.views(), dense.views()):
        ent = torch.from_numpy(pack_shadow_entries(v.shadow_info, v.shadow_a, v.shadow_b)).cuda()
        imgs = [torch.empty_like(dv.color) for _ in range(3)]
        unpack_shadows(imgs[2], imgs[0], imgs[1], ent)
        sparse_views.append(DeviceView(dv.color, dv.z, dv.motion, imgs[0], imgs[1], imgs[2], dv.viewproj, dv.inv_viewproj))
    sv = sparse_views
    sparse = DeviceFrame(sv[0], sv[1], sv[2::2], sv[3::2], list(dense.aux_priority))
    clients = [seq.client(0, b) for b in (1, 2, 3)]
    r = Renderer()
    prev = torch.full((180, 320, 4), 5, dtype=torch.uint8, device="cuda")
    want = [prev.clone() for _ in clients]
    got = [prev.clone() for _ in clients]
    r.render_batch(want, clients, dense, chain=True)
    r.render_batch(got, clients, sparse, chain=True)
    torch.cuda.synchronize()
    assert r.device_status() == 0
    for k, (x, y) in enumerate(zip(got, want)):
        assert torch.equal(x, y), f"frame {k}: {int((x != y).any(-1).sum())} pixels differ"
    r.close()


def test_cpp_header_packs_like_python(tmp_path):
    """isti::pack_shadow_entries (C++ header) writes the same entries as the Python packer."""
    import os
    import shutil
    import subprocess

    from imagebasedspatiotemporalinterpolation_gb300 import _build
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "shadow_pack_hpp")
    res = subprocess.run([gxx, "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", "-I", _build.INCLUDE,
                          "-I", os.path.join(_build._cuda_home(), "include"),
                          os.path.join(root, "tests", "cpp", "shadow_pack_hpp.cpp"), "-o", exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    info, a, b = _images(5, 41, 23)
    src = tmp_path / "in.bin"
    src.write_bytes(np.array([41 * 23], "<u4").tobytes() + info.tobytes() + a.tobytes() + b.tobytes())
    res = subprocess.run([exe, str(src), str(tmp_path / "out.bin")], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stdout + res.stderr
    want = pack_shadow_entries(info, a, b)
    assert res.stdout.split() == ["ok", str(len(want))]
    assert (tmp_path / "out.bin").read_bytes() == want.tobytes()
