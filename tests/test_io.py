"""Dataset-format codecs, cam.json parsing, the frame loop's matrix steps and
the splinter CLI's argument handling (CPU only: no kernel is launched).

Pinned against the reference's own image libraries: tests/golden/io holds
PNG/EXR files and the decodes of stb_image / tinyexr (oracle/ref_io.py, built
from the reference tree by tests/golden/make_golden.py io); where the reference
tree is present the libraries are also compared live on fresh random files.
"""
import json
import os
import subprocess
import zlib

import numpy as np
import pytest

from imagebasedspatiotemporalinterpolation_gb300 import _build, files, native, scene
from oracle import frame_loop as fl
from oracle import ref_io
from tests.golden import png_writer

IO_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io")


def _expected():
    with np.load(os.path.join(IO_DIR, "expected.npz")) as z:
        return {k: z[k] for k in z.files}


def _bits(a):
    return a.view(np.uint32) if a.dtype == np.float32 else a


@pytest.mark.parametrize("kind", ["png", "exr"])
def test_codec_fixtures_match_reference_decoders(built, kind):
    exp = _expected()
    names = sorted(n for n in exp if n.endswith("." + kind))
    assert len(names) > 20
    for name in names:
        want = exp[name]
        path = os.path.join(IO_DIR, name)
        read = files.read_png if kind == "png" else files.read_exr
        if want.dtype.kind == "U":  # the reference rejects the file
            with pytest.raises(native.IstiError):
                read(path)
            continue
        got = read(path)
        assert got.shape == want.shape, name
        assert (_bits(got) == _bits(want)).all(), name


@pytest.mark.skipif(not ref_io.available(), reason="reference image libraries not built (no reference tree)")
def test_codecs_against_live_reference(built, tmp_path):
    rng = np.random.default_rng(7)
    for i, (h, w, c) in enumerate([(1, 1, 4), (5, 3, 3), (64, 37, 4), (120, 200, 4)]):
        img = rng.integers(0, 256, (h, w, c), dtype=np.uint8)
        img[h // 2:] = img[h // 2:, :1]
        p = str(tmp_path / f"e{i}.png")
        files.write_png(p, img)
        want = img if c == 4 else np.concatenate([img, np.full((h, w, 1), 255, np.uint8)], -1)
        assert (ref_io.png_load(p) == want).all() and (files.read_png(p) == want).all()
    for i, color in enumerate((0, 2, 3, 4, 6)):
        depth = 8 if color != 0 else 4
        ch = png_writer.CHANNELS[color]
        s = rng.integers(0, 1 << depth, (9, 14, ch))
        pal = rng.integers(0, 256, 3 * 256, dtype=np.uint8).tobytes() if color == 3 else None
        p = str(tmp_path / f"v{i}.png")
        with open(p, "wb") as f:
            f.write(png_writer.make_png(s, depth, color, palette=pal, interlace=i % 2))
        assert (files.read_png(p) == ref_io.png_load(p)).all()
    for comp in (0, 1, 2, 3, 4):
        for pt in (1, 2):
            planes = (rng.standard_normal((4, 21, 30)) * 9).astype(np.float32)
            p = str(tmp_path / f"x{comp}{pt}.exr")
            ref_io.exr_save(p, planes, ["A", "B", "G", "R"], pt, comp)
            assert (_bits(files.read_exr(p)) == _bits(ref_io.exr_load(p))).all()
    # PIZ over several 32-line blocks and odd sizes: few distinct words (14-bit wavelet
    # path), smooth ramps, and random bits over the whole 16-bit range (16-bit path)
    yy, xx = np.mgrid[0:77, 0:101].astype(np.float32)
    cases = {"few": rng.integers(0, 5, (4, 77, 101)).astype(np.float32) * 0.25,
             "ramp": np.stack([xx * 0.01 + yy, yy * 0.5 - xx, np.sin(xx * 0.1) * yy, xx * yy]),
             "wide": rng.integers(0, 1 << 32, (4, 77, 101), dtype=np.uint64).astype(np.uint32).view(np.float32)}
    # many chunks (decoded on several threads), every compression
    tall = (rng.standard_normal((4, 300, 61)) * 9).astype(np.float32)
    tall[:, ::5] = 0.25
    for comp in (0, 1, 2, 3, 4):
        for pt in (1, 2):
            p = str(tmp_path / f"tall{comp}{pt}.exr")
            ref_io.exr_save(p, tall, ["A", "B", "G", "R"], pt, comp)
            assert (_bits(files.read_exr(p)) == _bits(ref_io.exr_load(p))).all(), (comp, pt)
    for name, planes in cases.items():
        planes = np.nan_to_num(planes, nan=1.0, posinf=2.0, neginf=-2.0)
        for pt in (1, 2):
            for names in (["A", "B", "G", "R"], ["Y"]):
                p = str(tmp_path / f"piz_{name}{pt}{len(names)}.exr")
                ref_io.exr_save(p, planes[:len(names)], names, pt, 4)
                assert (_bits(files.read_exr(p)) == _bits(ref_io.exr_load(p))).all(), (name, pt, names)
    for ch in (1, 4):
        for zip_c in (False, True):
            img = (rng.standard_normal((19, 33) if ch == 1 else (19, 33, 4)) * 3).astype(np.float32)
            p = str(tmp_path / f"w{ch}{zip_c}.exr")
            files.write_exr(p, img, zip_c)
            assert (_bits(ref_io.exr_load(p)) == _bits(img)).all()


def test_png_encoder_round_trip(built, tmp_path):
    rng = np.random.default_rng(8)
    for c in (3, 4):
        img = rng.integers(0, 256, (37, 41, c), dtype=np.uint8)
        img[10:20] = 7
        data = files.encode_png(img)
        assert data[:8] == b"\x89PNG\r\n\x1a\n"
        got = files.decode_png(data)
        assert (got[..., :c] == img).all() and (got[..., 3] == (img[..., 3] if c == 4 else 255)).all()


def test_exr_encoder_round_trip(built, tmp_path):
    img = np.random.default_rng(9).standard_normal((23, 29, 4)).astype(np.float32)
    img[0, 0] = [np.inf, -np.inf, np.nan, -0.0]
    for zip_c in (False, True):
        p = str(tmp_path / f"r{zip_c}.exr")
        files.write_exr(p, img, zip_c)
        assert (_bits(files.read_exr(p)) == _bits(img)).all()
        files.write_exr(p, img[..., 0], zip_c)
        assert (_bits(files.read_exr(p)) == _bits(img[..., 0])).all()


def test_exr_many_chunks_decode_in_parallel(built, tmp_path):
    """Images with many chunks are decoded on several threads: same bits as written, and a
    damaged chunk still fails cleanly."""
    rng = np.random.default_rng(12)
    img = (rng.standard_normal((701, 257, 4)) * 100).astype(np.float32)
    img[::7] = 0.5  # some compressible rows
    for zip_c in (False, True):  # 701 one-line chunks, 44 sixteen-line chunks
        p = str(tmp_path / f"big{zip_c}.exr")
        files.write_exr(p, img, zip_c)
        assert (_bits(files.read_exr(p)) == _bits(img)).all()
    data = bytearray(open(str(tmp_path / "bigTrue.exr"), "rb").read())
    for k in range(len(data) // 3, len(data) // 3 + 64):  # garble the middle of the chunk data
        data[k] ^= 0x5a
    with pytest.raises(native.IstiError):
        files.decode_exr(bytes(data))


def test_zlib_streams(built):
    rng = np.random.default_rng(10)
    data = rng.integers(0, 6, 70000, dtype=np.uint8).tobytes() + bytes(3000) + rng.bytes(5000)
    for level in range(10):
        assert files.zlib_decompress(zlib.compress(data, level)) == data
    assert files.zlib_decompress(zlib.compress(b"", 9)) == b""
    good = bytearray(zlib.compress(data, 6))
    bad = bytes(good[:-1]) + bytes([good[-1] ^ 1])  # checksum
    with pytest.raises(native.IstiError):
        files.zlib_decompress(bad)
    with pytest.raises(native.IstiError):
        files.zlib_decompress(bytes(good[: len(good) // 2]))  # truncated
    with pytest.raises(native.IstiError):
        files.zlib_decompress(b"\x78\x9c\xff\xff\xff\xff")  # invalid block type


def test_corrupt_images_fail_cleanly(built, tmp_path):
    rng = np.random.default_rng(11)
    png = files.encode_png(rng.integers(0, 256, (16, 16, 4), dtype=np.uint8))
    for bad in (png[:20], png[:-30], b"\x89PNG\r\n\x1a\n" + rng.bytes(100), rng.bytes(64), b""):
        with pytest.raises(native.IstiError):
            files.decode_png(bad) if bad else files.read_png(str(tmp_path / "missing.png"))
    exr_path = str(tmp_path / "a.exr")
    files.write_exr(exr_path, np.ones((8, 8), np.float32))
    raw = open(exr_path, "rb").read()
    for bad in (raw[:30], raw[:-10], b"\x76\x2f\x31\x01" + rng.bytes(60)):
        with pytest.raises(native.IstiError):
            files.decode_exr(bad)


def _cam_doc(frames, **kw):
    doc = {"resolution": {"x": 64, "y": 36}, "frames": frames}
    doc.update(kw)
    return doc


def _mat_json(m):
    return {f"e{r}{c}": m[r][c] for r in range(4) for c in range(4)}


def test_camera_path_parsing(built, tmp_path):
    """FrameFileReader::initCamInfo (src/file_reader.cu:78-107): e<row><col>
    matrices, integer and real literals, defaults 60/10/60, priority."""
    m = [[1, 0, 0, 0.5], [0, -1, 0, 1e-3], [0, 0, 1, -2.25], [0, 0, 0, 1]]
    p = [[0.1 * (r + 1) + c for c in range(4)] for r in range(4)]
    d = tmp_path / "cam"
    d.mkdir()
    (d / "cam.json").write_text(json.dumps(_cam_doc([{"idx": 7, "w2c": _mat_json(m), "proj": _mat_json(p)},
                                                     {"idx": 8, "w2c": _mat_json(p), "proj": _mat_json(m)}],
                                                    shadowGradients=False)))
    info = files.read_camera_path(str(d))
    assert (info["width"], info["height"]) == (64, 36)
    assert (info["client_fps"], info["server_fps"], info["shadow_fps"]) == (60, 10, 60)
    assert info["priority"] == 2  # objectMotion (default true) * 2 + shadowGradients
    assert [f["idx"] for f in info["frames"]] == [7, 8]
    assert (info["frames"][0]["w2c"] == np.array(m, np.float32)).all()
    assert (info["frames"][0]["proj"] == np.array(p, np.float32)).all()
    (d / "cam.json").write_text(json.dumps(_cam_doc([], clientFps=120)))
    with pytest.raises(native.IstiError, match="Could not load any frames"):
        files.read_camera_path(str(d))
    (d / "cam.json").write_text('{"frames": [{"idx": 1, "w2c": {"e00": 1}}], "resolution": {"x": 2, "y": 2}}')
    with pytest.raises(native.IstiError, match="missing key"):
        files.read_camera_path(str(d))
    (d / "cam.json").write_text('{"frames": [')
    with pytest.raises(native.IstiError):
        files.read_camera_path(str(d))
    with pytest.raises(native.IstiError, match="Failed to open camera file"):
        files.read_camera_path(str(tmp_path / "nowhere"))


def _prod(fn, *ms, t=None):
    import ctypes as C
    lib = native.load()
    out = native.Mat16()
    args = [native.mat16(m) for m in ms]
    if t is None:
        getattr(lib, fn)(*args, out)
    else:
        getattr(lib, fn)(*args, C.c_float(t), out)
    return np.array(list(out), np.float32).reshape(4, 4).T


def test_frame_loop_matrices_match_oracle(built):
    """mat4 product, inverse, glm::interpolate and normalizeProjMat of the host
    loop (csrc/host/isti_mat4.hpp) against the oracle's C restatement, bit for bit."""
    rng = np.random.default_rng(12)
    for _ in range(300):
        a = rng.standard_normal((4, 4)).astype(np.float32)
        b = rng.standard_normal((4, 4)).astype(np.float32)
        assert (_prod("isti_mat4_mul", a, b).view(np.uint32) == fl.mat_mul(a, b).view(np.uint32)).all()
        assert (_prod("isti_mat4_inverse", a).view(np.uint32) == fl.mat_inverse(a).view(np.uint32)).all()
        assert (files.normalize_proj(a).view(np.uint32) == fl.normalize_proj(a).view(np.uint32)).all()
    for i in range(140):
        yaw, pitch = rng.uniform(-3, 3), rng.uniform(-1, 1)
        eye = rng.standard_normal(3)
        dyaw = [0.0, 1e-6, 1e-3, 0.02, 0.5, 3.0, np.pi][i % 7]
        m1 = scene.view_matrix(eye, yaw, pitch).astype(np.float32)
        m2 = scene.view_matrix(eye + rng.standard_normal(3) * 0.05, yaw + dyaw, pitch).astype(np.float32)
        t = float(np.float32(rng.uniform(0.0, 1.75)))
        got = _prod("isti_mat4_interpolate", m1, m2, t=t)
        assert (got.view(np.uint32) == fl.mat_interpolate(m1, m2, t).view(np.uint32)).all()
    # glm::interpolate end points and inverse accuracy
    m1 = scene.view_matrix(np.zeros(3), 0.1, 0.05).astype(np.float32)
    m2 = scene.view_matrix(np.full(3, 0.05), 0.12, 0.04).astype(np.float32)
    assert np.abs(_prod("isti_mat4_interpolate", m1, m2, t=0.0) - m1).max() < 1e-6
    assert np.abs(_prod("isti_mat4_interpolate", m1, m2, t=1.0) - m2).max() < 1e-5
    vp = (scene.perspective(90, 16 / 9, 0.1, 100) @ m1).astype(np.float32)
    assert np.abs(_prod("isti_mat4_inverse", vp) @ vp - np.eye(4)).max() < 1e-5


def test_normalize_proj_recovers_gl_projection(built):
    gl = scene.perspective(90.0, 16 / 9, 0.1, 100.0)
    back = files.normalize_proj(files.raw_projection(gl))
    assert np.abs(back - gl).max() < 1e-5


def _splinter(*args):
    return subprocess.run([_build.splinter_path(), *args], capture_output=True, text=True, timeout=60)


def test_splinter_cli_arguments(built, tmp_path):
    """src/main.cu:66-106: the same flags; parse errors print the usage and exit 1."""
    r = _splinter("-h")
    assert r.returncode == 0
    for flag in ("--camera-path", "--write-images", "--resolution", "--aux-dirs", "--latency", "--mode",
                 "--latency-hold-last", "--no-shadows", "--holes-black"):
        assert flag in r.stdout
    for args in ((), ("only_input",), ("a", "b", "-m", "5"), ("a", "b", "-r", "10"), ("a", "b", "-a"),
                 ("a", "b", "-l", "x"), ("a", "b", "--bogus")):
        r = _splinter(*args)
        assert r.returncode == 1 and "Argument parsing failed" in r.stdout, args
    r = _splinter(str(tmp_path / "missing"), str(tmp_path / "out"))
    assert r.returncode == 1 and "Input directory invalid" in r.stdout
