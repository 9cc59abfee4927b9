"""The C oracle against the reference renderer (CPU, no GPU needed).

* golden fixtures: outputs of the reference's own src/renderer.cu, committed
  under tests/golden (generated by tests/golden/make_golden.py);
* live comparison with the reference compiled for the CPU (oracle/_ref),
  where the reference tree is available.
Everything must match bit for bit: output image, 64-bit splat keys, flow fields.
"""
import numpy as np
import pytest

import oracle
from imagebasedspatiotemporalinterpolation_gb300.scene import Sequence
from tests.golden import fixtures


def _assert_same(got, exp_out, exp_splat, exp_cam=None, exp_full=None):
    out, splats, cams, fulls = got
    assert np.array_equal(out, exp_out), f"{int((out != exp_out).any(-1).sum())} output pixels differ"
    for k, (a, b) in enumerate(zip(splats, exp_splat)):
        assert np.array_equal(a, b), f"view {k}: {int((a != b).sum())} splat keys differ"
    for name, got_l, exp_l in (("cam_ff", cams, exp_cam), ("full_ff", fulls, exp_full)):
        if exp_l is None:
            continue
        for k, (a, b) in enumerate(zip(got_l, exp_l)):
            if b is None:
                continue
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"view {k}: {name} differs"


@pytest.mark.parametrize("path", fixtures.cases(), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_matches_golden(built, path):
    frame, client, prev, exp = fixtures.load(path)
    got = oracle.run_oracle(frame, client, prev)
    _assert_same(got, exp["out"], exp["splat"], exp["cam_ff"], exp["full_ff"])


def test_golden_fixtures_present():
    names = [p.split("/")[-1] for p in fixtures.cases()]
    assert len(names) >= 10
    assert any("aux" in n for n in names) and any("mode1" in n for n in names) and any("mode3" in n for n in names)


@pytest.mark.parametrize("nthreads", [1, 3])
def test_oracle_thread_count_invariant(built, nthreads):
    seq = Sequence(200, 120, 2, seed=5, aux_offsets=(0.3,), shadows=True)
    frame, client = seq.frame(0), seq.client(0, 2)
    a = oracle.run_oracle(frame, client, nthreads=0)
    b = oracle.run_oracle(frame, client, nthreads=nthreads)
    _assert_same(b, a[0], a[1], a[2], a[3])


def test_oracle_rejects_bad_arguments(built):
    seq = Sequence(64, 36, 2, seed=3)
    frame, client = seq.frame(0), seq.client(0, 2)
    client.width = 32  # render resolution must equal the keyframes'
    with pytest.raises(ValueError):
        oracle.run_oracle(frame, client)
    client = seq.client(0, 2)
    client.shadow_frames_per_anchor = 17
    with pytest.raises(ValueError):
        oracle.run_oracle(frame, client)


needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference renderer not built here")


@needs_ref
@pytest.mark.parametrize("seed,mode,b,aux,shadows", [
    (21, 0, 1, (), False), (22, 0, 3, (), False), (23, 3, 2, (), False), (24, 1, 2, (), False),
    (25, 2, 1, (-0.3, 0.3), True), (26, 0, 2, (-0.3, 0.3), True), (27, 1, 3, (0.3,), True),
])
def test_oracle_matches_reference_live(built, seed, mode, b, aux, shadows):
    seq = Sequence(256, 144, 2, seed=seed, aux_offsets=aux, shadows=shadows, max_speed=3.0)
    frame, client = seq.frame(0), seq.client(0, b, mode=mode)
    prev = np.full((client.height, client.width, 4), 7, np.uint8)
    ref = oracle.run_reference(frame, client, prev)
    _assert_same(oracle.run_oracle(frame, client, prev), ref[0], ref[1], ref[2], ref[3])


@needs_ref
def test_oracle_matches_reference_alpha_edges(built):
    # t = 0 (forward search enabled), t = 1 (forward skipped, src/renderer.cu:335), t > 1 (latency extrapolation)
    seq = Sequence(160, 90, 2, seed=31, aux_offsets=(0.3,), shadows=True, max_speed=3.0)
    frame = seq.frame(0)
    for alpha in (0.0, 1.0, 1.25):
        client = seq.client(0, 0, alpha=alpha)
        ref = oracle.run_reference(frame, client)
        _assert_same(oracle.run_oracle(frame, client), ref[0], ref[1], ref[2], ref[3])
