"""isti_render_pairs: many keyframe pairs in one persistent launch.

The batched workload of the benchmark list -- 16 keyframe pairs x 3 t values x 2 eyes,
the pairs at 1280x720, 1920x1080 and 2064x2208 in turn, main camera only, no shadows,
mode 0 -- rendered by ONE isti_render_pairs call (a cooperative kernel over a device work
queue of key-initialisation, splat and reprojection units) must equal per-frame
isti_render calls bit for bit, frame by frame; a smaller mixed case checks chained
outputs, aux cameras with soft shadows and mode 1 against isti_render_batch.
"""
import numpy as np
import pytest

from imagebasedspatiotemporalinterpolation_gb300 import native, scene
from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer

pytestmark = pytest.mark.gpu

RES = ((1280, 720), (1920, 1080), (2064, 2208))
EYES = (-0.032, 0.032)


def eye_client(seq, k, b, offset, mode=0):
    t = b / seq.fpa
    pose = seq.poses[k].lerp(seq.poses[k + 1], t)
    eye = pose.eye + scene.right_vector(pose.yaw, pose.pitch) * offset
    vp = seq.proj_main @ scene.view_matrix(eye, pose.yaw, pose.pitch)
    return scene.Client(seq.width, seq.height, float(np.float32(t)), vp.astype(np.float32), np.linalg.inv(vp).astype(np.float32),
                        seq.fpa, seq.sfpa, False, mode)


def test_sixteen_pairs_one_launch_equal_per_frame_calls(cuda):
    import torch
    jobs, per_res = [], {}
    for j, (w, h) in enumerate(RES):
        n = len(range(j, 16, 3))
        per_res[(w, h)] = scene.Sequence(w, h, n + 1, seed=4100 + j)
    counters = {r: 0 for r in RES}
    for i in range(16):
        w, h = RES[i % 3]
        seq = per_res[(w, h)]
        k = counters[(w, h)]
        counters[(w, h)] += 1
        clients = [eye_client(seq, k, b, e) for b in (1, 2, 3) for e in EYES]
        frame = DeviceFrame.from_host(seq.frame(k))
        outs = [torch.full((h, w, 4), 3, dtype=torch.uint8, device="cuda") for _ in clients]
        jobs.append((outs, clients, frame))
    r = Renderer()
    r.render_pairs(jobs)
    torch.cuda.synchronize()
    assert r.device_status() == native.ISTI_OK
    ref = Renderer()
    for i, (outs, clients, frame) in enumerate(jobs):
        for k, (o, c) in enumerate(zip(outs, clients)):
            want = torch.full_like(o, 3)
            ref.render(want, c, frame)
            torch.cuda.synchronize()
            assert torch.equal(o, want), f"pair {i} frame {k}: {int((o != want).any(-1).sum())} pixels differ"
    r.close()
    ref.close()


@pytest.mark.parametrize("units", [(0, 0), (1, 16), (7, 48), (64, 1024)], ids=lambda u: f"rows{u[0]}-kib{u[1]}")
@pytest.mark.parametrize("mode", [0, 1])
def test_mixed_pairs_chained_equal_render_batch(cuda, mode, units):
    import torch
    seqs = [scene.Sequence(320, 180, 3, seed=4200, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=2.0),
            scene.Sequence(400, 240, 3, seed=4201, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=2.0)]
    jobs, wants = [], []
    ref = Renderer()
    for i in range(4):
        seq = seqs[i % 2]
        k = i // 2
        clients = [seq.client(k, b, mode=mode) for b in (1, 2, 3)]
        frame = DeviceFrame.from_host(seq.frame(k))
        prev = torch.full((seq.height, seq.width, 4), 11, dtype=torch.uint8, device="cuda")
        want = [prev.clone() for _ in clients]
        ref.render_batch(want, clients, frame, chain=True)
        jobs.append(([prev.clone() for _ in clients], clients, frame))
        wants.append(want)
    r = Renderer()
    r.set_pair_units(*units)
    r.render_pairs(jobs, chain=True)
    torch.cuda.synchronize()
    assert r.device_status() == native.ISTI_OK
    for i, ((outs, _, _), want) in enumerate(zip(jobs, wants)):
        for k, (a, b) in enumerate(zip(outs, want)):
            assert torch.equal(a, b), f"pair {i} frame {k}: {int((a != b).any(-1).sum())} pixels differ"
    r.close()
    ref.close()


def test_graph_capture_and_uncaptured_calls_alternate(cuda):
    """A captured isti_render_pairs call replays with its own parameters after uncaptured calls
    of the same renderer with other parameters (separate staging buffers)."""
    import torch
    seq = scene.Sequence(320, 180, 4, seed=4300)
    jobs_a, jobs_b = [], []
    for k, jobs in ((0, jobs_a), (1, jobs_b)):
        clients = [seq.client(k, b) for b in (1, 2, 3)]
        jobs.append(([torch.zeros((180, 320, 4), dtype=torch.uint8, device="cuda") for _ in clients], clients,
                     DeviceFrame.from_host(seq.frame(k))))
    ref = Renderer()
    want = {}
    for name, jobs in (("a", jobs_a), ("b", jobs_b)):
        outs, clients, frame = jobs[0]
        w = [torch.zeros_like(o) for o in outs]
        ref.render_batch(w, clients, frame, chain=False)
        want[name] = w
    r = Renderer()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        r.render_pairs(jobs_a, stream=stream)          # sizes the arena and both staging buffers
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            r.render_pairs(jobs_a, stream=stream)
    for _ in range(2):
        for o in jobs_a[0][0] + jobs_b[0][0]:
            o.zero_()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            r.render_pairs(jobs_b, stream=stream)      # uncaptured, other parameters
            graph.replay()                             # must still render pair a
        stream.synchronize()
        assert r.device_status() == native.ISTI_OK
        for got, exp in ((jobs_a[0][0], want["a"]), (jobs_b[0][0], want["b"])):
            for a, b in zip(got, exp):
                assert torch.equal(a, b)
    r.close()
    ref.close()


def test_stalled_dependency_wait_times_out_and_the_next_call_renders(cuda):
    """Failure detection of the persistent launch: the reprojection units of one pair wait
    for a splat unit that does not exist (test hook), their bounded waits run out, the call
    reports ISTI_ERR_TIMEOUT instead of hanging, and the next call renders every pair bit for
    bit."""
    import torch
    seq = scene.Sequence(320, 180, 4, seed=4400, aux_offsets=(-0.3, 0.3), shadows=True)
    jobs, wants = [], []
    ref = Renderer()
    for k in range(3):
        clients = [seq.client(k, b) for b in (1, 2, 3)]
        frame = DeviceFrame.from_host(seq.frame(k))
        want = [torch.zeros((180, 320, 4), dtype=torch.uint8, device="cuda") for _ in clients]
        ref.render_batch(want, clients, frame, chain=False)
        jobs.append(([torch.zeros_like(w) for w in want], clients, frame))
        wants.append(want)
    r = Renderer()
    r.test_stall_pair(1, 4096)
    r.render_pairs(jobs)
    torch.cuda.synchronize()
    assert r.device_status() == native.ISTI_ERR_TIMEOUT
    r.test_stall_pair(-1)
    for outs, _, _ in jobs:
        for o in outs:
            o.zero_()
    r.render_pairs(jobs)
    torch.cuda.synchronize()
    assert r.device_status() == native.ISTI_OK
    for (outs, _, _), want in zip(jobs, wants):
        for a, b in zip(outs, want):
            assert torch.equal(a, b)
    r.close()
    ref.close()
