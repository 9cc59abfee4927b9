"""The serving loop on the GPU: results of requests served in a mix (three clients of
different sizes, one with an aux camera and soft shadows, three slots, batches of up to
four frames, keyframe pairs replaced while requests run) equal rendering each eye's
requests alone, one isti_render call at a time into one persistent buffer, and the first
frame equals the oracle."""
import random

import numpy as np
import pytest

import oracle
from imagebasedspatiotemporalinterpolation_gb300 import scene
from imagebasedspatiotemporalinterpolation_gb300.renderer import DeviceFrame, Renderer
from imagebasedspatiotemporalinterpolation_gb300.serving import CudaBackend, PinnedPair, Server, SimClient, eye_client, \
    eye_info, simulate

EYES = (-0.032, 0.032)


def make_clients():
    specs = [(96, 54, (), False), (128, 72, (), False), (132, 78, (0.3,), True)]
    out = []
    for cid, (w, h, aux, sh) in enumerate(specs):
        seq = scene.Sequence(w, h, 4, seed=500 + cid, aux_offsets=aux, shadows=sh, max_speed=2.0)
        out.append((cid, seq, [PinnedPair(seq.frame(p)) for p in range(3)]))
    return out


@pytest.mark.gpu
def test_requests_in_a_mix_equal_requests_alone(cuda):
    import torch
    rng = random.Random(7)
    clients = make_clients()
    results = {}
    server = Server(CudaBackend(), hbm_budget=8 << 30, n_slots=3, max_batch=4, slot_pixels=132 * 78, slot_views=4,
                    on_complete=lambda r: results.__setitem__(r.rid, r.out.cpu()))
    pair_of = {}
    log = []            # (rid, cid, eye, pair index, alpha)
    for cid, seq, pairs in clients:
        assert server.open_client(cid, seq.width, seq.height, len(EYES), pairs[0])
        pair_of[cid] = [0]
        server.push_pair(cid, pairs[0])
    for _ in range(240):
        cid, seq, pairs = clients[rng.randrange(len(clients))]
        if rng.random() < 0.06:
            p = len(pair_of[cid]) % len(pairs)
            server.push_pair(cid, pairs[p])
            pair_of[cid].append(p)
        for _ in range(rng.randint(0, 4)):   # bursts: several frames of one eye wait together
            eye = rng.randrange(len(EYES))
            alpha = rng.choice((0.0, 0.25, 0.5, 0.75, 1.0))
            p = pair_of[cid][-1]
            r = server.submit(cid, eye, eye_info(seq, p, alpha, EYES[eye]))
            log.append((r.rid, cid, eye, p, alpha))
        server.step()
    server.drain()
    torch.cuda.synchronize()
    assert len(results) == len(log) > 150
    assert server.stats()["frames_per_batch"] > 1.0
    assert server.uploads >= 4

    # alone: every eye's requests in submission order, frame by frame into one buffer
    single = Renderer()
    frames = {}
    bufs = {}
    for rid, cid, eye, p, alpha in log:
        seq = clients[cid][1]
        if (cid, p) not in frames:
            frames[(cid, p)] = DeviceFrame.from_host(seq.frame(p))
        buf = bufs.setdefault((cid, eye), torch.zeros((seq.height, seq.width, 4), dtype=torch.uint8, device="cuda"))
        single.render(buf, eye_info(seq, p, alpha, EYES[eye]), frames[(cid, p)])
        assert torch.equal(buf.cpu(), results[rid]), f"request {rid} (client {cid}, eye {eye}) differs from rendering it alone"
    single.close()

    # the first frame of each client against the oracle
    for cid, seq, _ in clients:
        rid, _, eye, p, alpha = next(e for e in log if e[1] == cid)
        prev = np.zeros((seq.height, seq.width, 4), np.uint8)
        exp = oracle.run_oracle(seq.frame(p), eye_client(seq, p, alpha, EYES[eye]), prev, with_intermediates=False)[0]
        np.testing.assert_array_equal(results[rid].numpy(), exp)


@pytest.mark.gpu
def test_simulated_clients_report_latency(cuda):
    clients = make_clients()
    server = Server(CudaBackend(), hbm_budget=8 << 30, n_slots=2, max_batch=8, slot_pixels=132 * 78, slot_views=4)
    sims = []
    for cid, seq, pairs in clients:
        server.open_client(cid, seq.width, seq.height, len(EYES), pairs[0])
        sims.append(SimClient(cid, seq, pairs, rate_hz=100.0, phase_s=0.002 * cid))
    st = simulate(server, sims, seconds=1.0, seed=3)
    assert st["requests"] > 300 and st["refused_requests"] == 0
    assert st["requests"] == st["offered_requests"]
    assert 0 < st["p50_ms"] <= st["p99_ms"] < 1000
    assert st["keyframe_pairs_pushed"] >= 3 * 30 - 3


@pytest.mark.gpu
def test_budget_admission_and_closing_on_the_device(cuda):
    """A budget that holds the slots and two of the three clients: the third waits, is
    admitted when the first closes, and every result still equals rendering alone."""
    import torch
    clients = make_clients()
    results = {}
    be = CudaBackend()
    slot_px = 132 * 78
    footprints = []
    probe = Server(be, hbm_budget=1 << 40, n_slots=1, max_batch=2, slot_pixels=slot_px, slot_views=4)
    for cid, seq, pairs in clients:
        footprints.append(probe.footprint(seq.width, seq.height, len(EYES), pairs[0]))
    del probe
    # room for clients 0 and 1, or for 1 and 2 (client 0 is the smallest)
    assert footprints[0] < footprints[2]
    budget = be.slot_bytes(slot_px, 4, 2) + footprints[1] + footprints[2] + footprints[0] // 2
    server = Server(be, hbm_budget=budget, n_slots=1, max_batch=2, slot_pixels=slot_px, slot_views=4,
                    on_complete=lambda r: results.__setitem__(r.rid, r.out.cpu()))
    admitted = [server.open_client(cid, seq.width, seq.height, len(EYES), pairs[0]) for cid, seq, pairs in clients]
    assert admitted == [True, True, False]
    for cid, _, pairs in clients:
        server.push_pair(cid, pairs[1])          # the waiting client keeps its newest pair
    log = []
    for cid, seq, _ in clients[:2]:
        for eye in range(len(EYES)):
            r = server.submit(cid, eye, eye_info(seq, 1, 0.5, EYES[eye]))
            log.append((r.rid, cid, eye, 0.5))
    server.close_client(0)
    server.drain()
    assert server.admitted(2) and not server.admitted(0)
    assert server.reserved <= server.budget
    cid, seq, _ = clients[2]
    for alpha in (0.25, 0.75):
        for eye in range(len(EYES)):
            r = server.submit(cid, eye, eye_info(seq, 1, alpha, EYES[eye]))
            log.append((r.rid, cid, eye, alpha))
    server.drain()
    torch.cuda.synchronize()
    single = Renderer()
    bufs = {}
    for rid, cid, eye, alpha in log:
        seq = clients[cid][1]
        buf = bufs.setdefault((cid, eye), torch.zeros((seq.height, seq.width, 4), dtype=torch.uint8, device="cuda"))
        single.render(buf, eye_info(seq, 1, alpha, EYES[eye]), DeviceFrame.from_host(seq.frame(1)))
        assert torch.equal(buf.cpu(), results[rid]), f"request {rid} differs from rendering it alone"
    single.close()
