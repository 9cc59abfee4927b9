"""Scheduling logic of the serving loop (imagebasedspatiotemporalinterpolation_gb300/serving.py)
on a fake device.

The fake device keeps a FIFO of operations per stream and runs them lazily in a random
order that respects only stream order and the event waits the server asks for, so a
missing wait shows up as a wrong result.  A frame's fake "render" folds the request's
info and the keyframe pair's content into the eye's previous output, so every result
pins the whole chain before it: results must equal rendering each eye's requests one by
one in submission order (the reference's persistent render buffer, src/main.cu:137-191).
"""
import collections
import random

import pytest

from imagebasedspatiotemporalinterpolation_gb300.serving import Server, percentile

MASK = (1 << 61) - 1


def fold(prev, info, pair):
    return (prev * 1_000_003 + info * 7919 + pair * 104_729 + 1) & MASK


class Buf:
    def __init__(self):
        self.v = 0


class Pair:
    def __init__(self, nbytes):
        self.nb = nbytes

    def nbytes(self):
        return self.nb


class HostPair(Pair):
    def __init__(self, content, nbytes=1000):
        super().__init__(nbytes)
        self.content = content


class DevPair:
    def __init__(self):
        self.content = None


class Event:
    def __init__(self):
        self.fired = False


class FakeBackend:
    max_batch = 8

    def __init__(self, rng, max_advance=3):
        self.rng = rng
        self.max_advance = max_advance
        self.streams = []
        self.upload_stream = self._stream()
        self.consumer = self._stream()
        self.in_flight = collections.Counter()   # (client tag, eye) -> batches not finished
        self.launch_log = []

    def _stream(self):
        s = collections.deque()
        self.streams.append(s)
        return s

    @staticmethod
    def slot_bytes(pixels, views, frames):
        return pixels * views * (20 * frames + 17)

    @staticmethod
    def pair_bytes(template):
        return template.nbytes()

    @staticmethod
    def output_bytes(w, h):
        return w * h * 4

    def new_slot(self):
        return self._stream()

    def alloc_pair(self, template):
        return DevPair()

    def alloc_output(self, w, h):
        return Buf()

    def _enqueue(self, stream, waits, fn):
        ev = Event()
        stream.append((list(waits), fn, ev))
        return ev

    def upload(self, dev, host, waits):
        def run():
            dev.content = host.content
        return self._enqueue(self.upload_stream, waits, run)

    def launch(self, slot, outs, infos, dev, prefill, chain, waits):
        self.launch_log.append((len(outs), tuple(i[0] for i in infos), tuple(i[2] for i in infos), chain,
                                tuple(i[1] for i in infos)))
        tags = set(i[1] for i in infos)
        assert chain or len(tags) == len(infos), "an unchained batch holds two frames of one eye"
        assert not chain or len(tags) == 1, "a chained batch mixes eyes"
        for tag in tags:
            assert self.in_flight[tag] == 0, "two batches of one eye in flight"
            self.in_flight[tag] += 1

        def run():
            assert dev.content is not None, "batch ran before its pair was uploaded"
            for i, src in prefill:
                outs[i].v = src.v
            prev = outs[0].v
            for o, info in zip(outs, infos):
                assert info[2] == dev.content, "batch ran on a pair slot that held another pair"
                base = prev if chain else o.v
                prev = fold(base, info[0], dev.content)
                o.v = prev
            for tag in tags:
                self.in_flight[tag] -= 1
        return self._enqueue(slot, waits, run)

    def _runnable(self):
        return [s for s in self.streams if s and all(w.fired for w in s[0][0])]

    def advance(self, n):
        for _ in range(n):
            ready = self._runnable()
            if not ready:
                return
            s = self.rng.choice(ready)
            _, fn, ev = s.popleft()
            fn()
            ev.fired = True

    def done(self, ev):
        self.advance(self.rng.randint(0, self.max_advance))
        return ev.fired

    def consumer_event(self):
        ev = Event()
        ev.fired = True
        return ev

    def wait_host(self, ev):
        while not ev.fired:
            before = sum(len(s) for s in self.streams)
            self.advance(1)
            assert sum(len(s) for s in self.streams) < before, "device stalled"


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-4
        return self.t


def run_mix(seed, n_clients=4, n_eyes=2, n_slots=3, max_batch=4, steps=600, push_p=0.03, submit_p=0.5, out_ring=None,
            max_advance=3, multi_eye=True):
    rng = random.Random(seed)
    be = FakeBackend(rng, max_advance)
    results = {}
    server = Server(be, hbm_budget=10**12, n_slots=n_slots, max_batch=max_batch, out_ring=out_ring, slot_pixels=64 * 36,
                    clock=Clock(), on_complete=lambda r: results.__setitem__(r.rid, r.out.v), multi_eye=multi_eye)
    pair_content = {}
    submitted = collections.defaultdict(list)     # (cid, eye) -> [(rid, info value, pair content)]
    next_content = 1
    for c in range(n_clients):
        assert server.open_client(c, 64, 36, n_eyes, Pair(1000))
        server.push_pair(c, HostPair(next_content))
        pair_content[(c, 0)] = next_content
        next_content += 1
    for _ in range(steps):
        c = rng.randrange(n_clients)
        if rng.random() < push_p:
            seq = server.push_pair(c, HostPair(next_content))
            pair_content[(c, seq)] = next_content
            next_content += 1
        if rng.random() < submit_p:
            eye = rng.randrange(n_eyes)
            seq = server.clients[c].newest
            info_v = rng.randrange(1 << 20)
            r = server.submit(c, eye, (info_v, (c, eye), pair_content[(c, seq)]))
            submitted[(c, eye)].append((r.rid, info_v, pair_content[(c, seq)]))
        server.step()
    server.drain(timeout_s=5.0)
    return server, be, results, submitted


@pytest.mark.parametrize("multi_eye", [True, False], ids=["stereo-batches", "eye-batches"])
@pytest.mark.parametrize("seed", range(8))
def test_results_equal_sequential_renders_in_any_device_order(seed, multi_eye):
    server, be, results, submitted = run_mix(seed, n_eyes=2 + seed % 2, multi_eye=multi_eye)
    n = 0
    for key, reqs in submitted.items():
        prev = 0
        for rid, info_v, content in reqs:
            prev = fold(prev, info_v, content)
            assert results[rid] == prev, f"request {rid} of eye {key} differs from the sequential render"
            n += 1
    assert n == server.requests_done > 100
    assert server.uploads >= 4


@pytest.mark.parametrize("seed", range(6))
def test_keyframe_pairs_replaced_under_load(seed):
    """A slow device, one slot and new keyframe pairs arriving almost every step: uploads
    must wait for the batches still reading the older pair slot and for the requests
    still queued on it."""
    server, _, results, submitted = run_mix(100 + seed, n_clients=2, n_slots=1, max_batch=3, steps=500, push_p=0.6,
                                            submit_p=0.9, max_advance=1)
    for reqs in submitted.values():
        prev = 0
        for rid, info_v, content in reqs:
            prev = fold(prev, info_v, content)
            assert results[rid] == prev
    assert server.uploads > 50


def test_batches_respect_size_and_pair_limits():
    server, be, _, _ = run_mix(3, n_clients=2, max_batch=3, submit_p=0.9, push_p=0.05, steps=800)
    assert be.launch_log
    for size, _, pairs, _, _ in be.launch_log:
        assert 1 <= size <= 3
        assert len(set(pairs)) == 1, "a batch mixed keyframe pairs"
    assert any(size > 1 and chain for size, _, _, chain, _ in be.launch_log), "no eye's frames were ever batched"
    assert any(not chain for _, _, _, chain, _ in be.launch_log), "no stereo batch"


def test_small_output_ring_applies_backpressure():
    server, _, results, submitted = run_mix(5, n_clients=2, max_batch=2, out_ring=3, submit_p=0.9, steps=400)
    for reqs in submitted.values():
        prev = 0
        for rid, info_v, content in reqs:
            prev = fold(prev, info_v, content)
            assert results[rid] == prev


def test_admission_waits_for_budget_and_follows_closing_clients():
    rng = random.Random(1)
    be = FakeBackend(rng)
    slot = FakeBackend.slot_bytes(64 * 36, 2, 2)
    pair = Pair(5000)
    need = 2 * 5000 + 2 * 5 * 64 * 36 * 4
    server = Server(be, hbm_budget=slot + need + need // 2, n_slots=1, max_batch=2, slot_pixels=64 * 36, clock=Clock())
    assert server.open_client(0, 64, 36, 2, pair)
    assert not server.open_client(1, 64, 36, 2, pair)
    assert server.stats()["waiting_clients"] == 1
    with pytest.raises(KeyError):
        server.submit(1, 0, (1, (1, 0), 1))
    server.push_pair(1, HostPair(7))          # kept for the waiting client
    server.push_pair(0, HostPair(3))
    r = server.submit(0, 0, (5, (0, 0), 3))
    server.close_client(0)
    server.drain()
    assert r.t_done is not None
    assert server.admitted(1) and not server.admitted(0)
    assert server.reserved <= server.budget and server.peak_reserved <= server.budget
    r1 = server.submit(1, 1, (9, (1, 1), 7))  # the pair pushed while waiting was uploaded on admission
    server.drain()
    assert r1.t_done is not None and server.uploads == 2
    with pytest.raises(ValueError):
        Server(be, hbm_budget=slot - 1, n_slots=1, max_batch=2, slot_pixels=64 * 36)
    with pytest.raises(ValueError):
        server.open_client(2, 64, 36, 2, Pair(10**9))


def test_submit_errors():
    be = FakeBackend(random.Random(0))
    server = Server(be, hbm_budget=10**9, n_slots=1, max_batch=2, slot_pixels=64 * 36, clock=Clock())
    server.open_client(0, 64, 36, 2, Pair(10))
    with pytest.raises(ValueError):
        server.submit(0, 0, (1, (0, 0), 1))   # no keyframe pair yet
    server.push_pair(0, HostPair(1))
    with pytest.raises(ValueError):
        server.submit(0, 2, (1, (0, 2), 1))   # no such eye
    with pytest.raises(ValueError):
        server.open_client(0, 64, 36, 2, Pair(10))


def test_percentile():
    assert percentile([], 50) != percentile([], 50)   # NaN
    assert percentile([3.0], 99) == 3.0
    assert percentile([1.0, 2.0, 3.0, 4.0], 50) == 2.5
    assert percentile(list(range(101)), 99) == 99.0


def test_pair_slot_keeps_only_running_readers():
    """A client whose keyframes stop arriving: its pair slot remembers only the batches
    still running on it (the events a later upload has to wait for), not every batch."""
    server, _, _, _ = run_mix(11, n_clients=1, n_slots=2, push_p=0.0, submit_p=0.9, steps=300)
    c = server.clients[0]
    assert server.batches > 100
    assert all(len(s.last_use or []) <= len(server.slots) for s in c.slots)


def test_closing_an_idle_client_frees_its_budget_at_once():
    be = FakeBackend(random.Random(2))
    slot = FakeBackend.slot_bytes(64 * 36, 2, 2)
    need = 2 * 5000 + 2 * 5 * 64 * 36 * 4
    server = Server(be, hbm_budget=slot + need, n_slots=1, max_batch=2, slot_pixels=64 * 36, clock=Clock())
    assert server.open_client(0, 64, 36, 2, Pair(5000))
    assert not server.open_client(1, 64, 36, 2, Pair(5000))
    server.close_client(0)                 # nothing waiting or running
    assert not server.admitted(0) and server.admitted(1)
    assert server.reserved == slot + need
    server.close_client(1)
    assert server.reserved == slot and not server.clients


def _fold_chain(prev, infos_and_content):
    v = prev
    for info_v, content in infos_and_content:
        v = fold(v, info_v, content)
    return v


def test_client_disconnecting_mid_batch():
    """A client closes while one of its batches runs on the device: its requests already
    submitted are completed (results equal sequential renders), new requests are refused,
    its budget is released only after the batch finished, and another client is unaffected."""
    rng = random.Random(5)
    be = FakeBackend(rng, max_advance=0)          # nothing runs until waited for
    results = {}
    server = Server(be, hbm_budget=10**12, n_slots=2, max_batch=4, slot_pixels=64 * 36, clock=Clock(),
                    on_complete=lambda r: results.__setitem__(r.rid, r.out.v))
    for c in (0, 1):
        assert server.open_client(c, 64, 36, 1, Pair(100))
        server.push_pair(c, HostPair(10 + c))
    reqs = {0: [], 1: []}
    for i in range(3):
        for c in (0, 1):
            reqs[c].append((server.submit(c, 0, (i + 7 * c, (c, 0), 10 + c)), i + 7 * c))
    server.step()
    assert any(b is not None and b.client.cid == 0 for b in server.running), "client 0 has a batch in flight"
    reserved = server.reserved
    server.close_client(0)
    assert server.admitted(0)                      # still draining its requests
    with pytest.raises(ValueError):
        server.submit(0, 0, (99, (0, 0), 10))
    be.max_advance = 3                             # let the device run
    server.drain(timeout_s=5.0)
    assert not server.admitted(0) and server.admitted(1)
    assert server.reserved < reserved
    for c in (0, 1):
        prev = 0
        for r, info_v in reqs[c]:
            prev = fold(prev, info_v, 10 + c)
            assert results[r.rid] == prev


def test_keyframe_missing_at_request_time():
    """No keyframe pair yet: the request is refused.  A pair pushed but not yet uploaded on
    the device: the request is accepted and its batch waits for the upload (the fake device
    asserts that no batch runs before its pair's upload)."""
    rng = random.Random(6)
    be = FakeBackend(rng, max_advance=0)
    results = {}
    server = Server(be, hbm_budget=10**12, n_slots=1, max_batch=2, slot_pixels=64 * 36, clock=Clock(),
                    on_complete=lambda r: results.__setitem__(r.rid, r.out.v))
    assert server.open_client(0, 64, 36, 1, Pair(100))
    with pytest.raises(ValueError):
        server.submit(0, 0, (1, (0, 0), 21))
    server.push_pair(0, HostPair(21))
    r = server.submit(0, 0, (1, (0, 0), 21))      # the upload has not run on the device yet
    server.step()
    be.max_advance = 3
    server.drain(timeout_s=5.0)
    assert results[r.rid] == fold(0, 1, 21)


def test_back_pressure_refuses_requests_beyond_max_waiting():
    """With max_waiting = 2 an eye holds at most two waiting requests; further submits are
    refused (None) and counted, and the accepted ones still equal sequential renders."""
    rng = random.Random(11)
    be = FakeBackend(rng, max_advance=2)          # nothing runs before the loop steps
    results = {}
    server = Server(be, hbm_budget=10**12, n_slots=1, max_batch=2, slot_pixels=64 * 36, clock=Clock(),
                    on_complete=lambda r: results.__setitem__(r.rid, r.out.v), max_waiting=2)
    assert server.open_client(0, 64, 36, 1, Pair(1000))
    server.push_pair(0, HostPair(5))
    got = [server.submit(0, 0, (v, (0, 0), 5)) for v in range(5)]
    assert [r is not None for r in got] == [True, True, False, False, False]
    assert server.stats()["refused_queue_full"] == 3
    server.drain(timeout_s=5.0)
    prev = 0
    for r, v in zip(got[:2], range(2)):
        prev = fold(prev, v, 5)
        assert results[r.rid] == prev
    # once the queue has drained the eye accepts requests again
    assert server.submit(0, 0, (9, (0, 0), 5)) is not None
    server.drain(timeout_s=5.0)


class FakeSeq:
    def __init__(self, w, h):
        self.width, self.height = w, h


def test_sessions_defer_admission_and_every_accepted_request_completes():
    """Client churn under a budget that admits only some clients at a time: clients leave
    after their sessions and replacements open; the ones that do not fit wait (deferred)
    and are admitted as others close.  Every request accepted from an admitted client is
    rendered; requests of waiting clients and beyond max_waiting are refused."""
    from imagebasedspatiotemporalinterpolation_gb300.serving import SimClient, simulate
    rng = random.Random(4)
    be = FakeBackend(rng, max_advance=2)
    slot = FakeBackend.slot_bytes(64 * 36, 2, 2)
    need = 2 * 1000 + 2 * 5 * 64 * 36 * 4
    server = Server(be, hbm_budget=slot + 3 * need, n_slots=1, max_batch=2, slot_pixels=64 * 36, clock=Clock(),
                    max_waiting=2)
    seq = FakeSeq(64, 36)
    pairs = [HostPair(11), HostPair(12)]
    sims = [SimClient(c, seq, pairs, rate_hz=400.0, phase_s=0.0) for c in range(6)]
    for s in sims:
        server.open_client(s.cid, 64, 36, 2, pairs[0])
    assert server.stats()["admitted"] == 3 and server.stats()["waiting_clients"] == 3

    def make_info(sim, p, alpha, e, off):
        return (int(alpha * 32), (sim.cid, e), sim.pairs[p].content)

    st = simulate(server, sims, seconds=0.6, keyframe_hz=30.0, eyes=(-0.03, 0.03), seed=3, session_mean_s=0.1,
                  rate_hz=lambda g: 400.0, make_info=make_info)
    assert st["sessions_closed"] > 3
    assert st["clients_opened"] == 6 + st["sessions_closed"]
    assert st["deferred_clients"] >= 3
    assert st["admission_wait_p50_ms"] > 0.0
    assert st["refused_not_admitted"] > 0
    assert st["peak_reserved_bytes"] <= server.budget
    assert st["requests"] == st["offered_requests"] - st["refused_requests"]


def test_backlogged_eye_takes_a_chained_batch_before_the_stereo_call():
    """One request per eye: both eyes share one unchained (stereo) call.  An eye with a
    backlog on the pair takes a chained batch of its own frames first."""
    for backlog, want in ((1, (2, False)), (3, (3, True))):
        rng = random.Random(2)
        be = FakeBackend(rng, max_advance=0)
        server = Server(be, hbm_budget=10**12, n_slots=1, max_batch=4, slot_pixels=64 * 36, clock=Clock())
        assert server.open_client(0, 64, 36, 2, Pair(1000))
        server.push_pair(0, HostPair(5))
        for i in range(backlog):
            server.submit(0, 0, (i, (0, 0), 5))
        server.submit(0, 1, (9, (0, 1), 5))
        server.step()
        be.advance(10)              # the upload
        server.step()
        assert be.launch_log, "nothing launched"
        size, _, _, chain, _ = be.launch_log[0]
        assert (size, chain) == want
        be.max_advance = 3
        server.drain(timeout_s=5.0)
