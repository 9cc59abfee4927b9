"""Serving loop: client frame requests rendered with continuous batching over
isti_render_batch, keyframes resident on the device, admission against an HBM budget.

The reference renders one client frame per call on the legacy stream
(src/main.cu:137-191, src/renderer.cu:607-694).  This module is the caller side for
many clients at once:

  client   one remote viewer: a render resolution, its keyframe pairs resident in device
           memory (two pair slots: the pair being rendered and the next one being
           uploaded), and per eye a chain of outputs: temporal hole filling continues
           from that eye's previous frame (pixels without a valid result keep the
           previous output, src/renderer.cu:400-465).
  request  one eye's frame at interpolation factor alpha between the client's newest
           keyframe pair (the pair current when the request is submitted).
  slot     a CUDA stream with its own renderer (intermediates); at most one batch in flight.

Admission: a client is admitted when its device footprint (two keyframe pairs and the
output rings of its eyes) fits into the budget beside the clients already admitted and
the slots' renderer arenas; otherwise it waits (deferred, in arrival order) until clients
close.  A request waits while its eye has no free output buffer.  Back-pressure: with
`max_waiting`, a request is refused when its eye already has that many requests waiting
(the device is behind; the client renders that frame itself or drops it).

Continuous batching: whenever a slot is free, the eye with the oldest waiting request
(among eyes with no batch in flight whose pair is uploaded) takes it; up to `max_batch`
of that eye's waiting requests on the same pair are rendered by one chained
isti_render_batch call on the slot's stream, the first output starting as a copy of
the eye's previous output.  When several eyes of that client are ready on the same pair
(a stereo request) and the picked eye has only one request waiting on it, their next
frames share one unchained call instead, each output starting as a copy of its own
eye's previous output: one splat of the keyframe pair for both eyes.  (With a backlog
the chained batch of the picked eye is larger than the stereo call, so it goes first.)  Batches of different clients overlap on the device (one stream per slot).  A new keyframe pair is uploaded into the client's older pair slot
once no waiting or running request uses that slot's pair; the upload waits for the
last batch that read the slot, and batches on the new pair wait for the upload (CUDA
events, no host blocking).

Every result equals rendering the eye's requests one by one, in submission order, into
one persistent buffer with isti_render: the device work is the same whether a request is
served alone or in a mix (tests/test_serving.py, tests/test_serving_gpu.py).

The device side is behind a small backend (CudaBackend here); the scheduling logic runs
unchanged on a fake backend in the CPU tests.
"""
from __future__ import annotations

import collections
import itertools
import time
from dataclasses import dataclass, field

import numpy as np


# ------------------------------------------------------------------ requests and clients

@dataclass
class Request:
    client: int
    eye: int
    info: object              # render info (IstiRenderInfo for CudaBackend)
    pair_seq: int             # keyframe pair the request interpolates in
    rid: int = 0
    pixels: int = 0
    t_submit: float = 0.0
    t_done: float | None = None
    out: object = None        # output buffer while the completion callback runs
    batch: int = -1           # id of the batch that rendered it

    @property
    def latency_ms(self) -> float:
        return (self.t_done - self.t_submit) * 1e3 if self.t_done is not None else float("nan")


@dataclass
class _PairSlot:
    dev: object = None        # backend pair buffers
    seq: int = -1             # keyframe pair held (-1: none)
    ready: object = None      # event: upload done
    last_use: list | None = None  # events of the batches that read it since its upload
    running: int = 0          # batches in flight that read it


@dataclass
class _OutBuf:
    buf: object
    after: list | None = None  # events after which the buffer may be overwritten


@dataclass
class _Eye:
    waiting: collections.deque = field(default_factory=collections.deque)
    free: list = field(default_factory=list)    # _OutBuf
    head: _OutBuf | None = None                 # the eye's previous output (chain start)
    busy: bool = False


@dataclass
class _Client:
    cid: int
    width: int
    height: int
    footprint: int
    eyes: list
    slots: list                                   # two _PairSlot
    arrived: collections.deque = field(default_factory=collections.deque)  # (seq, host pair) not uploaded yet
    newest: int = -1                              # newest pair seq submitted to push_pair
    closing: bool = False


@dataclass
class _Batch:
    bid: int
    slot: int
    client: _Client
    parts: list               # (eye index, its requests, its output buffers) in render order
    pair: _PairSlot
    done: object              # event


def percentile(values, q: float) -> float:
    """q-th percentile (0..100) by linear interpolation between order statistics."""
    if not values:
        return float("nan")
    v = sorted(values)
    pos = (len(v) - 1) * q / 100.0
    lo = int(pos)
    hi = min(lo + 1, len(v) - 1)
    return v[lo] + (v[hi] - v[lo]) * (pos - lo)


# ------------------------------------------------------------------ the request loop

class Server:
    """Continuous-batching request loop over one backend (see the module docstring)."""

    def __init__(self, backend, hbm_budget: int, n_slots: int = 4, max_batch: int = 8, out_ring: int | None = None,
                 slot_pixels: int = 2064 * 2208, slot_views: int = 2, clock=time.perf_counter, on_complete=None,
                 multi_eye: bool = True, max_waiting: int | None = None):
        if n_slots < 1 or not 1 <= max_batch <= backend.max_batch:
            raise ValueError(f"need n_slots >= 1 and 1 <= max_batch <= {backend.max_batch}")
        self.be = backend
        self.budget = int(hbm_budget)
        self.max_batch = max_batch
        self.out_ring = out_ring or (2 * max_batch + 1)
        if self.out_ring < max_batch + 1:
            raise ValueError("out_ring must hold a full batch beside the eye's previous output")
        self.clock = clock
        self.on_complete = on_complete
        self.multi_eye = multi_eye
        if max_waiting is not None and max_waiting < 1:
            raise ValueError("max_waiting must be at least 1")
        self.max_waiting = max_waiting
        self.refused_full = 0            # requests refused by back-pressure (max_waiting)
        self.deferred = 0                # clients that had to wait for budget when they opened
        self.admission_waits: list = []  # seconds from open_client to admission, deferred clients
        self.peak_waiting_clients = 0
        self.clients_opened = 0
        self._opened_at: dict[int, float] = {}
        self._deferred_cids: set = set()
        self.slot_bytes = backend.slot_bytes(slot_pixels, slot_views, max_batch)
        self.reserved = n_slots * self.slot_bytes
        if self.reserved > self.budget:
            raise ValueError(f"{n_slots} slots need {self.reserved} bytes, more than the budget {self.budget}")
        self.slots = [backend.new_slot() for _ in range(n_slots)]
        self.running: list[_Batch | None] = [None] * n_slots
        self.clients: dict[int, _Client] = {}
        self.admit_queue: collections.deque = collections.deque()   # (cid, w, h, n_eyes, template, footprint)
        self.waiting_pairs: dict[int, collections.deque] = {}         # pairs pushed for clients not admitted yet
        self._pair_refs: dict[tuple[int, int], int] = collections.Counter()  # (cid, seq) -> waiting requests
        self._rid = 0
        self._bid = 0
        self.latencies: collections.deque = collections.deque(maxlen=1 << 20)   # the latest requests' latencies (ms)
        self.pixels_done = 0
        self.requests_done = 0
        self.batches = 0
        self.frames_in_batches = 0
        self.uploads = 0
        self.peak_reserved = self.reserved
        self.t_first = None
        self.t_last = None

    # ---- clients

    def footprint(self, width: int, height: int, n_eyes: int, template) -> int:
        return 2 * self.be.pair_bytes(template) + n_eyes * self.out_ring * self.be.output_bytes(width, height)

    def open_client(self, cid: int, width: int, height: int, n_eyes: int, template) -> bool:
        """Registers a client; True when admitted now, False when it waits for budget."""
        if cid in self.clients or any(q[0] == cid for q in self.admit_queue):
            raise ValueError(f"client {cid} already open")
        need = self.footprint(width, height, n_eyes, template)
        if need > self.budget - len(self.slots) * self.slot_bytes:
            raise ValueError(f"client {cid} needs {need} bytes, more than the budget leaves beside the slots")
        self.admit_queue.append((cid, width, height, n_eyes, template, need))
        self.waiting_pairs.setdefault(cid, collections.deque())
        self.clients_opened += 1
        self._opened_at[cid] = self.clock()
        self._admit()
        if cid not in self.clients:
            self.deferred += 1
            self._deferred_cids.add(cid)
            self.peak_waiting_clients = max(self.peak_waiting_clients, len(self.admit_queue))
            return False
        return True

    def admitted(self, cid: int) -> bool:
        return cid in self.clients

    def close_client(self, cid: int) -> None:
        """The client leaves once its waiting and running requests are done."""
        if cid in self.clients:
            c = self.clients[cid]
            c.closing = True
            if not any(e.waiting or e.busy for e in c.eyes):
                self._release(c)
                self._admit()
        else:
            self.admit_queue = collections.deque(q for q in self.admit_queue if q[0] != cid)
            self.waiting_pairs.pop(cid, None)
            self._opened_at.pop(cid, None)
            self._deferred_cids.discard(cid)

    def _admit(self) -> int:
        n = 0
        while self.admit_queue and self.reserved + self.admit_queue[0][5] <= self.budget:
            cid, w, h, n_eyes, template, need = self.admit_queue.popleft()
            slots = [_PairSlot(dev=self.be.alloc_pair(template)) for _ in range(2)]
            eyes = [_Eye(free=[_OutBuf(self.be.alloc_output(w, h)) for _ in range(self.out_ring)]) for _ in range(n_eyes)]
            c = _Client(cid, w, h, need, eyes, slots)
            pend = self.waiting_pairs.pop(cid, collections.deque())
            for seq, host in pend:
                c.arrived.append((seq, host))
                c.newest = seq
            self.clients[cid] = c
            self.reserved += need
            self.peak_reserved = max(self.peak_reserved, self.reserved)
            t_open = self._opened_at.pop(cid, None)
            if cid in self._deferred_cids:
                self._deferred_cids.discard(cid)
                self.admission_waits.append(self.clock() - t_open)
            n += 1
        if n and hasattr(self.be, "settle"):
            self.be.settle()       # the new clients' buffers are initialised before any batch uses them
        return n

    def _release(self, c: _Client) -> None:
        for s in c.slots:
            if s.ready is not None:
                self.be.wait_host(s.ready)
        del self.clients[c.cid]
        self.reserved -= c.footprint

    # ---- keyframes and requests

    def push_pair(self, cid: int, host_pair) -> int:
        """A new keyframe pair arrived for the client (host data in the backend's upload
        format); requests submitted from now on interpolate in it."""
        if cid in self.clients:
            c = self.clients[cid]
            c.newest += 1
            c.arrived.append((c.newest, host_pair))
            return c.newest
        q = self.waiting_pairs.get(cid)
        if q is None:
            raise KeyError(f"client {cid} is not open")
        seq = q[-1][0] + 1 if q else 0
        q.append((seq, host_pair))
        while len(q) > 1:      # a waiting client keeps only its newest pair
            q.popleft()
        return seq

    def submit(self, cid: int, eye: int, info, pixels: int = 0, t_submit: float | None = None) -> Request | None:
        """Queues one eye's frame in the client's newest pair.  Its latency runs from
        t_submit (the server clock; default now).  None: refused by back-pressure (the eye
        already has max_waiting requests waiting)."""
        c = self.clients.get(cid)
        if c is None:
            raise KeyError(f"client {cid} is not admitted")
        if c.closing:
            raise ValueError(f"client {cid} is closing")
        if c.newest < 0:
            raise ValueError(f"client {cid} has no keyframe pair yet")
        if not 0 <= eye < len(c.eyes):
            raise ValueError(f"client {cid} has {len(c.eyes)} eyes")
        if self.max_waiting is not None and len(c.eyes[eye].waiting) >= self.max_waiting:
            self.refused_full += 1
            return None
        now = self.clock() if t_submit is None else t_submit
        self._rid += 1
        r = Request(cid, eye, info, c.newest, self._rid, pixels or c.width * c.height, now)
        c.eyes[eye].waiting.append(r)
        self._pair_refs[(cid, c.newest)] += 1
        if self.t_first is None:
            self.t_first = now
        return r

    # ---- the loop

    def step(self) -> int:
        """Completes finished batches, uploads arrived pairs, launches onto free slots and
        admits waiting clients.  Returns how many of these happened."""
        n = self._complete()
        n += self._uploads()
        n += self._launch()
        n += self._admit()
        return n

    def idle(self) -> bool:
        if any(b is not None for b in self.running):
            return False
        return not any(e.waiting for c in self.clients.values() for e in c.eyes)

    def drain(self, timeout_s: float = 60.0) -> None:
        """Runs the loop until every waiting request is done."""
        t_end = time.perf_counter() + timeout_s
        while not self.idle():
            if not self.step():
                if time.perf_counter() > t_end:
                    raise TimeoutError("requests still waiting after the drain timeout")
                time.sleep(20e-6)
        self.step()

    def _complete(self) -> int:
        n = 0
        for si, b in enumerate(self.running):
            if b is None or not self.be.done(b.done):
                continue
            now = self.clock()
            c = b.client
            for _, reqs, outs in b.parts:
                for r, o in zip(reqs, outs):
                    r.t_done = now
                    r.out = o.buf
                    if self.on_complete is not None:
                        self.on_complete(r)
                    r.out = None
                    self.latencies.append(r.latency_ms)
                    self.pixels_done += r.pixels
                    self.requests_done += 1
            consumed = self.be.consumer_event()
            for ei, _, outs in b.parts:
                eye = c.eyes[ei]
                for o in outs[:-1]:
                    o.after = [consumed]
                    eye.free.append(o)
                outs[-1].after = [consumed]   # the eye's new chain head; freed by its next batch
                eye.busy = False
            b.pair.running -= 1
            if b.pair.last_use and b.done in b.pair.last_use:
                b.pair.last_use.remove(b.done)   # finished: a later upload need not wait for it
            self.running[si] = None
            self.t_last = now
            n += 1
            if c.closing and not any(e.waiting or e.busy for e in c.eyes):
                self._release(c)
        return n

    def _uploads(self) -> int:
        n = 0
        for c in self.clients.values():
            while c.arrived:
                seq, host = c.arrived[0]
                if len(c.arrived) > 1 and self._pair_refs.get((c.cid, seq), 0) == 0:
                    c.arrived.popleft()        # superseded before any request used it
                    continue
                target = min(c.slots, key=lambda s: s.seq)
                if target.seq >= 0 and self._pair_refs.get((c.cid, target.seq), 0) > 0:
                    break                      # requests still wait on the older pair
                waits = [e for e in (target.last_use or []) if e is not None]
                target.ready = self.be.upload(target.dev, host, waits)
                target.seq = seq
                target.last_use = []
                c.arrived.popleft()
                self.uploads += 1
                n += 1
        return n

    def _pick(self):
        best = None
        for c in self.clients.values():
            for ei, e in enumerate(c.eyes):
                if e.busy or not e.waiting or not e.free:
                    continue
                r = e.waiting[0]
                slot = next((s for s in c.slots if s.seq == r.pair_seq), None)
                if slot is None:
                    continue
                if best is None or r.rid < best[0].rid:
                    best = (r, c, ei, slot)
        return best

    def _ready_eyes(self, c: _Client, pslot: _PairSlot) -> list:
        return [ei for ei, e in enumerate(c.eyes)
                if not e.busy and e.free and e.waiting and e.waiting[0].pair_seq == pslot.seq]

    def _launch(self) -> int:
        n = 0
        for si in range(len(self.slots)):
            if self.running[si] is not None:
                continue
            pick = self._pick()
            if pick is None:
                break
            _, c, ei, pslot = pick
            ready = self._ready_eyes(c, pslot)[:self.max_batch] if self.multi_eye else [ei]
            # an eye with a backlog on this pair (the device is behind) takes a chained batch of
            # its own frames instead: fewer, larger calls while the load lasts
            backlog = sum(1 for r in itertools.islice(c.eyes[ei].waiting, 2) if r.pair_seq == pslot.seq) > 1
            if len(ready) > 1 and not backlog:
                # the next frame of every ready eye in one unchained call: each output
                # starts as a copy of its own eye's previous output
                takes, chain = [(x, 1) for x in ready], False
            else:
                e = c.eyes[ei]
                k, m = min(self.max_batch, len(e.free)), 0
                for r in e.waiting:
                    if m >= k or r.pair_seq != pslot.seq:
                        break
                    m += 1
                takes, chain = [(ei, m)], True
            parts, infos, bufs, prefill, waits = [], [], [], [], [pslot.ready]
            for x, m in takes:
                e = c.eyes[x]
                reqs = [e.waiting.popleft() for _ in range(m)]
                outs = [e.free.pop() for _ in reqs]
                for o in outs:
                    waits += o.after or []
                if e.head is not None:
                    waits += e.head.after or []
                    prefill.append((len(bufs), e.head.buf))
                parts.append((x, reqs, outs))
                infos += [r.info for r in reqs]
                bufs += [o.buf for o in outs]
            done = self.be.launch(self.slots[si], bufs, infos, pslot.dev, prefill, chain, waits)
            self._bid += 1
            for x, reqs, outs in parts:
                e = c.eyes[x]
                for r in reqs:
                    r.batch = self._bid
                    self._pair_refs[(c.cid, r.pair_seq)] -= 1
                    if self._pair_refs[(c.cid, r.pair_seq)] == 0:
                        del self._pair_refs[(c.cid, r.pair_seq)]
                if e.head is not None:
                    e.head.after = (e.head.after or []) + [done]   # also read by this batch's copy
                    e.free.append(e.head)
                e.head = outs[-1]
                e.busy = True
            pslot.running += 1
            pslot.last_use = (pslot.last_use or []) + [done]
            self.running[si] = _Batch(self._bid, si, c, parts, pslot, done)
            self.batches += 1
            self.frames_in_batches += len(bufs)
            n += 1
        return n

    def stats(self) -> dict:
        span = (self.t_last - self.t_first) if self.t_first is not None and self.t_last is not None else 0.0
        return {"requests": self.requests_done, "batches": self.batches,
                "frames_per_batch": self.frames_in_batches / self.batches if self.batches else 0.0,
                "uploads": self.uploads, "p50_ms": percentile(self.latencies, 50), "p99_ms": percentile(self.latencies, 99),
                "mpix_per_s": self.pixels_done / span / 1e6 if span > 0 else 0.0, "span_s": span,
                "admitted": len(self.clients), "waiting_clients": len(self.admit_queue),
                "reserved_bytes": self.reserved, "peak_reserved_bytes": self.peak_reserved, "budget_bytes": self.budget,
                "refused_queue_full": self.refused_full, "clients_opened": self.clients_opened,
                "deferred_clients": self.deferred, "peak_waiting_clients": self.peak_waiting_clients,
                "admission_wait_p50_ms": percentile([w * 1e3 for w in self.admission_waits], 50),
                "admission_wait_p99_ms": percentile([w * 1e3 for w in self.admission_waits], 99)}


# ------------------------------------------------------------------ CUDA backend

class PinnedPair:
    """A keyframe pair's host data in pinned memory, ready for asynchronous upload: per view
    (fwd, bwd, then aux curr/next) colour RGBA8, z f32, motion f16x3, shadow A/B/Info RGBA8
    (when present) and the view's matrices."""

    def __init__(self, frame):
        import torch

        def pin(a):
            if a is None:
                return None
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()

        self.views = []
        for v in frame.views():
            mot = None if v.motion is None else pin(v.motion.astype(np.float16))
            self.views.append((pin(v.color), pin(v.z.astype(np.float32)), mot, pin(v.shadow_a), pin(v.shadow_b),
                               pin(v.shadow_info), np.asarray(v.viewproj, np.float32), np.asarray(v.inv_viewproj, np.float32)))
        self.n_aux = len(frame.aux_curr)
        self.aux_priority = list(frame.aux_priority)
        self.width, self.height = frame.fwd.width, frame.fwd.height

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for v in self.views for t in v[:6] if t is not None)


class CudaBackend:
    """Device side of the request loop: torch for buffers, streams and events, libisti for
    every pixel.  With a learned-initialiser checkpoint (`learned_weights`), batches of
    main-camera frames in modes 0/2 go through isti_render_learned (network guess, 1 search
    iteration, per-tile plain fallback); every other batch through isti_render_batch.  Each
    slot owns its network instance (activations are per instance)."""

    def __init__(self, device="cuda", learned_weights: str | None = None, learned_iterations: int = 1):
        import torch

        from .native import MAX_BATCH_FRAMES
        self.torch = torch
        self.device = torch.device(device)
        self.max_batch = MAX_BATCH_FRAMES
        self.upload_stream = torch.cuda.Stream(self.device)
        self.learned_weights = learned_weights
        self.learned_iterations = learned_iterations
        self.learned_batches = self.plain_batches = 0

    @staticmethod
    def slot_bytes(pixels: int, views: int, frames: int) -> int:
        """Renderer arena of one slot: per view splat keys (8 B/px) and client-camera flow
        (x, y and depth, 12 B/px) per frame, keyframe flow (16 B/px) and visibility (1 B/px)."""
        return pixels * views * (20 * frames + 17)

    @staticmethod
    def pair_bytes(template) -> int:
        return template.nbytes()

    @staticmethod
    def output_bytes(width: int, height: int) -> int:
        return width * height * 4

    def new_slot(self):
        from .renderer import Renderer
        slot = [self.torch.cuda.Stream(self.device), Renderer()]
        if self.learned_weights:
            from . import train_flownet
            slot.append(train_flownet.load(self.learned_weights))
        return tuple(slot)

    def alloc_pair(self, template):
        from .renderer import DeviceFrame, DeviceView
        torch = self.torch

        def like(t):
            return None if t is None else torch.empty(tuple(t.shape), dtype=t.dtype, device=self.device)

        views = [DeviceView(like(c), like(z), like(m), like(a), like(b), like(i)) for c, z, m, a, b, i, _, _ in template.views]
        n = template.n_aux
        return DeviceFrame(views[0], views[1], views[2::2][:n], views[3::2][:n], list(template.aux_priority))

    def alloc_output(self, width: int, height: int):
        return self.torch.zeros((height, width, 4), dtype=self.torch.uint8, device=self.device)

    def settle(self) -> None:
        """Waits for the zero fills of newly allocated outputs (issued on the current stream,
        which the slot streams do not order against)."""
        self.torch.cuda.current_stream(self.device).synchronize()

    def _wait(self, stream, events) -> None:
        for ev in events:
            if ev is not None:
                stream.wait_event(ev)

    def upload(self, dev_pair, host: PinnedPair, waits):
        torch = self.torch
        s = self.upload_stream
        self._wait(s, waits)
        with torch.cuda.stream(s):
            for dv, (c, z, m, a, b, i, vp, ivp) in zip(dev_pair.views(), host.views):
                for dst, src in ((dv.color, c), (dv.z, z), (dv.motion, m), (dv.shadow_a, a), (dv.shadow_b, b), (dv.shadow_info, i)):
                    if dst is not None:
                        dst.copy_(src, non_blocking=True)
                dv.viewproj, dv.inv_viewproj = vp, ivp
        dev_pair._c = None      # matrices changed: marshal again
        ev = torch.cuda.Event()
        ev.record(s)
        return ev

    def launch(self, slot, outs, infos, dev_pair, prefill, chain, waits):
        """Renders infos into outs (chained or not) after copying each (index, buffer) of
        `prefill` into outs[index]."""
        torch = self.torch
        stream, renderer = slot[0], slot[1]
        net = slot[2] if len(slot) > 2 else None
        self._wait(stream, waits)
        with torch.cuda.stream(stream):
            for i, src in prefill:
                outs[i].copy_(src, non_blocking=True)
            if net is not None and not dev_pair.aux_curr and all(int(i.mode) in (0, 2) for i in infos):
                renderer.render_learned(outs, infos, dev_pair, net, self.learned_iterations, chain=chain, stream=stream)
                self.learned_batches += 1
            else:
                renderer.render_batch(outs, infos, dev_pair, chain=chain, stream=stream)
                self.plain_batches += 1
        ev = torch.cuda.Event()
        ev.record(stream)
        return ev

    @staticmethod
    def done(ev) -> bool:
        return ev.query()

    def consumer_event(self):
        ev = self.torch.cuda.Event()
        ev.record(self.torch.cuda.current_stream(self.device))
        return ev

    @staticmethod
    def wait_host(ev) -> None:
        ev.synchronize()


# ------------------------------------------------------------------ simulated clients

@dataclass
class SimClient:
    """A simulated viewer: stereo frame requests as a Poisson process, keyframe pairs
    arriving periodically (cycling through the pinned pairs of one scene sequence)."""
    cid: int
    seq: object               # scene.Sequence
    pairs: list               # PinnedPair per pair index of seq
    rate_hz: float
    phase_s: float
    closed: bool = False


_INFO_STEPS = 32   # client cameras are taken at alpha quantised to 1/32 (cached)


def eye_client(seq, k: int, alpha: float, offset: float, mode: int = 0):
    """Client camera (scene.Client) of one eye, `offset` metres along the camera's right
    vector, at interpolation factor alpha between keyframes k and k + 1 of seq."""
    from . import scene
    pose = seq.poses[k].lerp(seq.poses[k + 1], alpha)
    eye = pose.eye + scene.right_vector(pose.yaw, pose.pitch) * offset
    vp = seq.proj_main @ scene.view_matrix(eye, pose.yaw, pose.pitch)
    return scene.Client(seq.width, seq.height, float(np.float32(alpha)), vp.astype(np.float32),
                        np.linalg.inv(vp).astype(np.float32), seq.fpa, seq.sfpa, False, mode)


def eye_info(seq, k: int, alpha: float, offset: float, mode: int = 0):
    """Render info (IstiRenderInfo) of eye_client(seq, k, alpha, offset, mode)."""
    from .renderer import render_info
    return render_info(eye_client(seq, k, alpha, offset, mode))


def simulate(server: Server, sims: list, seconds: float, keyframe_hz: float = 30.0, eyes=(-0.032, 0.032),
             seed: int = 0, session_mean_s: float | None = None, rate_hz=None, make_info=None) -> dict:
    """Runs the clients against the server in real time for `seconds`, then drains.
    Latency runs from a request's scheduled arrival to the loop seeing its batch done.

    session_mean_s: every client leaves after an exponentially distributed session of this
    mean and a new client (next free id, same scene and resolution, request rate drawn by
    `rate_hz(rng)`) opens in its place, admitted when the budget allows.  The clients must
    have been opened on the server by the caller.  make_info(sim, pair index, alpha, eye
    index, eye offset) gives a request's render info (default: eye_info of the sim's scene)."""
    import heapq
    rng = np.random.default_rng(seed)
    heap, order = [], 0
    next_cid = max((s.cid for s in sims), default=-1) + 1

    def schedule(s, t_start):
        nonlocal order
        heap.append((t_start + s.phase_s, order, "kf", s))
        heap.append((t_start + s.phase_s + rng.exponential(1.0 / s.rate_hz), order + 1, "req", s))
        order += 2
        if session_mean_s is not None:
            heap.append((t_start + rng.exponential(session_mean_s), order, "end", s))
            order += 1

    for s in sims:
        schedule(s, 0.0)
    heapq.heapify(heap)
    kf_count = {s.cid: 0 for s in sims}
    kf_time = {s.cid: 0.0 for s in sims}
    pair_of = {s.cid: 0 for s in sims}
    infos = {}
    offered = refused = closed = 0
    t0 = server.clock()
    while True:
        now = server.clock() - t0
        if now >= seconds:
            break
        while heap and heap[0][0] <= now:
            t, _, kind, s = heapq.heappop(heap)
            if s.closed:
                continue
            if kind == "end":
                server.close_client(s.cid)
                s.closed = True
                closed += 1
                n = SimClient(next_cid, s.seq, s.pairs, rate_hz=float(rate_hz(rng)) if rate_hz else s.rate_hz,
                              phase_s=float(rng.uniform(0.0, 1.0 / keyframe_hz)))
                next_cid += 1
                server.open_client(n.cid, n.seq.width, n.seq.height, len(eyes), n.pairs[0])
                kf_count[n.cid], kf_time[n.cid], pair_of[n.cid] = 0, 0.0, 0
                for ev in ((t + n.phase_s, "kf"), (t + n.phase_s + rng.exponential(1.0 / n.rate_hz), "req"),
                           (t + rng.exponential(session_mean_s), "end")):
                    heapq.heappush(heap, (ev[0], order, ev[1], n))
                    order += 1
            elif kind == "kf":
                p = kf_count[s.cid] % len(s.pairs)
                server.push_pair(s.cid, s.pairs[p])
                pair_of[s.cid], kf_time[s.cid] = p, t
                kf_count[s.cid] += 1
                heapq.heappush(heap, (t + 1.0 / keyframe_hz, order, "kf", s))
            else:
                offered += len(eyes)
                if server.admitted(s.cid) and kf_count[s.cid] > 0:
                    q = min(_INFO_STEPS, int((t - kf_time[s.cid]) * keyframe_hz * _INFO_STEPS))
                    for e, off in enumerate(eyes):
                        if make_info is not None:
                            info = make_info(s, pair_of[s.cid], q / _INFO_STEPS, e, off)
                        else:
                            key = (id(s.seq), pair_of[s.cid], q, e)
                            if key not in infos:
                                infos[key] = eye_info(s.seq, pair_of[s.cid], q / _INFO_STEPS, off)
                            info = infos[key]
                        server.submit(s.cid, e, info, t_submit=t0 + t)
                else:
                    refused += len(eyes)
                heapq.heappush(heap, (t + rng.exponential(1.0 / s.rate_hz), order, "req", s))
            order += 1
        server.step()
    server.drain()
    st = server.stats()
    st.update({"offered_requests": offered, "refused_requests": refused, "refused_not_admitted": refused,
               "seconds": seconds, "clients": len(sims), "sessions_closed": closed,
               "keyframe_pairs_pushed": sum(kf_count.values())})
    st["refused_requests"] = refused + st["refused_queue_full"]
    return st
