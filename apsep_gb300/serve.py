"""Serving loop: APSE requests as they arrive, batched into segmented runs
over device-resident pools (continuous batching).

    server = PoolServer(budget_bytes=8 << 30)
    stats = server.serve(requests)        # requests: list[Request], arrival times in seconds
    stats.p50_ms, stats.p99_ms, stats.requests_per_s, stats.keys_per_s

A request is one array of keys (int32 or float32; device memory, or pinned
host memory) with a comparator, an arrival time and where its answers go.
The server carves, from an HBM byte budget, one ring of keys and one ring of
answers per kind (key type x comparator) and a few lanes (a stream and a plan
each).  Arrived requests are admitted in FIFO order as ring space frees up,
their keys gathered into the ring (one native copy launch per batch's worth
of requests); each idle lane runs the next admitted requests that sit back to
back in the ring as ONE segmented launch, in place; a completed launch
releases its requests' ring spans.  Copies of the next batch overlap the run
of this one on other streams, and both kinds' lanes run side by side.
`device_loop` is the baseline it is measured against: one apsep_run per
request, synchronised after each.
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np
import torch

from . import _lib
from .api import Plan


@dataclasses.dataclass
class Request:
    rid: int
    keys: torch.Tensor            # int32 or float32 keys: pinned host memory, or (PoolServer) device memory
    arrival: float = 0.0          # seconds after serve() starts
    inclusive: bool = False       # <= instead of <
    answers: np.ndarray | None = None  # filled when keep_answers
    t_done: float | None = None
    out: torch.Tensor | None = None    # PoolServer: where the answers go (int32, device or pinned host)
    failed: bool = False               # PoolServer: its launch reported a device-side error
    slot: int | None = None            # PoolServer: start of its span in the ring (None: run in place)
    _copied: object = None             # PoolServer: event after the copy of its keys into the ring

    @property
    def kind(self) -> tuple:
        return (self.keys.dtype, bool(self.inclusive))

    @property
    def n(self) -> int:
        return int(self.keys.numel())


@dataclasses.dataclass
class ServeStats:
    requests: int
    keys: int
    makespan_s: float
    latencies_ms: list
    batches: int
    device_bytes: int

    @property
    def requests_per_s(self) -> float:
        return self.requests / self.makespan_s if self.makespan_s > 0 else 0.0

    @property
    def keys_per_s(self) -> float:
        return self.keys / self.makespan_s if self.makespan_s > 0 else 0.0

    def pct(self, q: float) -> float:
        return float(np.percentile(np.asarray(self.latencies_ms), q)) if self.latencies_ms else 0.0

    @property
    def p50_ms(self) -> float:
        return self.pct(50)

    @property
    def p99_ms(self) -> float:
        return self.pct(99)

    def as_dict(self) -> dict:
        return {"requests": self.requests, "keys": self.keys, "makespan_s": round(self.makespan_s, 6),
                "requests_per_s": round(self.requests_per_s, 2), "keys_per_s": round(self.keys_per_s, 1),
                "useful_gbs": round(8.0 * self.keys_per_s / 1e9, 2),
                "p50_ms": round(self.p50_ms, 4), "p99_ms": round(self.p99_ms, 4), "batches": self.batches,
                "device_bytes": self.device_bytes}


# ---------------------------------------------------------------------------
# Continuous batching over device-resident pools
# ---------------------------------------------------------------------------
class RingPool:
    """Host bookkeeping of a ring of `capacity` key slots in device memory.

    alloc(n) hands out a contiguous span of whole `align`-key units at the
    head (so every span starts 16-byte aligned and a batch of consecutive
    spans streams through TMA), wrapping to the start of the ring when the
    span does not fit before its end; it returns None when no such span is
    free.  free(start) releases a span in any order; the space of the oldest
    spans is reclaimed from the tail as soon as they are free."""

    def __init__(self, capacity: int, align: int = 4):
        self.align = int(align)
        self.capacity = int(capacity) // self.align * self.align
        self._spans = collections.deque()  # [start, size, freed], in allocation order
        self._live = {}
        self.head = 0

    def span_size(self, n: int) -> int:
        return max(self.align, (int(n) + self.align - 1) // self.align * self.align)

    @property
    def used(self) -> int:
        """Slots between the tail and the head (live spans and the gaps among them)."""
        if not self._spans:
            return 0
        tail = self._spans[0][0]
        return self.head - tail if self.head > tail else self.capacity - tail + self.head

    def alloc(self, n: int):
        size = self.span_size(n)
        if size > self.capacity:
            return None
        if not self._spans:
            start = 0
        else:
            tail = self._spans[0][0]
            if self.head == tail:  # head caught up with the tail: full
                return None
            if self.head > tail:  # free: [head, capacity) and [0, tail)
                if self.head + size <= self.capacity:
                    start = self.head
                elif size <= tail:
                    start = 0
                else:
                    return None
            else:  # wrapped; free: [head, tail)
                if self.head + size <= tail:
                    start = self.head
                else:
                    return None
        e = [start, size, False]
        self._spans.append(e)
        self._live[start] = e
        self.head = start + size
        return start

    def free(self, start: int) -> None:
        e = self._live.pop(int(start))
        e[2] = True
        while self._spans and self._spans[0][2]:
            self._spans.popleft()
        if not self._spans:
            self.head = 0


class _Lane:
    def __init__(self, kind, capacity_keys: int, max_segments: int, device):
        dtype, incl = kind
        self.plan = Plan(capacity_keys, dtype, inclusive=incl, device=device)
        self.stream = torch.cuda.Stream(device=device)
        self.event = torch.cuda.Event()
        self.offs = torch.empty(max_segments + 1, dtype=torch.int64, device=device)
        self.offs_host = torch.empty(max_segments + 1, dtype=torch.int64).pin_memory()
        self.err_host = torch.zeros(1, dtype=torch.int32).pin_memory()
        self.batch: list = []

    def device_bytes(self) -> int:
        return int(self.plan.info().scratch_bytes) + self.offs.numel() * 8


class PoolServer:
    """Continuous batching: APSE requests as they arrive, over device-resident
    pools carved from an HBM byte budget.

    Per kind (key type x comparator) the server owns a ring of keys and a
    ring of answers in HBM (RingPool bookkeeping), `lanes_per_kind` lanes
    (a stream and a plan each) and a copy stream.  A request's keys live in
    the client's memory (device, or pinned host); its answers go to
    `request.out` (device or pinned host, int32), or, when out is None and
    keep_answers is set, to host memory.

    The loop admits arrived requests of each kind in FIFO order as ring space
    frees up (a span of whole 4-key units; nothing is allocated per request)
    and copies their keys in on the copy stream.  Whenever a lane is idle it
    takes the admitted requests that sit back to back in the ring (up to
    max_batch_keys and max_segments) and runs them as ONE segmented launch in
    place, then copies each request's answers out, all on the lane's stream,
    which waits for the copy-in only through an event: the next batch's
    copies overlap this batch's run, and the lanes of both kinds run side by
    side.  When a lane's batch completes its requests are done and their
    ring spans are released.  Size classes: a request of at least
    direct_min_keys keys whose keys are device memory on a 16-byte boundary
    is not copied at all: it runs from its own keys on a lane as a
    single-array launch, into its device output (on a 16-byte boundary) or,
    with out None, into a span of the answer ring.  After every launch the lane enqueues a copy of its
    plan's error word; a batch whose word is nonzero is marked failed when it
    retires (and the plan re-armed), so an error is tied to its requests."""

    def __init__(self, budget_bytes: int = 8 << 30, kinds=((torch.int32, False), (torch.float32, False)),
                 lanes_per_kind: int = 2, max_batch_keys: int = 1 << 27, max_segments: int = 4096,
                 direct_min_keys: int | None = None, ring_keys: int | None = None, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.kinds = [(k[0], bool(k[1])) for k in kinds]
        self.budget_bytes = int(budget_bytes)
        self.max_batch_keys = int(max_batch_keys)
        self.max_segments = int(max_segments)
        self.direct_min_keys = None if direct_min_keys is None else int(direct_min_keys)
        self.lanes = {k: [_Lane(k, self.max_batch_keys, self.max_segments, self.device)
                          for _ in range(lanes_per_kind)] for k in self.kinds}
        lane_bytes = sum(ln.device_bytes() for ls in self.lanes.values() for ln in ls)
        fit = (self.budget_bytes - lane_bytes) // (8 * len(self.kinds)) // 4 * 4  # keys + answers per slot
        cap = fit if ring_keys is None else min(int(ring_keys), fit)
        if cap < 4:
            self.close()
            raise ValueError("budget of %d bytes leaves no room for the rings" % budget_bytes)
        self.rings = {}
        for k in self.kinds:
            # zeros: the padding after a request (its span's last 0-3 keys) then only ever
            # holds earlier requests' keys, never a NaN bit pattern
            self.rings[k] = (torch.zeros(cap, dtype=k[0], device=self.device),
                             torch.empty(cap, dtype=torch.int32, device=self.device))
        self.ring_keys = int(cap)
        self.copy_streams = {k: torch.cuda.Stream(device=self.device) for k in self.kinds}
        self.device_bytes = lane_bytes + 8 * cap * len(self.kinds)
        if self.device_bytes > self.budget_bytes:
            self.close()
            raise RuntimeError("pools (%d bytes) exceed the budget (%d bytes)" % (self.device_bytes, budget_bytes))

    def close(self) -> None:
        for ls in getattr(self, "lanes", {}).values():
            for ln in ls:
                ln.plan.close()

    def _direct(self, r: Request) -> bool:
        # device keys on a 16-byte boundary; answers to a device out on one, or
        # (out None) into the answer ring
        return (self.direct_min_keys is not None and r.n >= self.direct_min_keys and r.keys.is_cuda
                and r.keys.data_ptr() % 16 == 0 and r.n <= self.max_batch_keys
                and ((r.out is None and r.n <= self.ring_keys) or
                     (r.out is not None and r.out.is_cuda and r.out.data_ptr() % 16 == 0)))

    def _finish_launch(self, ln: _Lane) -> None:
        ln.plan.error_async(ln.err_host, stream=ln.stream)
        ln.event.record(ln.stream)

    def _launch_direct(self, kind, ln: _Lane, r: Request) -> None:
        ln.batch = [r]
        out = r.out[:r.n] if r.out is not None else self.rings[kind][1][r.slot:r.slot + r.n]
        ln.plan.run(r.keys, out=out, n=r.n, stream=ln.stream)
        self._finish_launch(ln)

    def _launch_batch(self, kind, ln: _Lane, batch: list, copied: torch.cuda.Event) -> None:
        keys_ring, ans_ring = self.rings[kind]
        base = batch[0].slot
        offs = [r.slot - base for r in batch]
        total = batch[-1].slot + batch[-1]._span - base  # the last span's padding included
        offs.append(total)
        ns = len(batch)
        ln.batch = batch
        ln.stream.wait_event(copied)
        with torch.cuda.stream(ln.stream):
            ln.offs_host[:ns + 1] = torch.tensor(offs, dtype=torch.int64)
            ln.offs[:ns + 1].copy_(ln.offs_host[:ns + 1], non_blocking=True)
            ln.plan.run_segmented(keys_ring[base:base + total], ln.offs[:ns + 1],
                                  out=ans_ring[base:base + total], stream=ln.stream)
            srcs, dsts, nb = [], [], []
            a0 = ans_ring.data_ptr()
            for r in batch:
                if r.out is None or r.n == 0:
                    continue
                if r.out.is_cuda:  # device answers: one gathered copy for the batch
                    srcs.append(a0 + 4 * r.slot)
                    dsts.append(r.out.data_ptr())
                    nb.append(4 * r.n)
                else:
                    r.out[:r.n].copy_(ans_ring[r.slot:r.slot + r.n], non_blocking=True)
            _lib.copy_spans(srcs, dsts, nb, ln.stream.cuda_stream)
        self._finish_launch(ln)

    def _retire(self, kind, ln: _Lane, now: float, on_done) -> None:
        if int(ln.err_host[0]) != 0:
            try:
                ln.plan.check(stream=ln.stream)  # decode and clear; the batch's answers are not valid
            except Exception:
                pass
            for r in ln.batch:
                r.failed = True
        ans_ring = self.rings[kind][1]
        for r in ln.batch:
            r.t_done = now
            if on_done is not None:
                # the answers in the pool (or r.out), valid during the call
                on_done(r, ans_ring[r.slot:r.slot + r.n] if r.slot is not None else r.out[:r.n])
            if r.slot is not None:
                self._pools[kind].free(r.slot)
        ln.batch = []

    def _admit_chunk(self, k, waiting, admitted, ahead) -> bool:
        """Admit waiting requests of kind k, in order, while ring space allows, up
        to a batch's worth of keys; one gathered copy of their keys into the ring
        and one event after it.  A request run in place goes to an idle lane
        instead.  False when nothing could be admitted."""
        ring = self._pools[k]
        keys_ring = self.rings[k][0]
        cs = self.copy_streams[k]
        k0, esz = keys_ring.data_ptr(), keys_ring.element_size()
        srcs, dsts, nb, chunk = [], [], [], []
        keys = 0
        while waiting and keys < self.max_batch_keys:
            r = waiting[0]
            if r._direct:
                if admitted or chunk:
                    break  # FIFO: the batched requests before it go first
                idle = [ln for ln in self.lanes[k] if not ln.batch]
                if not idle:
                    break
                if r.out is None:  # its answers take a ring span (its keys stay where they are)
                    start = ring.alloc(r._n)
                    if start is None:
                        break
                    r.slot = start
                waiting.popleft()
                self._launch_direct(k, idle[0], r)
                self._nbatches += 1
                return True
            start = ring.alloc(r._n)
            if start is None:
                break
            waiting.popleft()
            r.slot = start
            if r._dev:
                if r._n:
                    srcs.append(r._ptr)
                    dsts.append(k0 + esz * start)
                    nb.append(esz * r._n)
            else:
                with torch.cuda.stream(cs):
                    keys_ring[start:start + r._n].copy_(r.keys, non_blocking=True)
            chunk.append(r)
            keys += r._span
        if not chunk:
            return False
        _lib.copy_spans(srcs, dsts, nb, cs.cuda_stream)
        ev = torch.cuda.Event()
        ev.record(cs)
        for r in chunk:
            r._copied = ev
        admitted.extend(chunk)
        ahead[k] += keys
        return True

    def _launch_ready(self, k, admitted, ahead) -> bool:
        """Each idle lane of kind k takes the next run of back-to-back admitted
        requests (up to max_batch_keys, max_segments) as one launch."""
        launched = False
        for ln in self.lanes[k]:
            if ln.batch or not admitted:
                continue
            batch = [admitted.popleft()]
            keys = batch[0]._span
            while admitted and len(batch) < self.max_segments:
                r = admitted[0]
                if r.slot != batch[-1].slot + batch[-1]._span or keys + r._span > self.max_batch_keys:
                    break
                batch.append(admitted.popleft())
                keys += r._span
            ahead[k] -= keys
            self._launch_batch(k, ln, batch, batch[-1]._copied)
            self._nbatches += 1
            launched = True
        return launched

    def serve(self, requests: list, keep_answers: bool = False, realtime: bool = True,
              on_done=None) -> ServeStats:
        """Run the loop until every request completes.  realtime=False makes
        every request arrive at once (saturation throughput).  A request with
        out=None leaves its answers in the pool: on_done(request, answers) is
        called when it completes, with a device view that stays valid only
        during the call (its pool span is released right after);
        keep_answers gives such requests a pinned host out instead."""
        for r in requests:
            if r.kind not in self.lanes:
                raise ValueError("no pool for keys of %s (inclusive=%s)" % r.kind)
            if r.n > min(self.max_batch_keys, self.ring_keys) and not self._direct(r):
                raise ValueError("request %d (%d keys) exceeds a batch (%d keys)" % (r.rid, r.n,
                                 min(self.max_batch_keys, self.ring_keys)))
            if not r.keys.is_contiguous() or (r.out is not None and (not r.out.is_contiguous()
                                                                   or r.out.dtype != torch.int32
                                                                   or r.out.numel() < r.n)):
                raise ValueError("request %d: keys and out must be contiguous, out int32 of n entries" % r.rid)
            if keep_answers and r.out is None:
                r.out = torch.empty(r.n, dtype=torch.int32).pin_memory()
            r.failed = False
            r.slot = None
            r.t_done = None
        self._pools = {k: RingPool(self.ring_keys) for k in self.kinds}
        for r in requests:  # looked up once: the loop below runs per request
            r._n = r.n
            r._kind = r.kind
            r._span = self._pools[r._kind].span_size(r._n)
            r._dev = r.keys.is_cuda
            r._ptr = r.keys.data_ptr()
            r._direct = self._direct(r)
        order = sorted(requests, key=lambda r: r.arrival if realtime else 0.0)
        waiting = {k: collections.deque() for k in self.kinds}
        admitted = {k: collections.deque() for k in self.kinds}  # in the ring, not yet launched
        ahead = {k: 0 for k in self.kinds}  # keys admitted, not yet launched
        lookahead = 2 * self.max_batch_keys
        self._nbatches = 0
        nxt = done = 0
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        while done < len(order):
            now = time.perf_counter() - t0
            while nxt < len(order) and (not realtime or order[nxt].arrival <= now):
                waiting[order[nxt]._kind].append(order[nxt])
                nxt += 1
            progressed = False
            for k in self.kinds:
                for ln in self.lanes[k]:
                    if ln.batch and ln.event.query():
                        done += len(ln.batch)
                        self._retire(k, ln, time.perf_counter() - t0, on_done)
                        progressed = True
                # admission (FIFO: a request waits for ring space, or, run in place, for a
                # lane) a batch's worth at a time, each chunk's launch right behind its copy
                while True:
                    if self._launch_ready(k, admitted[k], ahead):
                        progressed = True
                    if not waiting[k] or ahead[k] >= lookahead:
                        break
                    if not self._admit_chunk(k, waiting[k], admitted[k], ahead):
                        break
                    progressed = True
            if not progressed:
                time.sleep(0)
        t_end = time.perf_counter() - t0
        if keep_answers:
            for r in order:
                r.answers = r.out[:r.n].cpu().numpy() if r.out.is_cuda else r.out[:r.n].numpy().copy()
        lat = [1e3 * (r.t_done - (r.arrival if realtime else 0.0)) for r in order]
        return ServeStats(len(order), sum(r.n for r in order), t_end, lat, self._nbatches, self.device_bytes)


def device_loop(requests: list, realtime: bool = True, device=None) -> ServeStats:
    """The per-request baseline of PoolServer: for each request in arrival
    order, one apsep_run from its keys into its output (copying the answers
    to the host when out is host memory), then synchronise."""
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else torch.device(device).index or 0)
    nmax = max(r.n for r in requests)
    plans, scratch = {}, {}
    for r in requests:
        if r.kind not in plans:
            plans[r.kind] = Plan(nmax, r.keys.dtype, inclusive=r.inclusive, device=dev)
            scratch[r.kind] = (torch.empty(nmax, dtype=r.keys.dtype, device=dev),
                               torch.empty(nmax, dtype=torch.int32, device=dev))
    stream = torch.cuda.current_stream(dev)
    order = sorted(requests, key=lambda r: r.arrival if realtime else 0.0)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for r in order:
        if realtime:
            while time.perf_counter() - t0 < r.arrival:
                pass
        x, y = scratch[r.kind]
        keys = r.keys
        if not keys.is_cuda:
            x[:r.n].copy_(keys, non_blocking=True)
            keys = x[:r.n]
        if r.out is not None and r.out.is_cuda:
            plans[r.kind].run(keys, out=r.out[:r.n], n=r.n)
        else:
            plans[r.kind].run(keys, out=y[:r.n], n=r.n)
            if r.out is not None:
                r.out[:r.n].copy_(y[:r.n], non_blocking=True)
        stream.synchronize()
        r.t_done = time.perf_counter() - t0
    t_end = time.perf_counter() - t0
    for p in plans.values():
        p.check()
        p.close()
    lat = [1e3 * (r.t_done - (r.arrival if realtime else 0.0)) for r in order]
    return ServeStats(len(order), sum(r.n for r in order), t_end, lat, len(order), 0)
