"""Serving loop: APSE requests as they arrive, batched into segmented runs.

    server = Server(budget_bytes=8 << 30)
    stats = server.serve(requests)        # requests: list[Request], arrival times in seconds
    stats.p50_ms, stats.p99_ms, stats.requests_per_s, stats.keys_per_s

Model.  A request is one array of host keys (int32 or float32, pinned for
asynchronous copies) with a comparator and an arrival time.  The server
keeps every device byte it touches in fixed, device-resident pools carved
out of an HBM byte budget at construction: per kind (key type x
comparator) `slots_per_kind` slots, each an input region, an answer region, a
segment-offset array and a plan whose scratch is sized for the slot.  The
loop admits arrived requests into a FIFO per kind; whenever a slot of that
kind is idle it takes the waiting requests, in arrival order, while their
keys fit the slot (admission by bytes: nothing is allocated per request), copies them
host -> device into consecutive segments, runs ONE apsep_run_segmented over
the batch, copies the answers back and records an event, all on the slot's
stream.  Slots of a kind alternate, so one batch's copies overlap another's
compute.  A request completes when its batch's event has fired; its latency
is completion minus arrival on the server clock.

`plain_loop` is the baseline the server is measured against: one request at
a time, copy in, apsep_run, copy out, synchronise.

Device-resident requests (`ResidentServer`): when the keys are produced on
the GPU (or uploaded by the client ahead of time), the pool is a ring of
keys and answers in HBM that requests occupy in arrival order, each in a
slot of whole 4-key units (16-byte aligned starts, so every launch streams
through TMA from its first tile).  A batch is a contiguous span of arrived
requests and runs in place, one segmented launch with no copies;
`resident_loop` is its per-request baseline (one apsep_run per request on the
same memory, synchronised).
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np
import torch

from .api import Plan


@dataclasses.dataclass
class Request:
    rid: int
    keys: torch.Tensor            # host keys, int32 or float32 (pinned for overlap)
    arrival: float = 0.0          # seconds after serve() starts
    inclusive: bool = False       # <= instead of <
    answers: np.ndarray | None = None  # filled when keep_answers
    t_done: float | None = None

    @property
    def kind(self) -> tuple:
        return (self.keys.dtype, bool(self.inclusive))

    @property
    def n(self) -> int:
        return int(self.keys.numel())


class BatchPlanner:
    """Admission policy (host only): from a FIFO of waiting requests, the
    longest prefix whose keys fit `capacity_keys` in at most `max_segments`
    segments.  A request larger than a slot can never be admitted; submit
    rejects it."""

    def __init__(self, capacity_keys: int, max_segments: int):
        self.capacity_keys = int(capacity_keys)
        self.max_segments = int(max_segments)

    def fits(self, n: int) -> bool:
        return 0 <= n <= self.capacity_keys

    def take(self, waiting: collections.deque) -> list:
        batch, keys = [], 0
        while waiting and len(batch) < self.max_segments and keys + waiting[0].n <= self.capacity_keys:
            r = waiting.popleft()
            batch.append(r)
            keys += r.n
        return batch


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


class _Slot:
    def __init__(self, kind, capacity_keys: int, max_segments: int, device):
        dtype, incl = kind
        self.kind = kind
        self.keys_in = torch.empty(capacity_keys, dtype=dtype, device=device)
        self.answers = torch.empty(capacity_keys, dtype=torch.int32, device=device)
        self.offs = torch.empty(max_segments + 1, dtype=torch.int64, device=device)
        self.offs_host = torch.empty(max_segments + 1, dtype=torch.int64).pin_memory()
        self.answers_host = torch.empty(capacity_keys, dtype=torch.int32).pin_memory()
        self.plan = Plan(capacity_keys, dtype, inclusive=incl, device=device)
        self.stream = torch.cuda.Stream(device=device)
        self.event = torch.cuda.Event()
        self.batch: list = []
        self.spans: list = []

    def device_bytes(self) -> int:
        return (self.keys_in.numel() * 4 + self.answers.numel() * 4 + self.offs.numel() * 8 +
                int(self.plan.info().scratch_bytes))

    def close(self):
        self.plan.close()


def slot_bytes_per_key() -> float:
    """Device bytes one slot needs per key of capacity (keys, answers, plan scratch)."""
    with Plan(1 << 20, torch.int32, tuning=None) as p:
        scratch = int(p.info().scratch_bytes)
    return 8.0 + scratch / float(1 << 20)


class Server:
    def __init__(self, budget_bytes: int = 8 << 30, slot_keys: int | None = None, slots_per_kind: int = 2,
                 max_segments: int = 4096, kinds=((torch.int32, False), (torch.float32, False)), device=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.kinds = [(k[0], bool(k[1])) for k in kinds]
        nslots = slots_per_kind * len(self.kinds)
        per_key = slot_bytes_per_key()
        fit = int((budget_bytes / nslots - 8 * (max_segments + 1)) / per_key)
        cap = fit if slot_keys is None else min(int(slot_keys), fit)
        if cap < 1:
            raise ValueError("budget of %d bytes leaves no room for %d slots" % (budget_bytes, nslots))
        self.budget_bytes = int(budget_bytes)
        self.planner = BatchPlanner(cap, max_segments)
        self.slots = {k: [_Slot(k, cap, max_segments, self.device) for _ in range(slots_per_kind)]
                      for k in self.kinds}
        self.device_bytes = sum(s.device_bytes() for ss in self.slots.values() for s in ss)
        if self.device_bytes > self.budget_bytes:
            raise RuntimeError("pools (%d bytes) exceed the budget (%d bytes)" % (self.device_bytes, budget_bytes))

    @property
    def slot_keys(self) -> int:
        return self.planner.capacity_keys

    def close(self):
        for ss in self.slots.values():
            for s in ss:
                s.close()

    def _launch(self, slot: _Slot, batch: list) -> None:
        slot.batch = batch
        slot.spans = []
        offs = [0]
        with torch.cuda.stream(slot.stream):
            for r in batch:
                a = offs[-1]
                slot.keys_in[a:a + r.n].copy_(r.keys, non_blocking=True)
                slot.spans.append((a, a + r.n))
                offs.append(a + r.n)
            total = offs[-1]
            ns = len(batch)
            slot.offs_host[:ns + 1] = torch.tensor(offs, dtype=torch.int64)
            slot.offs[:ns + 1].copy_(slot.offs_host[:ns + 1], non_blocking=True)
            slot.plan.run_segmented(slot.keys_in[:total], slot.offs[:ns + 1], out=slot.answers[:total],
                                    stream=slot.stream)
            slot.answers_host[:total].copy_(slot.answers[:total], non_blocking=True)
            slot.event.record(slot.stream)

    def _retire(self, slot: _Slot, now: float, keep_answers: bool) -> None:
        for r, (a, b) in zip(slot.batch, slot.spans):
            r.t_done = now
            if keep_answers:
                r.answers = slot.answers_host[a:b].numpy().copy()
        slot.batch = []
        slot.spans = []

    def serve(self, requests: list, keep_answers: bool = False, realtime: bool = True) -> ServeStats:
        """Run the loop until every request completes.  realtime=False makes
        every request arrive at once (saturation throughput)."""
        for r in requests:
            if r.kind not in self.slots:
                raise ValueError("no pool for keys of %s (inclusive=%s)" % r.kind)
            if not self.planner.fits(r.n):
                raise ValueError("request %d (%d keys) exceeds a slot (%d keys)" % (r.rid, r.n, self.slot_keys))
        order = sorted(requests, key=lambda r: r.arrival if realtime else 0.0)
        waiting = {k: collections.deque() for k in self.kinds}
        nxt = 0
        done = 0
        batches = 0
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        while done < len(order):
            now = time.perf_counter() - t0
            while nxt < len(order) and (not realtime or order[nxt].arrival <= now):
                waiting[order[nxt].kind].append(order[nxt])
                nxt += 1
            progressed = False
            for k, ss in self.slots.items():
                for s in ss:
                    if s.batch and s.event.query():
                        done += len(s.batch)
                        self._retire(s, time.perf_counter() - t0, keep_answers)
                        progressed = True
                    if not s.batch and waiting[k]:
                        batch = self.planner.take(waiting[k])
                        if batch:
                            self._launch(s, batch)
                            batches += 1
                            progressed = True
            if not progressed:
                time.sleep(0)
        t_end = time.perf_counter() - t0
        for ss in self.slots.values():
            for s in ss:
                s.plan.check(stream=s.stream)
        lat = [1e3 * (r.t_done - (r.arrival if realtime else 0.0)) for r in order]
        return ServeStats(len(order), sum(r.n for r in order), t_end, lat, batches, self.device_bytes)


def plain_loop(requests: list, keep_answers: bool = False, realtime: bool = True, device=None) -> ServeStats:
    """The baseline: one request at a time -- copy in, apsep_run, copy out, synchronise."""
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else torch.device(device).index or 0)
    nmax = max(r.n for r in requests)
    plans, bufs = {}, {}
    for r in requests:
        if r.kind not in plans:
            plans[r.kind] = Plan(nmax, r.keys.dtype, inclusive=r.inclusive, device=dev)
            bufs[r.kind] = (torch.empty(nmax, dtype=r.keys.dtype, device=dev),
                            torch.empty(nmax, dtype=torch.int32, device=dev))
    host_out = torch.empty(nmax, dtype=torch.int32).pin_memory()
    stream = torch.cuda.current_stream(dev)
    order = sorted(requests, key=lambda r: r.arrival if realtime else 0.0)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for r in order:
        if realtime:
            while time.perf_counter() - t0 < r.arrival:
                pass
        x, y = bufs[r.kind]
        x[:r.n].copy_(r.keys, non_blocking=True)
        plans[r.kind].run(x[:r.n], out=y[:r.n])
        host_out[:r.n].copy_(y[:r.n], non_blocking=True)
        stream.synchronize()
        r.t_done = time.perf_counter() - t0
        if keep_answers:
            r.answers = host_out[:r.n].numpy().copy()
    t_end = time.perf_counter() - t0
    for p in plans.values():
        p.check()
        p.close()
    lat = [1e3 * (r.t_done - (r.arrival if realtime else 0.0)) for r in order]
    return ServeStats(len(order), sum(r.n for r in order), t_end, lat, len(order), 0)


# ---------------------------------------------------------------------------
# Device-resident requests
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class ResidentRequest:
    rid: int
    start: int            # first key in the ring
    n: int
    arrival: float = 0.0
    t_done: float | None = None


RESIDENT_SLOT_KEYS = 4  # ring slots are whole 4-key (16-byte) units


class ResidentServer:
    """Requests whose keys already sit in a device ring (in arrival order).

    keys/answers: the ring (device tensors of equal length); requests must
    not wrap.  Each request occupies a slot of whole RESIDENT_SLOT_KEYS units
    (it starts on a 16-byte boundary of the ring, so every batch does and its
    launch streams through TMA from its first tile); the up to 3 keys between a
    request's end and
    the next slot must hold padding that never qualifies as an answer
    (INT_MAX / +inf).  Each batch is the longest run of arrived, waiting
    requests that fits `max_batch_keys` and `max_segments`, launched in place:
    a request's segment also spans the padding after it, whose answers land in
    the matching gap of `answers`."""

    def __init__(self, keys: torch.Tensor, answers: torch.Tensor, inclusive: bool = False,
                 max_batch_keys: int = 64 << 20, max_segments: int = 4096, streams: int = 2,
                 budget_bytes: int = 8 << 30):
        self.keys, self.answers = keys, answers
        self.device = keys.device
        self.max_batch_keys = int(min(max_batch_keys, keys.numel()))
        self.max_segments = int(max_segments)
        # the ring plus each lane's plan must fit the HBM budget
        need = keys.numel() * 8 + streams * (self.max_batch_keys * (slot_bytes_per_key() - 8.0) +
                                             8 * (max_segments + 1))
        if need > budget_bytes:
            raise ValueError("ring and plans need %d bytes, over the budget of %d" % (need, budget_bytes))
        self.device_bytes = int(need)
        self.lanes = []
        for _ in range(streams):
            self.lanes.append({"stream": torch.cuda.Stream(device=self.device), "event": torch.cuda.Event(),
                               "offs": torch.empty(max_segments + 1, dtype=torch.int64, device=self.device),
                               "offs_host": torch.empty(max_segments + 1, dtype=torch.int64).pin_memory(),
                               "plan": Plan(min(int(max_batch_keys), keys.numel()), keys.dtype,
                                            inclusive=inclusive, device=self.device),
                               "batch": []})

    def close(self):
        for ln in self.lanes:
            ln["plan"].close()

    def _launch(self, ln, batch):
        base = batch[0].start
        offs = [r.start - base for r in batch]
        total = batch[-1].start + batch[-1].n - base
        offs.append(total)
        ns = len(batch)
        ln["batch"] = batch
        with torch.cuda.stream(ln["stream"]):
            ln["offs_host"][:ns + 1] = torch.tensor(offs, dtype=torch.int64)
            ln["offs"][:ns + 1].copy_(ln["offs_host"][:ns + 1], non_blocking=True)
            ln["plan"].run_segmented(self.keys[base:base + total], ln["offs"][:ns + 1],
                                     out=self.answers[base:base + total], stream=ln["stream"])
            ln["event"].record(ln["stream"])

    def serve(self, requests: list, realtime: bool = True) -> ServeStats:
        order = sorted(requests, key=lambda r: r.start)
        for r in order:
            if r.start % RESIDENT_SLOT_KEYS:
                raise ValueError("resident requests must start on a %d-key boundary of the ring" % RESIDENT_SLOT_KEYS)
        for a, b in zip(order, order[1:]):
            if not 0 <= b.start - (a.start + a.n) < RESIDENT_SLOT_KEYS:
                raise ValueError("resident requests must fill consecutive slots of the ring, in arrival order")
        nxt = done = batches = 0
        waiting = collections.deque()
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        while done < len(order):
            now = time.perf_counter() - t0
            while nxt < len(order) and (not realtime or order[nxt].arrival <= now):
                waiting.append(order[nxt])
                nxt += 1
            progressed = False
            for ln in self.lanes:
                if ln["batch"] and ln["event"].query():
                    t = time.perf_counter() - t0
                    for r in ln["batch"]:
                        r.t_done = t
                    done += len(ln["batch"])
                    ln["batch"] = []
                    progressed = True
                if not ln["batch"] and waiting:
                    batch, keys = [], 0
                    while (waiting and len(batch) < self.max_segments and
                           (not batch or keys + waiting[0].n <= self.max_batch_keys)):
                        r = waiting.popleft()
                        batch.append(r)
                        keys += r.n
                    self._launch(ln, batch)
                    batches += 1
                    progressed = True
            if not progressed:
                time.sleep(0)
        t_end = time.perf_counter() - t0
        for ln in self.lanes:
            ln["plan"].check(stream=ln["stream"])
        lat = [1e3 * (r.t_done - (r.arrival if realtime else 0.0)) for r in order]
        return ServeStats(len(order), sum(r.n for r in order), t_end, lat, batches, self.device_bytes)


def resident_loop(keys: torch.Tensor, answers: torch.Tensor, requests: list, inclusive: bool = False,
                  realtime: bool = True) -> ServeStats:
    """The per-request baseline on device-resident keys: apsep_run, synchronise."""
    nmax = max(r.n for r in requests)
    plan = Plan(nmax, keys.dtype, inclusive=inclusive, device=keys.device)
    stream = torch.cuda.current_stream(keys.device)
    order = sorted(requests, key=lambda r: r.arrival if realtime else 0.0)
    torch.cuda.synchronize(keys.device)
    t0 = time.perf_counter()
    for r in order:
        if realtime:
            while time.perf_counter() - t0 < r.arrival:
                pass
        plan.run(keys[r.start:r.start + r.n], out=answers[r.start:r.start + r.n])
        stream.synchronize()
        r.t_done = time.perf_counter() - t0
    t_end = time.perf_counter() - t0
    plan.check()
    plan.close()
    lat = [1e3 * (r.t_done - (r.arrival if realtime else 0.0)) for r in order]
    return ServeStats(len(order), sum(r.n for r in order), t_end, lat, len(order), 0)
