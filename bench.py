"""Benchmark: single-array APSE at N = 2^25 int32 keys on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload ("apse_single_2p25_int32"): one step is one APSE pass over one
2^25-key int32 array; the steps rotate over the four seeded distributions of
the N=2^25 configuration -- uniform in [0, 2^31), strictly descending,
strictly ascending, uniform in [0, 16) -- so every distribution is timed.
Metric: useful GB/s = 2 * N * 4 B / time (read the keys, write the answers),
aggregated over the timed steps; the per-distribution figures are reported
beside it.

  value      device time: CUDA events on the launching stream around each
             apsep_run, inputs resident in HBM; L2 is flushed before every
             step, outside the events: a 512 MiB buffer is written and then
             read, so no line of the inputs stays cached and no dirty line of
             the flush is left for the timed kernel to write back.
  per_distribution  median (with p10 / p90) device time per distribution,
             the median of the same steps back to back without the flush, and
             the steady state (us_steady, frac_steady): 20 runs of one
             distribution back to back between one pair of events, as the
             reference times its kernels.
  reference_published  the reference's published SPT figures at N = 2^25
             (one GTX 1660 Ti, per distribution) and ours over them:
             context only, other hardware.
  e2e        the same metric through the public API with host buffers: each
             step copies the keys from pinned host memory, runs, and copies
             the answers back, all inside the timed region.  value: the steps
             kept in flight (copy in / run / copy out on three streams, two
             device buffers each way; whole-loop time); serial: one step at a
             time on one stream, events around each step.
  roofline   achieved = algorithmic bytes per launch (8 B/key) / mean launch
             time (roofline.steady_state: the same from the steady-state
             times), against the measured HBM copy bandwidth
             (MEASURED_PEAKS.json); traffic = DRAM bytes per launch from the
             committed ncu summary (profiles/), when present.
  cpu_baseline  the sequential monotone-stack oracle on one host core over a
             bounded sample (every distribution, full size).

Multi-GPU (torchrun, one rank per GPU): the path does not shard, so every
rank runs independent replicas of the same workload ("weak" scaling); value
is all ranks' useful bytes over the slowest rank's time.

Extra objects on the same line (one GPU only; --no-extras skips them):
  batched    4096 arrays, log-uniform lengths in [32, 2^20] (4.1e8 keys), in
             one apsep_run_segmented launch vs a loop of one apsep_run per
             array on one stream, both replayed from CUDA graphs; useful
             bytes 8*sum(L) + 8*(S+1).
  served     the serving loop (apsep_gb300.serve.PoolServer, continuous
             batching over device-resident pools within an 8 GiB HBM budget):
             400 requests with log-uniform lengths in [2^10, 2^24], int32 /
             float32 50/50, keys in device memory, answers left in the pool.
             Saturated throughput against one apsep_run per request
             (synchronised), p50/p99 latency at a Poisson offered load of half
             the server's saturated rate, and 1 % of the requests checked
             against the CPU oracle.  served.host_keys: the same stream with
             keys and answers in pinned host memory (host-link bound; the
             link's rates in served.host_link).
  consumers  previous greater, next smaller, stock span, Cartesian parents and
             largest rectangle at N = 2^25 (apsep_gb300.consumers): time,
             useful GB/s and the fraction of peak of all their HBM passes.
  wide       8-byte keys (int64 / float64) at N = 2^25: time, useful GB/s
             (12 B/key) and fraction of peak.
  long64     int64 positions beyond 2^31 keys (Plan.run64): N = 2^32 int32
             keys in two pieces of 2^31 - 4096, uniform and descending; time,
             useful GB/s (12 B/key: 4 in, 8 out) and fraction of peak.
  le         the previous-smaller-or-equal comparator (INCL=true) at
             N = 2^25, the four distributions: time, GB/s, fraction.
  sweep      single-array useful GB/s and roofline fraction for N = 2^14 ..
             2^30 (every second power of two), uniform and descending keys.

--impl reference times the reference's sequential CPU algorithm (the oracle
port of cpuApsep, src/main.cu:102-113) on the host cores, all threads busy on
independent arrays, same workload, metric and units.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N = 1 << 25
DISTS = ("uniform", "descending", "ascending", "dup16")
METRIC = "useful GB/s at N=32M (frac. of HBM peak)"
UNIT = "GB/s"
WORKLOAD = "apse_single_2p25_int32"
STEADY_RUNS = 20


def make_inputs(n: int = N, seed: int = 20250325) -> dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    return {
        "uniform": rng.integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32),
        "descending": np.arange(n - 1, -1, -1, dtype=np.int32),
        "ascending": np.arange(n, dtype=np.int32),
        "dup16": rng.integers(0, 16, n).astype(np.int32),
    }


def useful_gbs(n: int, seconds: float, count: int = 1) -> float:
    return 2.0 * n * 4 * count / seconds / 1e9


def max_over_ranks(values: list, dist=None, device="cpu") -> list:
    """Each value's maximum over the ranks (the slowest replica's times)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def whole_job_gbs(n: int, slowest_ms: float, steps: int, world: int) -> float:
    """All ranks' useful bytes over the slowest rank's time (weak scaling: replicas)."""
    return useful_gbs(n, slowest_ms / 1e3, steps * world)


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic() -> dict | None:
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.isfile(p):
        with open(p) as f:
            return json.load(f)
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples: list[tuple[float, list[str]]] = []
        self.proc = None
        self.t = None
        self.window = (0.0, 0.0)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def wait_ready(self, timeout: float = 5.0) -> None:
        """Until the first sample arrives: nvidia-smi's start-up (driver
        attach) then lies outside the timed region, where it would stall a
        launch and stretch that step's event time."""
        t_end = time.time() + timeout
        while self.proc is not None and not self.samples and time.time() < t_end:
            time.sleep(0.01)

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.12)
        self.proc.terminate()
        try:
            self.proc.wait(2)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        t0, t1 = self.window
        inside = [s for ts, s in self.samples if t0 - 0.05 <= ts <= t1 + 0.05]
        used = inside if inside else [s for _, s in self.samples]

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(s[1]) for s in used if len(s) >= 9 and num(s[1]) is not None]
        mx = [num(s[2]) for s in used if len(s) >= 9 and num(s[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in used if len(s) >= 9 for i in range(4) if s[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(used), "window": "timed" if inside else "whole run"}


def cpu_baseline(inputs: dict[str, np.ndarray], reps: int = 2) -> dict:
    """The sequential oracle on one core: every distribution, full size."""
    import oracle
    oracle.build()
    times = []
    for _ in range(reps):
        for name in DISTS:
            t0 = time.perf_counter()
            oracle.apse(inputs[name])
            times.append(time.perf_counter() - t0)
    tot = sum(times)
    return {"value": round(useful_gbs(N, tot, len(times)), 3), "unit": UNIT, "cores": 1, "kind": "port",
            "nproc": os.cpu_count(),
            "sample": "%d passes: %d reps x {%s} at N=2^25 int32, one thread, %.1f s" %
                      (len(times), reps, ",".join(DISTS), tot)}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import concurrent.futures as cf

    import oracle
    oracle.build()
    inputs = make_inputs()
    threads = os.cpu_count() or 1
    for i in range(args.warmup):
        oracle.apse(inputs[DISTS[i % 4]])
    order = [DISTS[i % 4] for i in range(args.steps)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:  # ctypes releases the GIL
        list(ex.map(lambda d: oracle.apse(inputs[d]), order))
    wall = time.perf_counter() - t0
    value = useful_gbs(N, wall, args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(wall * 1e3 / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "i32",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": WORKLOAD, "n": N, "distributions": list(DISTS), "cmp": "<"},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d full-size passes on %d threads (independent arrays), sequential "
                                   "monotone stack restating cpuApsep" % (args.steps, threads)},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batched(dev) -> dict:
    """The batch of 4096 arrays in one segmented launch against a loop of one
    apsep_run per array.  Both are captured in CUDA graphs and timed by
    replaying them (device time, no host enqueue cost in either); the loop as
    enqueued from Python is reported beside them."""
    import torch

    from apsep_gb300 import Plan
    from apsep_gb300.workloads import batch_workload

    S = 4096
    x, offs = batch_workload(S, seed=7, device=dev)
    n = x.numel()
    d_off = torch.from_numpy(offs).to(dev)
    out = torch.empty(n, dtype=torch.int32, device=dev)
    plan = Plan(n, torch.int32, device=dev)
    useful = 8.0 * n + 8.0 * (S + 1)
    bounds = [(int(offs[i]), int(offs[i + 1])) for i in range(S) if offs[i + 1] > offs[i]]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def batched():
        plan.run_segmented(x, d_off, out=out)

    def loop():
        for a, b in bounds:
            plan.run(x[a:b], out=out[a:b])

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        plan.check()
        return ts

    side = torch.cuda.Stream(device=dev)
    graphs = {}
    for name, fn in (("batched", batched), ("loop", loop)):
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            fn()  # warm-up (plans pick their configurations; nothing is allocated in a run)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            fn()
        graphs[name] = g
    batched_ms = statistics.median(timed(graphs["batched"].replay, 7))
    loop_ms = min(timed(graphs["loop"].replay, 3))
    loop_py_ms = min(timed(loop, 2))
    plan.close()
    return {"workload": "batch_4096_loguniform_32_2p20_int32", "segments": S, "keys": n,
            "useful_bytes": int(useful), "batched_ms": round(batched_ms, 4), "loop_ms": round(loop_ms, 3),
            "loop_ms_python_enqueue": round(loop_py_ms, 3),
            "batched_gbs": round(useful / batched_ms / 1e6, 1), "loop_gbs": round(useful / loop_ms / 1e6, 2),
            "speedup_vs_loop": round(loop_ms / batched_ms, 2), "launches": {"batched": 1, "loop": len(bounds)},
            "note": "device time (CUDA events) of graph replays: the batch as one captured launch, the loop as "
                    "one captured graph of one apsep_run per array"}


def run_consumers(dev, peak_gbs: float) -> dict:
    """The consumers of APSE at N = 2^25 int32 (uniform keys; heights uniform
    in [0, 2^20) for the histogram), device time with L2 flushed.  useful GB/s
    counts the caller's bytes (keys in, answers out); pass_bytes counts every
    pass over HBM, workspace included, for the roofline."""
    import torch

    from apsep_gb300 import Plan, consumers

    n = 1 << 25
    g = torch.Generator(device=dev)
    g.manual_seed(31)
    x = torch.randint(-(1 << 31), 1 << 31, (n,), generator=g, device=dev, dtype=torch.int64).to(torch.int32)
    h = torch.randint(0, 1 << 20, (n,), generator=g, device=dev, dtype=torch.int32)
    plan = Plan(n, torch.int32, device=dev)
    work = torch.empty(consumers.workspace_bytes(n), dtype=torch.uint8, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ops = {  # name: (call, caller bytes per key, pass bytes per key)
        "prev_greater": (lambda: consumers.prev_greater(x, plan=plan, work=work), 8, 8),  # one flipped run
        "next_smaller": (lambda: consumers.next_smaller(x, plan=plan, work=work), 8, 8),  # one reversed run
        "stock_span": (lambda: consumers.stock_span(x, plan=plan, work=work), 8, 8),  # flipped run, span out
        # two runs (forward, reversed) of 8 B a key, then the parent pass: L, R, the
        # two keys compared (gathers) and the answer, 20 B
        "cartesian_parents": (lambda: consumers.cartesian_parents(x, plan=plan, work=work), 8, 36),
        # two runs of 8 B a key, then the area pass over h, L and R, 12 B
        "largest_rectangle": (lambda: consumers.largest_rectangle(h, plan=plan, work=work), 4, 28),
    }
    res = {}
    for name, (call, ub, pb) in ops.items():
        for _ in range(3):
            call()
        ts = []
        for _ in range(7):
            flush_l2(flush)
            e0.record()
            call()
            e1.record()
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        ms = statistics.median(ts)
        res[name] = {"us": round(ms * 1e3, 1), "useful_gbs": round(ub * n / ms / 1e6, 1),
                     "pass_bytes_per_key": pb, "pass_gbs": round(pb * n / ms / 1e6, 1),
                     "frac": round(pb * n / ms / 1e6 / peak_gbs, 4)}
    plan.check()
    plan.close()
    return {"workload": "consumers_2p25_int32", "n": n, "ops": res,
            "note": "largest_rectangle returns one int64 (its time includes the read back)"}


def run_wide(dev, peak_gbs: float) -> dict:
    """8-byte keys at N = 2^25 (int64: uniform over the full range, descending,
    ascending; float64 normal): device time with L2 flushed; useful bytes
    12 per key (8 in, 4 out)."""
    import torch

    from apsep_gb300 import Plan

    n = 1 << 25
    g = torch.Generator(device=dev)
    g.manual_seed(41)
    inputs = {
        "int64_uniform": torch.randint(-(1 << 62), 1 << 62, (n,), generator=g, device=dev, dtype=torch.int64),
        "int64_descending": torch.arange(n, 0, -1, device=dev, dtype=torch.int64) * (1 << 20),
        "int64_ascending": torch.arange(n, device=dev, dtype=torch.int64) * (1 << 20),
        "float64_normal": torch.randn(n, generator=g, device=dev, dtype=torch.float64),
    }
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    out = torch.empty(n, dtype=torch.int32, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res = {}
    plans = {torch.int64: Plan(n, torch.int64, device=dev), torch.float64: Plan(n, torch.float64, device=dev)}
    for name, x in inputs.items():
        plan = plans[x.dtype]
        for _ in range(3):
            plan.run(x, out=out)
        ts = []
        for _ in range(9):
            flush_l2(flush)
            e0.record()
            plan.run(x, out=out)
            e1.record()
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        plan.check()
        ms = statistics.median(ts)
        gbs = 12.0 * n / ms / 1e6
        res[name] = {"us": round(ms * 1e3, 1), "gbs": round(gbs, 1), "frac": round(gbs / peak_gbs, 4)}
    for p in plans.values():
        p.close()
    return {"workload": "wide_keys_2p25", "n": n, "bytes_per_key": 12, "runs": res}


def run_le(dev, peak_gbs: float) -> dict:
    """The previous-smaller-or-equal comparator (the reference's INCL=true,
    src/apsep.cuh:2669-2673) on the headline workload: N = 2^25 int32, the
    same four distributions, device time with L2 flushed, 8 useful B/key."""
    import torch

    from apsep_gb300 import Plan

    xs = {k: torch.from_numpy(v).to(dev) for k, v in make_inputs().items()}
    out = torch.empty(N, dtype=torch.int32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res = {}
    with Plan(N, torch.int32, inclusive=True, device=dev) as plan:
        for name, x in xs.items():
            for _ in range(3):
                plan.run(x, out=out)
            ts = []
            for _ in range(9):
                flush_l2(flush)
                e0.record()
                plan.run(x, out=out)
                e1.record()
                torch.cuda.synchronize(dev)
                ts.append(e0.elapsed_time(e1))
            plan.check()
            ms = statistics.median(ts)
            gbs = 8.0 * N / ms / 1e6
            res[name] = {"us": round(ms * 1e3, 1), "gbs": round(gbs, 1), "frac": round(gbs / peak_gbs, 4)}
    return {"workload": "apse_le_2p25_int32", "n": N, "bytes_per_key": 8, "runs": res}


def run_long64(dev, peak_gbs: float) -> dict:
    """int64 positions beyond 2^31 keys: N = 2^32 int32 keys through
    Plan.run64 on a plan of the largest capacity (two pieces), uniform and
    strictly descending over the whole int32 range; device time with L2
    flushed; useful bytes 12 per key (4 in, 8 out)."""
    import torch

    from apsep_gb300 import Plan, _lib

    n = 1 << 32
    plan = Plan(_lib.MAX_KEYS, torch.int32, device=dev, tuning=None)
    work = torch.empty(plan.workspace64_bytes(n), dtype=torch.uint8, device=dev)
    out = torch.empty(n, dtype=torch.int64, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g = torch.Generator(device=dev)
    g.manual_seed(43)
    res = {}
    for name in ("uniform", "descending"):
        if name == "uniform":
            x = torch.randint(0, (1 << 31) - 1, (n,), generator=g, device=dev, dtype=torch.int32)
        else:
            x = (torch.arange(n - 1, -1, -1, device=dev, dtype=torch.int64) - (1 << 31)).to(torch.int32)
        for _ in range(2):
            plan.run64(x, out=out, work=work)
        ts = []
        for _ in range(5):
            flush_l2(flush)
            e0.record()
            plan.run64(x, out=out, work=work)
            e1.record()
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        plan.check()
        ms = statistics.median(ts)
        gbs = 12.0 * n / ms / 1e6
        res[name] = {"ms": round(ms, 2), "gbs": round(gbs, 1), "frac": round(gbs / peak_gbs, 4)}
        del x
    plan.close()
    del out, work
    return {"workload": "positions64_2p32_int32", "n": n, "pieces": 2, "bytes_per_key": 12, "runs": res}


SERVE_REQUESTS = 400
SERVE_BATCH_KEYS = 1 << 27  # 128 Mi keys per launch at most
SERVE_SAMPLE_EVERY = 100    # 1 % of the requests are checked against the CPU oracle


def _served_stream(dev, device_keys: bool, rate: float, seed: int) -> dict:
    """One stream through PoolServer against device_loop: saturated (all at
    once) throughput of both, then p50/p99 at an offered load of half the
    server's saturated rate, and the sampled oracle check."""
    import oracle
    from apsep_gb300.serve import PoolServer, Request, device_loop
    from apsep_gb300.workloads import pool_requests

    reqs = pool_requests(SERVE_REQUESTS, rate=0.0, seed=seed, device_keys=device_keys, device=dev)
    if device_keys:  # answers stay in the pool; the sampled ones go to host memory
        sampled = {r.rid for r in reqs if r.rid % SERVE_SAMPLE_EVERY == 0}
        for r in reqs:
            r.out = torch_pinned_i32(r.n) if r.rid in sampled else None
    srv = PoolServer(budget_bytes=8 << 30, lanes_per_kind=2, max_batch_keys=SERVE_BATCH_KEYS, device=dev)
    try:
        srv.serve(reqs[:40], realtime=False)  # warm-up
        sat = max((srv.serve(reqs, realtime=False) for _ in range(3)), key=lambda st: st.requests_per_s)
        # the sampled requests' answers (the last saturated pass) against the oracle
        ok = True
        for r in reqs:
            if r.rid % SERVE_SAMPLE_EVERY == 0:
                k = r.keys.cpu().numpy() if r.keys.is_cuda else r.keys.numpy()
                ok = ok and not r.failed and bool((r.out[:r.n].cpu().numpy() == oracle.apse(k)).all())
        base = max((device_loop(reqs, realtime=False, device=dev) for _ in range(2)),
                   key=lambda st: st.requests_per_s)
        # the same requests arriving as a Poisson stream at half the saturated rate
        live_rate = 0.5 * sat.requests_per_s
        gaps = np.random.default_rng(seed + 1).exponential(1.0 / live_rate, len(reqs))
        live_reqs = [Request(rid=r.rid, keys=r.keys, arrival=float(t), out=None if device_keys else r.out)
                     for r, t in zip(reqs, np.cumsum(gaps))]
        live = srv.serve(live_reqs, realtime=True)
        failed = sum(r.failed for r in reqs) + sum(r.failed for r in live_reqs)
    finally:
        srv.close()
    return {"keys_in": "device" if device_keys else "pinned host", "pool_bytes": srv.device_bytes,
            "saturated": sat.as_dict(), "plain_loop_saturated": base.as_dict(),
            "throughput_vs_plain_loop": round(sat.requests_per_s / base.requests_per_s, 2),
            "offered_load_req_per_s": round(live_rate, 1), "at_offered_load": live.as_dict(),
            "sampled_requests": len(range(0, SERVE_REQUESTS, SERVE_SAMPLE_EVERY)), "sampled_bit_exact": ok,
            "failed_requests": int(failed)}


def torch_pinned_i32(n: int):
    import torch
    return torch.empty(n, dtype=torch.int32).pin_memory()


def host_link_gbs(dev) -> dict:
    """Pinned host <-> device copy rates of this machine (256 MiB each way)."""
    import torch
    h = torch.empty(1 << 26, dtype=torch.int32).pin_memory()
    d = torch.empty(1 << 26, dtype=torch.int32, device=dev)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    best = [0.0, 0.0]
    for _ in range(3):
        e[0].record()
        d.copy_(h, non_blocking=True)
        e[1].record()
        h.copy_(d, non_blocking=True)
        e[2].record()
        torch.cuda.synchronize(dev)
        best[0] = max(best[0], 2**28 / e[0].elapsed_time(e[1]) / 1e6)
        best[1] = max(best[1], 2**28 / e[1].elapsed_time(e[2]) / 1e6)
    return {"h2d_gbs": round(best[0], 1), "d2h_gbs": round(best[1], 1)}


def run_served(dev) -> dict:
    """The served request stream (PoolServer, continuous batching): 400
    requests, lengths log-uniform in [2^10, 2^24], int32 / float32 50/50, an
    8 GiB pool budget; keys and answers in device memory (the headline), and
    the same stream with keys and answers in pinned host memory (bound by the
    host link, whose rates are reported beside it)."""
    import torch

    dev_stream = _served_stream(dev, device_keys=True, rate=0.0, seed=21)
    torch.cuda.empty_cache()
    host_stream = _served_stream(dev, device_keys=False, rate=0.0, seed=41)
    torch.cuda.empty_cache()
    out = {"workload": "serve_loguniform_2p10_2p24_i32_f32", "budget_bytes": 8 << 30, "requests": SERVE_REQUESTS,
           "max_batch_keys": SERVE_BATCH_KEYS}
    out.update(dev_stream)
    out["host_keys"] = host_stream
    out["host_link"] = host_link_gbs(dev)
    out["note"] = ("wall clock on the host; throughput_vs_plain_loop: the same requests through one apsep_run each "
                   "(device_loop), synchronised after each")
    return out


def pipelined_e2e_ms(plan, pinned_in: dict, n: int, steps: int, dev) -> float:
    """Whole-loop time (ms) of `steps` host-to-host runs kept in flight: per
    step a pinned host -> device copy of that step's keys, apsep_run, and a
    device -> host copy of its answers, on three streams (copy in, run, copy
    out) with two device buffers each way; events order the reuse of each
    buffer.  Each step's copies are inside the timed region."""
    import torch

    s_in, s_run, s_out = (torch.cuda.Stream(device=dev) for _ in range(3))
    xs = [torch.empty(n, dtype=torch.int32, device=dev) for _ in range(2)]
    outs = [torch.empty(n, dtype=torch.int32, device=dev) for _ in range(2)]
    host_out = [torch.empty(n, dtype=torch.int32).pin_memory() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(steps)]
    ran = [torch.cuda.Event() for _ in range(steps)]
    read = [torch.cuda.Event() for _ in range(steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    t0.record(s_in)
    s_run.wait_event(t0)
    s_out.wait_event(t0)
    for i in range(steps):
        b = i % 2
        with torch.cuda.stream(s_in):
            if i >= 2:
                s_in.wait_event(ran[i - 2])  # the run two steps back has read xs[b]
            xs[b].copy_(pinned_in[DISTS[i % 4]], non_blocking=True)
            copied[i].record(s_in)
        s_run.wait_event(copied[i])
        if i >= 2:
            s_run.wait_event(read[i - 2])  # the copy out two steps back has read outs[b]
        plan.run(xs[b], out=outs[b], stream=s_run)
        ran[i].record(s_run)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ran[i])
            host_out[b].copy_(outs[b], non_blocking=True)
            read[i].record(s_out)
    s_out.wait_event(read[steps - 1])
    t1.record(s_out)
    torch.cuda.synchronize(dev)
    plan.check()
    return t0.elapsed_time(t1)


def flush_l2(buf) -> None:
    """Evict L2: write a buffer larger than L2, then read it back, so the next
    kernel finds neither its inputs cached nor dirty lines to write back."""
    import torch

    buf.zero_()
    buf.view(torch.int32).max()


def run_sweep(dev, peak_gbs: float) -> list:
    import torch

    from apsep_gb300 import Plan

    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    rows = []
    nmax = 1 << 30
    plan = Plan(nmax, torch.int32, device=dev)
    out = torch.empty(nmax, dtype=torch.int32, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for lg in range(14, 31, 2):
        n = 1 << lg
        for name in ("uniform", "descending"):
            if name == "uniform":
                x = torch.randint(0, 1 << 31, (n,), generator=g, device=dev, dtype=torch.int64).to(torch.int32)
            else:
                x = torch.arange(n - 1, -1, -1, device=dev, dtype=torch.int32)
            for _ in range(3):
                plan.run(x, out=out[:n])
            ts = []
            for _ in range(5 if lg < 28 else 3):
                flush_l2(flush)
                e0.record()
                plan.run(x, out=out[:n])
                e1.record()
                plan.check()
                ts.append(e0.elapsed_time(e1))
            ms = statistics.median(ts)
            gbs = useful_gbs(n, ms / 1e3)
            rows.append({"log2_n": lg, "dist": name, "us": round(ms * 1e3, 2), "gbs": round(gbs, 1),
                         "frac": round(gbs / peak_gbs, 4)})
            del x
    plan.close()
    del out
    return rows


def run_ours(args) -> None:
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from apsep_gb300 import Plan

    dev = torch.device("cuda", local)
    host = make_inputs(seed=20250325 + rank)
    d_in = {k: torch.from_numpy(v).to(dev) for k, v in host.items()}
    pinned_in = {k: torch.from_numpy(v).pin_memory() for k, v in host.items()}
    pinned_out = torch.empty(N, dtype=torch.int32).pin_memory()
    out = torch.empty(N, dtype=torch.int32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan = Plan(N, torch.int32, device=dev)

    def sanity(name):  # closed forms; no oracle on this path
        o = out
        if name == "ascending":
            assert bool((o[1:] == torch.arange(0, N - 1, device=dev, dtype=torch.int32)).all()) and int(o[0]) == -1
        elif name == "descending":
            assert bool((o == -1).all())

    for i in range(max(args.warmup, 3)):
        name = DISTS[i % 4]
        plan.run(d_in[name], out=out)
        plan.check()
        sanity(name)

    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
        sampler.wait_ready()
        time.sleep(0.2)
    flush_l2(flush)  # one more untimed step once the sampler runs
    plan.run(d_in[DISTS[0]], out=out)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.time()
    for i in range(args.steps):
        flush_l2(flush)
        ev[i][0].record(stream)
        plan.run(d_in[DISTS[i % 4]], out=out)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.time()
    if dist:
        dist.barrier()
    plan.check()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)

    # the same steps back to back without the flush (answers of the previous
    # step may still be dirty in L2; a 2^25 input is larger than L2 anyway)
    ev_u = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        ev_u[i][0].record(stream)
        plan.run(d_in[DISTS[i % 4]], out=out)
        ev_u[i][1].record(stream)
    torch.cuda.synchronize()
    plan.check()
    step_ms_unflushed = [a.elapsed_time(b) for a, b in ev_u]
    # steady state, as the reference times (src/main.cu:125-142): STEADY_RUNS runs of
    # one distribution back to back between one pair of events, no flush
    steady_ms = {}
    for name in DISTS:
        plan.run(d_in[name], out=out)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(STEADY_RUNS):
            plan.run(d_in[name], out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        steady_ms[name] = e0.elapsed_time(e1) / STEADY_RUNS
    plan.check()

    # e2e through the public API: pinned host -> device, run, device -> host.
    # (a) serial: one step at a time on one stream (L2 flushed before each);
    # (b) pipelined: the steps in flight on three streams with two device
    #     buffers each way, so step i's copy in, step i-1's run and step i-2's
    #     copy out overlap (the copies in both directions share the host link).
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    x_dev = torch.empty(N, dtype=torch.int32, device=dev)
    for i in range(args.steps):
        flush_l2(flush)
        ev2[i][0].record(stream)
        x_dev.copy_(pinned_in[DISTS[i % 4]], non_blocking=True)
        plan.run(x_dev, out=out)
        pinned_out.copy_(out, non_blocking=True)
        ev2[i][1].record(stream)
    torch.cuda.synchronize()
    plan.check()
    e2e_serial_ms = sum(a.elapsed_time(b) for a, b in ev2)
    e2e_ms = pipelined_e2e_ms(plan, pinned_in, N, args.steps, dev)

    total_ms, e2e_ms, e2e_serial_ms = max_over_ranks([total_ms, e2e_ms, e2e_serial_ms], dist, dev)
    clocks = {}
    if rank == 0:
        sampler.mark(t_wall0, t_wall1)
        clocks = sampler.stop()
    if dist:
        dist.barrier()
    if rank != 0:
        dist.destroy_process_group()
        return

    value = whole_job_gbs(N, total_ms, args.steps, world)
    per = {}
    for j, name in enumerate(DISTS):
        ms = sorted(step_ms[i] for i in range(args.steps) if i % 4 == j)
        mu = sorted(step_ms_unflushed[i] for i in range(args.steps) if i % 4 == j)
        if ms:
            pct = lambda v, q: v[min(len(v) - 1, int(q * (len(v) - 1) + 0.5))]
            per[name] = {"gbs": round(useful_gbs(N, statistics.median(ms) / 1e3), 1),
                         "us_median": round(statistics.median(ms) * 1e3, 2),
                         "us_p10": round(pct(ms, 0.1) * 1e3, 2), "us_p90": round(pct(ms, 0.9) * 1e3, 2),
                         "us_median_unflushed": round(statistics.median(mu) * 1e3, 2),
                         "us_steady": round(steady_ms[name] * 1e3, 2)}
    peaks = measured_peaks()
    mean_s = total_ms / 1e3 / args.steps
    achieved = 8.0 * N / mean_s / 1e9
    traffic = profile_traffic()
    for name in per:
        per[name]["frac"] = round(per[name]["gbs"] / peaks["hbm_gbs"], 4)
        per[name]["frac_steady"] = round(useful_gbs(N, per[name]["us_steady"] / 1e6) / peaks["hbm_gbs"], 4)
    steady_mean_s = sum(steady_ms.values()) / len(steady_ms) / 1e3
    steady_achieved = 8.0 * N / steady_mean_s / 1e9
    # The reference's only published numbers for this metric: SPT at N = 2^25 on one
    # GTX 1660 Ti (README.md:27-29), per distribution; other hardware, so context
    # only (vs_baseline stays null: no published figure for this aggregate on GB300).
    published = {"uniform": 98.2, "descending": 181.7, "ascending": 174.4}
    reference_published = {"hardware": "GTX 1660 Ti (288 GB/s)", "gbs": published,
                           "ours_over_published": {k: round(per[k]["gbs"] / v, 1)
                                                   for k, v in published.items() if k in per}}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "i32", "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": WORKLOAD, "n": N, "distributions": list(DISTS), "cmp": "<",
                   "l2": "flushed before every step (512 MiB written then read, outside the timed events)",
                   "parallelism": "replicas x%d" % world},
        "per_distribution": per,
        "reference_published": reference_published,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "peak_source": peaks["source"] + " (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_launch": 8 * N,
                     "traffic": traffic.get("bytes_per_launch") if traffic else None,
                     "traffic_source": traffic.get("source") if traffic else None,
                     "steady_state": {"achieved": round(steady_achieved, 1),
                                      "frac": round(steady_achieved / peaks["hbm_gbs"], 4),
                                      "how": "%d runs of each distribution back to back between one pair of "
                                             "CUDA events, no L2 flush; mean over the four" % STEADY_RUNS}},
        "e2e": {"value": round(whole_job_gbs(N, e2e_ms, args.steps, world), 2), "unit": UNIT,
                "h2d_bytes_per_step": 4 * N, "d2h_bytes_per_step": 4 * N, "form": "pipelined",
                "serial": round(whole_job_gbs(N, e2e_serial_ms, args.steps, world), 2)},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "wall_s_timed_region": round(t_wall1 - t_wall0, 4),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(host)
    if world == 1 and not args.no_extras:
        plan.close()
        del d_in, out, flush
        torch.cuda.empty_cache()
        legs = {"batched": lambda: run_batched(dev), "served": lambda: run_served(dev),
                "consumers": lambda: run_consumers(dev, peaks["hbm_gbs"]),
                "wide": lambda: run_wide(dev, peaks["hbm_gbs"]), "long64": lambda: run_long64(dev, peaks["hbm_gbs"]),
                "le": lambda: run_le(dev, peaks["hbm_gbs"]), "sweep": lambda: run_sweep(dev, peaks["hbm_gbs"])}
        for name in (args.extras.split(",") if args.extras else legs):
            line[name] = legs[name]()
            torch.cuda.empty_cache()
    print(json.dumps(line), flush=True)
    if world > 1 or args.no_extras:
        plan.close()
    if dist:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched / served / sweep objects")
    ap.add_argument("--extras", default="", help="comma-separated subset of the extra objects (default: all)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
