"""Minimal profiling target (the role of the reference's src/profile_bottleneck.cu).

    python -m apsep_gb300.profile_target [--dist uniform|descending|ascending|dup16]
                                         [--n 33554432] [--reps 3] [--config 0]
                                         [--dtype int32|float32|int64|float64]
                                         [--piece KEYS] [--batch SEGMENTS]

Allocates one input and one output ((4 or 8) * n + 4 * n bytes), runs `reps` APSE
launches with a synchronisation after each, prints the last launch's time.
With --piece, each rep is one Plan.run64 (int64 positions, 8 * n bytes of
answers) on a plan of that capacity, so the array runs as pieces of that
many keys (engine run + fix-up pass per piece).  With --batch S, each rep is
one segmented run of the batch workload with S segments (log-uniform lengths
in [32, 2^20]; --dist mixed: its uniform / descending-run / sawtooth
segments; --dist uniform: the same lengths filled with uniform keys).
Small enough on the device for ncu captures; n = 2^25 keeps the 128 MiB
input above the 126 MiB L2.
"""
from __future__ import annotations

import argparse

import numpy as np
import torch

from apsep_gb300 import Plan


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--dist", default="uniform", choices=("uniform", "descending", "ascending", "dup16", "mixed"))
    ap.add_argument("--n", type=int, default=1 << 25)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--config", type=int, default=0)
    ap.add_argument("--dtype", default="int32", choices=("int32", "float32", "int64", "float64"))
    ap.add_argument("--piece", type=int, default=0)
    ap.add_argument("--batch", type=int, default=0)
    a = ap.parse_args()
    if a.batch:
        batch_main(a)
        return
    rng = np.random.default_rng(7)
    n = a.n
    if a.dist == "uniform":
        h = rng.integers(0, 1 << 31, n, dtype=np.int64)
    elif a.dist == "descending":
        h = np.arange(n - 1, -1, -1, dtype=np.int64)
    elif a.dist == "ascending":
        h = np.arange(n, dtype=np.int64)
    else:
        h = rng.integers(0, 16, n)
    dt = getattr(torch, a.dtype)
    x = torch.from_numpy(h.astype(getattr(np, a.dtype))).cuda()
    if a.piece:
        plan = Plan(a.piece, dt, tuning=None)
        out = torch.empty(n, dtype=torch.int64, device="cuda")
        work = torch.empty(max(plan.workspace64_bytes(n), 16), dtype=torch.uint8, device="cuda")

        def run():
            plan.run64(x, out=out, work=work)
    else:
        out = torch.empty(n, dtype=torch.int32, device="cuda")
        plan = Plan(n, dt)

        def run():
            plan.run(x, out=out)
    if dt in (torch.int32, torch.float32):
        plan.set_config(a.config)  # (8-byte keys have one configuration)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(a.reps):
        torch.cuda._sleep(200000)  # keep the stream busy so launch overhead stays off the clock
        e0.record()
        run()
        e1.record()
        plan.check()
        times.append(e0.elapsed_time(e1) * 1e3)
    t = sorted(times[1:] if len(times) > 1 else times)
    med = t[len(t) // 2]
    kb = x.element_size()
    print("done dist=%s dtype=%s n=%d median=%.1f us min=%.1f max=%.1f (%.1f GB/s useful at the median)"
          % (a.dist, a.dtype, n, med, t[0], t[-1], (kb + out.element_size()) * n / (med * 1e-6) / 1e9))
    plan.close()


def batch_main(a) -> None:
    from apsep_gb300.workloads import batch_workload

    x, offs = batch_workload(a.batch, seed=7)
    if a.dist == "uniform":
        g = torch.Generator(device="cuda")
        g.manual_seed(1)
        x = torch.randint(0, 1 << 31, (x.numel(),), generator=g, device="cuda", dtype=torch.int64).to(torch.int32)
    elif a.dist != "mixed":
        raise SystemExit("--batch takes --dist mixed or uniform")
    n = x.numel()
    d_offs = torch.from_numpy(offs).cuda()
    plan = Plan(n, torch.int32)
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(a.reps):
        torch.cuda._sleep(200000)
        e0.record()
        plan.run_segmented(x, d_offs, out=out)
        e1.record()
        plan.check()
        times.append(e0.elapsed_time(e1) * 1e3)
    t = sorted(times[1:] if len(times) > 1 else times)
    print("done batch=%d dist=%s n=%d median=%.1f us" % (a.batch, a.dist, n, t[len(t) // 2]))
    plan.close()


if __name__ == "__main__":
    main()
