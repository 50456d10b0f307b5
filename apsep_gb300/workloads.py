"""Seeded synthetic workloads of the batched and served forms.

batch_workload: S arrays with log-uniform lengths in [32, 2^20] (mean about
1e5 keys, 4.1e8 keys for S = 4096), int64 exclusive offsets; segment s holds
uniform keys in [0, 2^31) (s % 3 == 0), strictly descending runs of length
U[1, 4096] from random starts (s % 3 == 1), or the sawtooth k % 257
(s % 3 == 2).  Generated on the GPU from a seeded torch generator.

pool_requests: `count` requests with log-uniform lengths in [2^10, 2^24]
(mean about 1.7e6 keys), key type int32 / float32 50/50, Poisson arrivals at
`rate` per second.  int32 keys are uniform in [0, 2^31); float32 keys are
-1e6 + u * (2e6 / 2^24) with u uniform in [0, 2^24) (finite, exact).  Each
request owns its keys and its answer buffer: device memory (generated on the
GPU), or pinned host memory.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def segment_lengths(S: int, lo: int, hi: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(math.log(lo), math.log(hi), S))).astype(np.int64)


def _desc_runs(L: int, g: torch.Generator, device) -> torch.Tensor:
    rl = torch.randint(1, 4097, (L // 2048 + 2,), generator=g, device=device)
    while int(rl.sum()) < L:
        rl = torch.cat([rl, torch.randint(1, 4097, (L // 2048 + 2,), generator=g, device=device)])
    starts = torch.randint(4096, 1 << 30, (rl.numel(),), generator=g, device=device)
    rid = torch.repeat_interleave(torch.arange(rl.numel(), device=device), rl)[:L]
    first = torch.cumsum(rl, 0) - rl
    pos = torch.arange(L, device=device) - first[rid]
    return (starts[rid] - pos).to(torch.int32)


def batch_workload(S: int = 4096, seed: int = 7, device="cuda") -> tuple[torch.Tensor, np.ndarray]:
    """(keys on the device, offsets as a host int64 array of S + 1 entries)."""
    lengths = segment_lengths(S, 32, 1 << 20, seed)
    offs = np.zeros(S + 1, dtype=np.int64)
    offs[1:] = np.cumsum(lengths)
    n = int(offs[-1])
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    x = torch.empty(n, dtype=torch.int32, device=device)
    for s in range(S):
        a, b = int(offs[s]), int(offs[s + 1])
        L = b - a
        if L == 0:
            continue
        if s % 3 == 0:
            x[a:b] = torch.randint(0, 1 << 31, (L,), generator=g, device=device, dtype=torch.int64).to(torch.int32)
        elif s % 3 == 1:
            x[a:b] = _desc_runs(L, g, device)
        else:
            x[a:b] = (torch.arange(L, device=device) % 257).to(torch.int32)
    return x, offs


def pool_requests(count: int, rate: float, seed: int = 11, lo: int = 1 << 10, hi: int = 1 << 24,
                  device_keys: bool = True, device="cuda"):
    """The served workload for PoolServer: lengths log-uniform in [lo, hi],
    int32 / float32 50/50 (the value distributions above), Poisson
    arrivals at `rate` per second.  device_keys: every request owns its keys
    and its answer buffer in device memory (generated on the GPU); else the
    keys are pinned host slices and the answers go to pinned host buffers."""
    from .serve import Request

    rng = np.random.default_rng(seed)
    lengths = segment_lengths(count, lo, hi, seed + 1)
    gaps = rng.exponential(1.0 / rate, count) if rate > 0 else np.zeros(count)
    arrivals = np.cumsum(gaps)
    kinds = rng.random(count) < 0.5
    g = torch.Generator(device=device if device_keys else "cpu")
    g.manual_seed(seed)
    reqs = []
    for i in range(count):
        L = int(lengths[i])
        where = device if device_keys else "cpu"
        u = torch.randint(0, 1 << 31, (L,), generator=g, device=where, dtype=torch.int64)
        if kinds[i]:
            keys = u.to(torch.int32)
        else:
            keys = (-1e6 + (u & ((1 << 24) - 1)).to(torch.float64) * (2e6 / (1 << 24))).to(torch.float32)
        if device_keys:
            out = torch.empty(L, dtype=torch.int32, device=device)
        else:
            keys = keys.pin_memory()
            out = torch.empty(L, dtype=torch.int32).pin_memory()
        reqs.append(Request(rid=i, keys=keys, arrival=float(arrivals[i]), out=out))
    return reqs
