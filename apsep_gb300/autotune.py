"""Autotuner: the kernel configuration per size class, measured on this GPU.

The engine has one tunable knob, the kernel configuration: warps per CTA
{4, 8, 16} x keys per lane {8, 16} (`apsep_num_configs()` of them; 32 keys per
lane would double the in-lane compare ladder's cost per key, and there is no
cluster dimension: ranges are warp-independent).  A size class is floor(log2(n)); the tuner
times every configuration on seeded synthetic arrays of that size (uniform,
descending and ascending keys, the single-array benchmark's inputs; the runs
replayed from a CUDA graph, so device time without host enqueue cost), keeps
the one with the lowest total time, and stores {class: config} in a table.  A
Plan (or apse / the server) given a table picks the configuration per call:

    table = autotune.tune(dtype=torch.int32, classes=range(14, 27))
    autotune.save(table, "tuning.json")
    plan = Plan(n, torch.int32, tuning=autotune.load("tuning.json"))

The package ships the table measured on GB300 (tuning_gb300.json), used by
default when present.
"""
from __future__ import annotations

import json
import os

import torch

from . import _lib

DEFAULT_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json")


def size_class(n: int) -> int:
    return max(int(n), 1).bit_length() - 1


def num_configs() -> int:
    return int(_lib.load().apsep_num_configs())


def config_shape(config: int) -> tuple[int, int]:
    import ctypes
    t, k = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(_lib.load().apsep_config_shape(int(config), ctypes.byref(t), ctypes.byref(k)), "apsep_config_shape")
    return int(t.value), int(k.value)


class Table:
    """{size class: configuration} (for int32 keys, and per other key type in
    `by_dtype`); classes outside the table use the nearest one.  `timings`
    keeps the measured microseconds per run of every configuration."""

    def __init__(self, entries: dict[int, int], device_name: str = "", by_dtype: dict | None = None,
                 timings: dict | None = None):
        self.entries = {int(k): int(v) for k, v in entries.items()}
        self.device_name = device_name
        self.by_dtype = {str(d): {int(k): int(v) for k, v in e.items()} for d, e in (by_dtype or {}).items()}
        self.timings = timings or {}

    def config_for(self, n: int, dtype=None) -> int | None:
        name = str(dtype).replace("torch.", "") if dtype is not None else "int32"
        entries = self.by_dtype.get(name) or self.entries
        if not entries:
            return None
        c = size_class(n)
        best = min(entries, key=lambda k: (abs(k - c), k))
        return entries[best]

    def to_json(self) -> dict:
        d = {"device": self.device_name, "classes": {str(k): v for k, v in sorted(self.entries.items())}}
        if self.by_dtype:
            d["by_dtype"] = {t: {str(k): v for k, v in sorted(e.items())} for t, e in self.by_dtype.items()}
        if self.timings:
            d["timings_us"] = self.timings
        return d

    @staticmethod
    def from_json(d: dict) -> "Table":
        return Table({int(k): int(v) for k, v in d.get("classes", {}).items()}, d.get("device", ""),
                     d.get("by_dtype"), d.get("timings_us"))


def save(table: Table, path: str) -> None:
    with open(path, "w") as f:
        json.dump(table.to_json(), f, indent=1)


def load(path: str = DEFAULT_TABLE) -> Table | None:
    if not os.path.isfile(path):
        return None
    with open(path) as f:
        return Table.from_json(json.load(f))


def _inputs(n: int, dtype: torch.dtype, device) -> list[torch.Tensor]:
    g = torch.Generator(device=device)
    g.manual_seed(1000 + n)
    uni = torch.randint(0, 1 << 31, (n,), generator=g, device=device, dtype=torch.int64)
    xs = [uni.to(torch.int32), torch.arange(n - 1, -1, -1, device=device, dtype=torch.int32),
          torch.arange(n, device=device, dtype=torch.int32)]
    if dtype == torch.float32:
        xs = [x.to(torch.float32) for x in xs]
    return xs


def tune(dtype: torch.dtype = torch.int32, classes=range(14, 27), reps: int = 5, inclusive: bool = False,
         device=None, verbose: bool = False) -> Table:
    """Time every configuration at n = 2^class for each class; returns the table."""
    from .api import Plan

    dev = torch.device("cuda", torch.cuda.current_device() if device is None else torch.device(device).index or 0)
    classes = list(classes)
    nmax = 1 << max(classes)
    plan = Plan(nmax, dtype, inclusive=inclusive, device=dev)
    out = torch.empty(nmax, dtype=torch.int32, device=dev)
    entries, timings = {}, {}
    try:
        for c in classes:
            n = 1 << c
            xs = _inputs(n, dtype, dev)
            best, best_t = 0, float("inf")
            per = {}
            for cfg in range(num_configs()):
                plan.set_config(cfg)
                # the runs replayed from a CUDA graph: device time, without the
                # host's enqueue cost (which alone exceeds a small array's run)
                side = torch.cuda.Stream(device=dev)
                side.wait_stream(torch.cuda.current_stream(dev))
                with torch.cuda.stream(side):
                    for x in xs:  # warm-up (first launches set kernel attributes)
                        plan.run(x, out=out[:n])
                torch.cuda.synchronize(dev)
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph, stream=side):
                    for _ in range(reps):
                        for x in xs:
                            plan.run(x, out=out[:n])
                graph.replay()
                torch.cuda.synchronize(dev)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                graph.replay()
                e1.record()
                plan.check()
                del graph
                t = e0.elapsed_time(e1)
                per[cfg] = t * 1e3 / (reps * len(xs))
                if verbose:
                    print("class %d config %d: %.1f us per run" % (c, cfg, t * 1e3 / (reps * len(xs))))
                if t < best_t:
                    best, best_t = cfg, t
            entries[c] = best
            timings[str(c)] = {str(k): round(v, 2) for k, v in per.items()}
    finally:
        plan.close()
    return Table(entries, torch.cuda.get_device_name(dev), timings={str(dtype).replace("torch.", ""): timings})


def tune_all(classes=range(14, 31), reps: int = 5, device=None, verbose: bool = False) -> Table:
    """tune() for int32 and float32 keys; one table (int32 entries as the default)."""
    t_i = tune(torch.int32, classes, reps, device=device, verbose=verbose)
    t_f = tune(torch.float32, classes, reps, device=device, verbose=verbose)
    return Table(t_i.entries, t_i.device_name, by_dtype={"float32": t_f.entries},
                 timings={**t_i.timings, **t_f.timings})
