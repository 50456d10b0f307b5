"""Python host API over the C ABI (libapsep.so).

Mirrors the reference host interface (src/apsep.cuh) with the same meaning:

  alloc_spt_scratch(n)  -> Plan          allocSPTScratch<T,BS,IPT,INCL>(n)  apsep.cuh:3014-3040
  free_spt_scratch(s)                    freeSPTScratch(s)                  apsep.cuh:3042-3050
  run_spt(d_in, d_out, n, s)             runSPT  (async, no allocation)      apsep.cuh:3052-3067
  launch_spt(d_in, d_out, n)             launchSPT (alloc+run+sync+free)     apsep.cuh:3069-3076
  alloc_wstl_scratch / free_wstl_scratch / run_wstl / launch_wstl
                                         the WSTL names, apsep.cuh:2509-2605, on the same engine

Device buffers are torch CUDA tensors (plumbing only); runs go on the current
torch stream.  Errors raise ApsepError carrying the C status; n <= 0 is a
no-op as in the reference.  There is no CPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import ApsepError, PlanInfo  # noqa: F401

_DTYPES = {torch.int32: _lib.INT32, torch.float32: _lib.FLOAT32, torch.int64: _lib.INT64,
           torch.float64: _lib.FLOAT64}
_WIDE = (torch.int64, torch.float64)  # 8-byte keys: single arrays, one configuration


def _stream_handle(device: torch.device, stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream(device)
    return int(s.cuda_stream)


class Plan:
    """A run plan: device scratch for arrays of up to `capacity` keys."""

    def __init__(self, capacity: int, dtype: torch.dtype = torch.int32, inclusive: bool = False,
                 device=None, tuning="default"):
        """tuning: an autotune.Table (configuration per size class), "default"
        for the table shipped for GB300 when present, or None for the
        plan's fixed configuration (set_config)."""
        if dtype not in _DTYPES:
            raise TypeError("keys must be torch.int32, float32, int64 or float64, got %s" % dtype)
        self._lib = _lib.load()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.dtype = dtype
        self.inclusive = bool(inclusive)
        self.capacity = int(capacity)
        self._h = ctypes.c_void_p()
        self._cfg = 1 if dtype in _WIDE else 0
        if dtype in _WIDE:
            tuning = None  # one configuration for 8-byte keys
        if tuning == "default":
            from . import autotune
            tuning = autotune.load()
        self._tuning = tuning
        with torch.cuda.device(self.device):
            _lib.check(self._lib.apsep_plan_create(ctypes.byref(self._h), _DTYPES[dtype],
                                                   _lib.LE if inclusive else _lib.LT, self.capacity),
                       "apsep_plan_create")

    # -- reference-shaped accessors ------------------------------------------
    @property
    def handle(self) -> int:
        return self._h.value or 0

    def info(self) -> PlanInfo:
        inf = PlanInfo()
        _lib.check(self._lib.apsep_plan_get_info(self._h, ctypes.byref(inf)), "apsep_plan_get_info")
        return inf

    def set_config(self, config: int) -> None:
        """Fix the kernel configuration (turns per-size tuning off)."""
        _lib.check(self._lib.apsep_plan_set_config(self._h, int(config)), "apsep_plan_set_config")
        self._cfg = int(config)
        self._tuning = None

    def _tune_for(self, n: int) -> None:
        if self._tuning is None:
            return
        cfg = self._tuning.config_for(n, self.dtype)
        if cfg is not None and cfg != self._cfg:
            _lib.check(self._lib.apsep_plan_set_config(self._h, int(cfg)), "apsep_plan_set_config")
            self._cfg = cfg

    def run(self, x: torch.Tensor, out: torch.Tensor | None = None, n: int | None = None,
            inclusive: bool | None = None, stream=None) -> torch.Tensor:
        """Enqueue out[:n] = APSE(x[:n]) on the current (or given) stream."""
        if not x.is_cuda or x.dtype != self.dtype or not x.is_contiguous():
            raise ValueError("x must be a contiguous CUDA %s tensor" % self.dtype)
        n = x.numel() if n is None else int(n)
        if out is None:
            out = torch.empty(max(n, 0), dtype=torch.int32, device=x.device)
        if out.dtype != torch.int32 or not out.is_cuda or not out.is_contiguous():
            raise ValueError("out must be a contiguous CUDA int32 tensor")
        if n > x.numel() or n > out.numel():
            raise ValueError("n exceeds the buffers")
        incl = self.inclusive if inclusive is None else bool(inclusive)
        self._tune_for(n)
        st = self._lib.apsep_run_cmp(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     n, _lib.LE if incl else _lib.LT,
                                     ctypes.c_void_p(_stream_handle(x.device, stream)))
        _lib.check(st, "apsep_run")
        return out

    def run_segmented(self, x: torch.Tensor, offsets: torch.Tensor, out: torch.Tensor | None = None,
                      stream=None) -> torch.Tensor:
        """Enqueue a batched run: segment s is x[offsets[s]:offsets[s+1]]
        (offsets: CUDA int64, offsets[0] = 0, non-decreasing, offsets[-1] =
        x.numel()); out[i] is relative to the start of i's segment, -1 = none."""
        if not x.is_cuda or x.dtype != self.dtype or not x.is_contiguous():
            raise ValueError("x must be a contiguous CUDA %s tensor" % self.dtype)
        if (not offsets.is_cuda or offsets.dtype != torch.int64 or not offsets.is_contiguous()
                or offsets.numel() < 2):
            raise ValueError("offsets must be a contiguous CUDA int64 tensor of nseg + 1 >= 2 entries")
        n = x.numel()
        if out is None:
            out = torch.empty(n, dtype=torch.int32, device=x.device)
        if out.dtype != torch.int32 or not out.is_cuda or not out.is_contiguous() or out.numel() < n:
            raise ValueError("out must be a contiguous CUDA int32 tensor of x.numel() entries")
        self._tune_for(n)
        st = self._lib.apsep_run_segmented(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                           n, ctypes.c_void_p(offsets.data_ptr()), offsets.numel() - 1,
                                           ctypes.c_void_p(_stream_handle(x.device, stream)))
        _lib.check(st, "apsep_run_segmented")
        return out

    def workspace64_bytes(self, n: int) -> int:
        """Device workspace of run64 over n keys (-1: n out of range)."""
        return int(self._lib.apsep_run64_workspace_bytes(self._h, int(n)))

    def run64(self, x: torch.Tensor, out: torch.Tensor | None = None, inclusive: bool | None = None,
              work: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """Enqueue out = APSE(x) with int64 positions, for x of any length up
        to MAX_KEYS64: consecutive pieces of this plan's capacity, keys that
        their own piece does not answer answered from a hierarchy of minima
        over the keys before it (apsep_run64)."""
        if not x.is_cuda or x.dtype != self.dtype or not x.is_contiguous():
            raise ValueError("x must be a contiguous CUDA %s tensor" % self.dtype)
        n = x.numel()
        if out is None:
            out = torch.empty(n, dtype=torch.int64, device=x.device)
        if out.dtype != torch.int64 or not out.is_cuda or not out.is_contiguous() or out.numel() < n:
            raise ValueError("out must be a contiguous CUDA int64 tensor of x.numel() entries")
        need = self.workspace64_bytes(n)
        if need < 0:
            raise ValueError("n = %d is out of range for run64 on this plan" % n)
        if work is None:
            work = torch.empty(max(need, 16), dtype=torch.uint8, device=x.device)
        elif not work.is_cuda or work.numel() * work.element_size() < need:
            raise ValueError("work must be a CUDA buffer of at least %d bytes" % need)
        incl = self.inclusive if inclusive is None else bool(inclusive)
        st = self._lib.apsep_run64(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), n,
                                   _lib.LE if incl else _lib.LT, ctypes.c_void_p(work.data_ptr()),
                                   ctypes.c_void_p(_stream_handle(x.device, stream)))
        _lib.check(st, "apsep_run64")
        return out

    def check(self, stream=None) -> None:
        """Synchronise and raise on device-side errors of earlier runs."""
        _lib.check(self._lib.apsep_plan_check(self._h, ctypes.c_void_p(_stream_handle(self.device, stream))),
                   "apsep_plan_check")

    def error_async(self, host_word: torch.Tensor, stream=None) -> None:
        """Enqueue a copy of the plan's device-side error word into host_word
        (a pinned int32 host tensor of >= 1 element); nonzero once the stream
        has passed the copy means an earlier run failed (decode with check())."""
        if host_word.is_cuda or host_word.dtype != torch.int32 or host_word.numel() < 1:
            raise ValueError("host_word must be a pinned host int32 tensor")
        _lib.check(self._lib.apsep_plan_error_async(self._h, ctypes.c_void_p(host_word.data_ptr()),
                                                    ctypes.c_void_p(_stream_handle(self.device, stream))),
                   "apsep_plan_error_async")

    def debug_inject(self, range_index: int, spin_limit: int) -> None:
        """Fault injection: in the next run, range `range_index` never publishes."""
        _lib.check(self._lib.apsep_debug_inject(self._h, int(range_index), int(spin_limit)), "apsep_debug_inject")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.apsep_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


_cache: dict = {}


def apse(x: torch.Tensor, inclusive: bool = False, out: torch.Tensor | None = None) -> torch.Tensor:
    """One call: out[i] = max{j < i : x[j] < x[i]} (<= when inclusive), else -1."""
    if not x.is_cuda:
        raise ValueError("apse runs on CUDA tensors only (there is no CPU path)")
    x = x.contiguous()
    key = (x.device, x.dtype)
    plan = _cache.get(key)
    if plan is None or plan.capacity < x.numel():
        if plan is not None:
            plan.close()
        with torch.cuda.device(x.device):
            plan = Plan(max(x.numel(), 1 << 16), x.dtype, device=x.device)
        _cache[key] = plan
    return plan.run(x, out=out, inclusive=inclusive)


def apse_segmented(x: torch.Tensor, offsets: torch.Tensor, inclusive: bool = False,
                   out: torch.Tensor | None = None) -> torch.Tensor:
    """One call over a batch of back-to-back arrays (see Plan.run_segmented)."""
    if not x.is_cuda:
        raise ValueError("apse_segmented runs on CUDA tensors only (there is no CPU path)")
    x = x.contiguous()
    key = (x.device, x.dtype, bool(inclusive), "seg")
    plan = _cache.get(key)
    if plan is None or plan.capacity < x.numel():
        if plan is not None:
            plan.close()
        with torch.cuda.device(x.device):
            plan = Plan(max(x.numel(), 1 << 16), x.dtype, inclusive=inclusive, device=x.device)
        _cache[key] = plan
    return plan.run_segmented(x, offsets, out=out)


def apse64(x: torch.Tensor, inclusive: bool = False, out: torch.Tensor | None = None) -> torch.Tensor:
    """One call with int64 positions, for x of any length up to MAX_KEYS64
    (pieces of at most MAX_KEYS keys; see Plan.run64)."""
    if not x.is_cuda:
        raise ValueError("apse64 runs on CUDA tensors only (there is no CPU path)")
    x = x.contiguous()
    key = (x.device, x.dtype, "64")
    cap = min(max(x.numel(), 1 << 16), _lib.MAX_KEYS)
    plan = _cache.get(key)
    if plan is None or plan.capacity < cap:
        if plan is not None:
            plan.close()
        with torch.cuda.device(x.device):
            plan = Plan(cap, x.dtype, device=x.device)
        _cache[key] = plan
    return plan.run64(x, out=out, inclusive=inclusive)


# ---------------------------------------------------------------------------
# Reference-named mirror (src/apsep.cuh).  BLOCK_SIZE / IPT of the reference
# templates are tuning hints there; here the plan's autotuned configuration
# decides.  `inclusive` is the reference's INCL template argument.
# ---------------------------------------------------------------------------
def alloc_spt_scratch(n: int, dtype: torch.dtype = torch.int32, inclusive: bool = False) -> Plan:
    return Plan(max(int(n), 1), dtype, inclusive)


def free_spt_scratch(s: Plan) -> None:
    s.close()


def run_spt(d_in: torch.Tensor, d_out: torch.Tensor, n: int, s: Plan, inclusive: bool | None = None) -> None:
    if n <= 0:
        return
    s.run(d_in, out=d_out, n=n, inclusive=inclusive)


def launch_spt(d_in: torch.Tensor, d_out: torch.Tensor, n: int, inclusive: bool = False) -> None:
    if n <= 0:
        return
    with Plan(n, d_in.dtype, inclusive, device=d_in.device) as s:
        s.run(d_in, out=d_out, n=n)
        s.check()


alloc_wstl_scratch = alloc_spt_scratch
free_wstl_scratch = free_spt_scratch


def run_wstl(d_in: torch.Tensor, d_out: torch.Tensor, n: int, s: Plan) -> None:
    run_spt(d_in, d_out, n, s)


def launch_wstl(d_in: torch.Tensor, d_out: torch.Tensor, n: int) -> None:
    launch_spt(d_in, d_out, n)
