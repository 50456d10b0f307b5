"""Consumers of APSE: previous greater, next smaller, stock span, largest
rectangle in a histogram, Cartesian-tree parents (the callers the
reference names for its output, README.md:3, src/bench_spt_le.cu:1-3).

Each is one libapsep.so call (apsep_run_prev_greater, apsep_run_next_smaller,
apsep_stock_span, apsep_largest_rectangle, apsep_cartesian_parents): a few
memory-bound passes around one or two engine runs on a plan, with a device
workspace.  Pass `plan` (and `work`, apsep_consumer_workspace_bytes(n) bytes,
16-byte aligned) to keep a loop allocation-free; otherwise both are made per
call.  CUDA tensors only: there is no CPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .api import Plan, _stream_handle


def workspace_bytes(n: int) -> int:
    return int(_lib.load().apsep_consumer_workspace_bytes(int(n)))


def _prep(x: torch.Tensor, plan: Plan | None, work: torch.Tensor | None):
    if not x.is_cuda or x.dtype not in (torch.int32, torch.float32, torch.int64, torch.float64):
        raise ValueError("x must be a CUDA int32, float32, int64 or float64 tensor (there is no CPU path)")
    x = x.contiguous()
    n = x.numel()
    own = plan is None
    if own:
        plan = Plan(max(n, 1), x.dtype, device=x.device, tuning="default")
    elif plan.dtype != x.dtype or plan.capacity < n:
        raise ValueError("plan must hold %s keys of at least %d" % (x.dtype, n))
    need = workspace_bytes(n)
    if work is None:
        work = torch.empty(max(need, 16), dtype=torch.uint8, device=x.device)
    elif work.numel() * work.element_size() < need or not work.is_cuda:
        raise ValueError("work must be a CUDA buffer of at least %d bytes" % need)
    return x, n, plan, own, work


def _finish(st: int, what: str, plan: Plan, own: bool, stream) -> None:
    _lib.check(st, what)
    if own:
        plan.check(stream)
        plan.close()


def _run(fn_name: str, x: torch.Tensor, cmp: int | None, plan, work, stream):
    x, n, plan, own, work = _prep(x, plan, work)
    out = torch.empty(n, dtype=torch.int32, device=x.device)
    lib = _lib.load()
    args = [plan._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), n]
    if cmp is not None:
        args.append(cmp)
    args += [ctypes.c_void_p(work.data_ptr()), ctypes.c_void_p(_stream_handle(x.device, stream))]
    _finish(getattr(lib, fn_name)(*args), fn_name, plan, own, stream)
    return out


def prev_greater(x: torch.Tensor, inclusive: bool = False, plan: Plan | None = None,
                 work: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """out[i] = max{j < i : x[j] > x[i]} (>= when inclusive), else -1."""
    return _run("apsep_run_prev_greater", x, _lib.LE if inclusive else _lib.LT, plan, work, stream)


def next_smaller(x: torch.Tensor, inclusive: bool = False, plan: Plan | None = None,
                 work: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """out[i] = min{j > i : x[j] < x[i]} (<= when inclusive), else -1."""
    return _run("apsep_run_next_smaller", x, _lib.LE if inclusive else _lib.LT, plan, work, stream)


def stock_span(prices: torch.Tensor, plan: Plan | None = None, work: torch.Tensor | None = None,
               stream=None) -> torch.Tensor:
    """out[i] = the number of consecutive prices ending at i that are <= prices[i]."""
    return _run("apsep_stock_span", prices, None, plan, work, stream)


def cartesian_parents(x: torch.Tensor, plan: Plan | None = None, work: torch.Tensor | None = None,
                      stream=None) -> torch.Tensor:
    """Parent of each key in the min-rooted Cartesian tree (-1 at the root);
    a later equal key is the right child of an earlier one."""
    return _run("apsep_cartesian_parents", x, None, plan, work, stream)


def largest_rectangle(heights: torch.Tensor, plan: Plan | None = None, work: torch.Tensor | None = None,
                      stream=None) -> int:
    """Largest rectangle in the histogram of int32 heights >= 0 (synchronises)."""
    if heights.dtype != torch.int32:
        raise ValueError("heights must be int32")
    h, n, plan, own, work = _prep(heights, plan, work)
    area = torch.zeros(1, dtype=torch.int64, device=h.device)
    st = _lib.load().apsep_largest_rectangle(plan._h, ctypes.c_void_p(h.data_ptr()), n,
                                             ctypes.c_void_p(area.data_ptr()), ctypes.c_void_p(work.data_ptr()),
                                             ctypes.c_void_p(_stream_handle(h.device, stream)))
    _finish(st, "apsep_largest_rectangle", plan, own, stream)
    return int(area.item())
