"""apsep_run_noalloc: the run for callers that cannot allocate device memory.

Such callers (a host process that has reserved the whole device heap for its
own pool, or a path where cudaMalloc/cudaFree and their synchronisation are
not allowed) get their scratch from a static device array inside the
library.  This checks, through the C ABI, that two calls in a row give
bit-for-bit the answers of the plan-based apsep_run on the same inputs, that
sizes beyond the array's limit are refused, and that a device-side wait that
gives up is reported by apsep_noalloc_check instead of passing silently.  The
file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle

from apsep_gb300 import Plan, _lib

pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _noalloc(x, out, n, dtype, cmp):
    lib = _lib.load()
    return lib.apsep_run_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), n, dtype, cmp,
                                 _stream())


def _check():
    return _lib.load().apsep_noalloc_check(_stream())


def test_noalloc_matches_plan_on_two_calls_in_a_row():
    rng = np.random.default_rng(4242)
    cases = [
        (rng.integers(0, 1 << 31, 1_000_003, dtype=np.int64).astype(np.int32), _lib.INT32, _lib.LT),
        (np.arange(3 * 4096 + 5, dtype=np.int32)[::-1].copy(), _lib.INT32, _lib.LT),
        (rng.integers(0, 16, 777_777).astype(np.int32), _lib.INT32, _lib.LE),
        ((rng.integers(-1000, 1000, 250_001) * 0.5).astype(np.float32), _lib.FLOAT32, _lib.LT),
    ]
    for a, dtype, cmp in cases:
        n = a.shape[0]
        x = torch.from_numpy(a).cuda()
        with Plan(n, x.dtype, inclusive=(cmp == _lib.LE)) as plan:
            want = plan.run(x)
            plan.check()
        want = want.cpu()
        for _ in range(2):  # the shared static scratch carries state from call to call
            out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            assert _noalloc(x, out, n, dtype, cmp) == _lib.APSEP_OK
            assert _check() == _lib.APSEP_OK
            assert torch.equal(out.cpu(), want)


def test_noalloc_misaligned_view_at_full_capacity():
    """The largest no-alloc size behind a 3-key view head (the view then holds
    max + 3 keys, which the static scratch must still cover)."""
    n = _lib.NOALLOC_MAX_KEYS
    a = np.random.default_rng(77).integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
    xb = torch.zeros(n + 4, dtype=torch.int32, device="cuda")
    xb[3:3 + n] = torch.from_numpy(a).cuda()
    ob = torch.full((n + 4,), -7, dtype=torch.int32, device="cuda")
    assert _noalloc(xb[3:3 + n], ob[3:3 + n], n, _lib.INT32, _lib.LT) == _lib.APSEP_OK
    assert _check() == _lib.APSEP_OK
    got = ob.cpu().numpy()
    assert np.array_equal(got[3:3 + n], oracle.apse(a))
    assert (got[:3] == -7).all() and got[3 + n] == -7


def test_noalloc_refuses_sizes_beyond_its_static_scratch():
    n = _lib.NOALLOC_MAX_KEYS + 1
    x = torch.zeros(n, dtype=torch.int32, device="cuda")
    out = torch.empty_like(x)
    assert _noalloc(x, out, n, _lib.INT32, _lib.LT) == _lib.APSEP_EINVAL


def test_noalloc_wait_that_gives_up_is_reported():
    """One range never publishes (host-armed injection, bounded waits): the run
    finishes, apsep_noalloc_check reports APSEP_ETIMEOUT and clears it, and the
    next call on the shared static scratch is correct again."""
    n = 4096 * 6  # 48 tiles -> 48 one-tile ranges
    a = np.random.default_rng(8).integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
    x = torch.from_numpy(a).cuda()
    out = torch.empty_like(x)
    lib = _lib.load()
    assert lib.apsep_debug_inject(None, 2, 2000) == _lib.APSEP_OK
    assert _noalloc(x, out, n, _lib.INT32, _lib.LT) == _lib.APSEP_OK
    assert _check() == _lib.APSEP_ETIMEOUT
    assert _check() == _lib.APSEP_OK  # cleared
    out.fill_(-7)
    assert _noalloc(x, out, n, _lib.INT32, _lib.LT) == _lib.APSEP_OK
    assert _check() == _lib.APSEP_OK
    assert np.array_equal(out.cpu().numpy(), oracle.apse(a))
