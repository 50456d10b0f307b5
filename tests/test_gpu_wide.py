"""GPU parity of 8-byte keys (int64 / float64, int32 positions) through the C
ABI, bit-exact against the CPU oracle: keys that differ only in their low 32
bits, full-range magnitudes, float64 steps below float32 resolution, the
monotone shapes, ties under both comparators, every tile / range edge."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import ApsepError, Plan, _lib

pytestmark = pytest.mark.gpu

POISON = int(np.uint32(0xABABABAB).view(np.int32))


def keys(name, n, rng, dtype):
    if name == "uniform":
        a = rng.integers(-(1 << 63), (1 << 63) - 1, n, dtype=np.int64, endpoint=True)
    elif name == "lowbits":  # equal high words: only the low 32 bits order them
        a = (np.int64(1) << 40) + rng.integers(0, 1 << 32, n, dtype=np.int64)
    elif name == "desc":
        a = (np.int64(1) << 50) - np.arange(n, dtype=np.int64) * 3
    elif name == "asc":
        a = np.arange(n, dtype=np.int64) - (np.int64(1) << 45)
    elif name == "dup16":
        a = rng.integers(0, 16, n).astype(np.int64) << 33
    else:
        raise KeyError(name)
    if dtype == np.float64:
        # distinct below float32 resolution: 1 + k * 2^-40
        return 1.0 + (a % (1 << 20)).astype(np.float64) * 2.0 ** -40 if name != "uniform" else \
            rng.standard_normal(n) * 1e300
    return a


@pytest.fixture(scope="module")
def plans():
    cap = 3_000_001
    p = {np.int64: Plan(cap, torch.int64), np.float64: Plan(cap, torch.float64)}
    yield p
    for v in p.values():
        v.close()


def run(plan, a, le, offset=0):
    n = a.shape[0]
    xb = torch.zeros(n + 2, dtype=torch.from_numpy(a[:0]).dtype, device="cuda")
    xb[offset:offset + n] = torch.from_numpy(a).cuda()
    ob = torch.full((n + 4,), POISON, dtype=torch.int32, device="cuda")
    plan.run(xb[offset:offset + n], out=ob[offset:offset + n], n=n, inclusive=le)
    plan.check()
    got = ob.cpu().numpy()
    assert (got[:offset] == POISON).all() and (got[offset + n:] == POISON).all()
    return got[offset:offset + n]


@pytest.mark.parametrize("dtype", [np.int64, np.float64])
@pytest.mark.parametrize("name", ["uniform", "lowbits", "desc", "asc", "dup16"])
def test_wide_keys_vs_oracle(plans, dtype, name):
    rng = np.random.default_rng(sum(map(ord, name)) + (5 if dtype == np.float64 else 0))
    for n in (1, 2, 255, 256, 257, 5000, 100003, 3_000_001):
        a = keys(name, n, rng, dtype)
        for le in (False, True):
            got, want = run(plans[dtype], a, le), oracle.apse(a, le)
            if not np.array_equal(got, want):
                bad = int(np.flatnonzero(got != want)[0])
                pytest.fail("%s n=%d le=%s: first mismatch at %d: got %d want %d" %
                            (name, n, le, bad, got[bad], want[bad]))


def test_float64_signs_and_zeros(plans):
    """float64 keys compare through an order map of their bits: negative
    values, both zeros (equal under < and <=), subnormals, huge magnitudes."""
    rng = np.random.default_rng(99)
    vals = np.array([-0.0, 0.0, -1.0, 1.0, -5e-324, 5e-324, -1e308, 1e308, 2.5, -2.5], dtype=np.float64)
    for n in (1000, 100003):
        a = rng.choice(vals, n)
        for le in (False, True):
            assert np.array_equal(run(plans[np.float64], a, le), oracle.apse(a, le)), (n, le)


@pytest.mark.parametrize("dtype", [np.int64, np.float64])
def test_wide_segmented_batches(plans, dtype):
    """A batch of 8-byte-key arrays in one launch: per-array answers relative
    to each array's start, against the oracle array by array."""
    rng = np.random.default_rng(7 if dtype == np.int64 else 8)
    lengths = np.maximum(0, np.round(np.exp(rng.uniform(0, np.log(200000), 300))).astype(np.int64) - 1)
    lengths[:6] = [0, 1, 2, 255, 256, 257]
    names = ["uniform", "lowbits", "desc", "asc", "dup16"]
    parts = [keys(names[i % 5], int(L), rng, dtype) for i, L in enumerate(lengths)]
    a = np.concatenate(parts)
    offs = np.zeros(len(lengths) + 1, dtype=np.int64)
    offs[1:] = np.cumsum(lengths)
    n = a.shape[0]
    for le in (False, True):
        with Plan(n, torch.from_numpy(a[:0]).dtype, inclusive=le) as plan:
            out = torch.full((n,), POISON, dtype=torch.int32, device="cuda")
            plan.run_segmented(torch.from_numpy(a).cuda(), torch.from_numpy(offs).cuda(), out=out)
            plan.check()
        got = out.cpu().numpy()
        for s0, s1 in zip(offs[:-1], offs[1:]):
            if s1 > s0:
                assert np.array_equal(got[s0:s1], oracle.apse(np.ascontiguousarray(a[s0:s1]), le)), (s0, s1, le)


def test_wide_keys_off_a_16_byte_boundary(plans):
    """8-byte aligned but not 16: plain loads and stores throughout."""
    rng = np.random.default_rng(12)
    for name in ("uniform", "desc", "asc"):
        a = keys(name, 100003, rng, np.int64)
        assert np.array_equal(run(plans[np.int64], a, False, offset=1), oracle.apse(a)), name


def test_wide_full_size():
    n = 1 << 25
    rng = np.random.default_rng(25)
    with Plan(n, torch.int64) as plan:
        for name in ("uniform", "desc", "asc", "lowbits"):
            a = keys(name, n, rng, np.int64)
            assert np.array_equal(run(plan, a, False), oracle.apse(a)), name


def test_wide_unsupported_forms(plans):
    lib = _lib.load()
    plan = plans[np.int64]
    x = torch.zeros(1000, dtype=torch.int64, device="cuda")
    o = torch.zeros(1000, dtype=torch.int32, device="cuda")
    assert lib.apsep_plan_set_config(plan._h, 0) == _lib.APSEP_ENOTSUP
    assert lib.apsep_plan_set_config(plan._h, 1) == _lib.APSEP_OK
    vp = ctypes.c_void_p
    assert lib.apsep_run(plan._h, vp(x.data_ptr() + 4), vp(o.data_ptr()), 100, None) == _lib.APSEP_EINVAL
    assert lib.apsep_run_noalloc(vp(x.data_ptr()), vp(o.data_ptr()), 100, _lib.INT64, _lib.LT,
                                 None) == _lib.APSEP_EINVAL
    from apsep_gb300 import consumers
    w = torch.empty(consumers.workspace_bytes(1000), dtype=torch.uint8, device="cuda")
    area = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert lib.apsep_largest_rectangle(plan._h, vp(x.data_ptr()), 1000, vp(area.data_ptr()), vp(w.data_ptr()),
                                       None) == _lib.APSEP_ENOTSUP  # the histogram takes int32 heights


@pytest.mark.parametrize("dtype", [np.int64, np.float64])
def test_wide_consumers(plans, dtype):
    from oracle import consumers as oc
    from apsep_gb300 import consumers
    rng = np.random.default_rng(31)
    for name in ("uniform", "lowbits", "dup16"):
        a = keys(name, 100003, rng, dtype)
        x = torch.from_numpy(a).cuda()
        plan = plans[dtype]
        for le in (False, True):
            assert np.array_equal(consumers.prev_greater(x, le, plan=plan).cpu().numpy(), oc.prev_greater(a, le))
            assert np.array_equal(consumers.next_smaller(x, le, plan=plan).cpu().numpy(), oc.next_smaller(a, le))
        assert np.array_equal(consumers.stock_span(x, plan=plan).cpu().numpy(), oc.stock_span(a))
        assert np.array_equal(consumers.cartesian_parents(x, plan=plan).cpu().numpy(), oc.cartesian_parents(a))
        plan.check()
