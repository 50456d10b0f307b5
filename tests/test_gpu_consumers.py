"""GPU parity of the consumers (apsep_run_prev_greater, apsep_run_next_smaller,
apsep_stock_span, apsep_largest_rectangle, apsep_cartesian_parents) through
the C ABI, bit-exact against the CPU oracles: the monotone-stack
restatements on small inputs, their (CPU-pinned) compositions on large ones."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import consumers as oc
from apsep_gb300 import ApsepError, Plan, _lib, consumers

pytestmark = pytest.mark.gpu


def keys(name, n, rng, dtype=np.int32):
    if name == "uniform":
        a = rng.integers(-(1 << 31), 1 << 31, n, dtype=np.int64)
    elif name == "dup16":
        a = rng.integers(0, 16, n)
    elif name == "desc":
        a = np.arange(n, 0, -1)
    elif name == "asc":
        a = np.arange(n)
    else:
        raise KeyError(name)
    if dtype == np.float32:
        return (a % (1 << 20) * 0.25 - (1 << 17)).astype(np.float32)
    return a.astype(np.int32)


SIZES = [1, 2, 1000, 65543, 3_000_001]


@pytest.fixture(scope="module")
def plans():
    p = {np.int32: Plan(3_000_001, torch.int32), np.float32: Plan(3_000_001, torch.float32)}
    yield p
    for v in p.values():
        v.close()


def check(got, want, what):
    if not np.array_equal(got, want):
        bad = int(np.flatnonzero(got != want)[0])
        pytest.fail("%s: first mismatch at %d: got %d want %d" % (what, bad, got[bad], want[bad]))


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
@pytest.mark.parametrize("name", ["uniform", "dup16", "desc", "asc"])
def test_prev_greater_next_smaller_span_cartesian(plans, dtype, name):
    rng = np.random.default_rng(sum(map(ord, name)) + (7 if dtype == np.float32 else 0))
    plan = plans[dtype]
    for n in SIZES:
        a = keys(name, n, rng, dtype)
        x = torch.from_numpy(a).cuda()
        small = n <= 1000
        for le in (False, True):
            want = oc.prev_greater_stack(list(a), le) if small else oc.prev_greater(a, le)
            check(consumers.prev_greater(x, le, plan=plan).cpu().numpy(), want, "prev_greater %s %d" % (le, n))
            want = oc.next_smaller_stack(list(a), le) if small else oc.next_smaller(a, le)
            check(consumers.next_smaller(x, le, plan=plan).cpu().numpy(), want, "next_smaller %s %d" % (le, n))
        want = oc.stock_span_stack(list(a)) if small else oc.stock_span(a)
        check(consumers.stock_span(x, plan=plan).cpu().numpy(), want, "stock_span %d" % n)
        want = oc.cartesian_parents_stack(list(a)) if small else oc.cartesian_parents(a)
        check(consumers.cartesian_parents(x, plan=plan).cpu().numpy(), want, "cartesian %d" % n)
        plan.check()


@pytest.mark.parametrize("k", [2, 1000, 1 << 30])
def test_largest_rectangle(plans, k):
    rng = np.random.default_rng(k)
    for n in SIZES:
        h = rng.integers(0, k, n).astype(np.int32)
        want = oc.largest_rectangle_stack(list(h)) if n <= 1000 else oc.largest_rectangle(h)
        assert consumers.largest_rectangle(torch.from_numpy(h).cuda(), plan=plans[np.int32]) == want, n
    assert consumers.largest_rectangle(torch.tensor([2, 1, 5, 6, 2, 3], dtype=torch.int32, device="cuda")) == 10
    plans[np.int32].check()


def test_one_workspace_no_allocation_in_the_loop(plans):
    rng = np.random.default_rng(9)
    plan = plans[np.int32]
    n = 200_003
    work = torch.empty(consumers.workspace_bytes(n), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        a = rng.integers(0, 100, n).astype(np.int32)
        x = torch.from_numpy(a).cuda()
        check(consumers.stock_span(x, plan=plan, work=work).cpu().numpy(), oc.stock_span(a), "span")
        check(consumers.cartesian_parents(x, plan=plan, work=work).cpu().numpy(), oc.cartesian_parents(a), "cart")
    plan.check()


def test_invalid_arguments(plans):
    lib = _lib.load()
    plan = plans[np.int32]
    x = torch.zeros(1000, dtype=torch.int32, device="cuda")
    o = torch.zeros(1000, dtype=torch.int32, device="cuda")
    w = torch.empty(consumers.workspace_bytes(1000) + 64, dtype=torch.uint8, device="cuda")
    vp = ctypes.c_void_p
    # workspace off a 16-byte boundary
    assert lib.apsep_run_prev_greater(plan._h, vp(x.data_ptr()), vp(o.data_ptr()), 1000, _lib.LT,
                                      vp(w.data_ptr() + 4), None) == _lib.APSEP_EINVAL
    # workspace overlapping the output
    assert lib.apsep_stock_span(plan._h, vp(x.data_ptr()), vp(o.data_ptr()), 1000, vp(o.data_ptr()),
                                None) == _lib.APSEP_EINVAL
    # beyond the plan's capacity
    with Plan(10, torch.int32) as small:
        assert lib.apsep_run_next_smaller(small._h, vp(x.data_ptr()), vp(o.data_ptr()), 1000, _lib.LT,
                                          vp(w.data_ptr()), None) == _lib.APSEP_EINVAL
    # the histogram needs an int32 plan
    area = torch.zeros(1, dtype=torch.int64, device="cuda")
    xf = torch.zeros(1000, dtype=torch.float32, device="cuda")
    assert lib.apsep_largest_rectangle(plans[np.float32]._h, vp(xf.data_ptr()), 1000, vp(area.data_ptr()),
                                       vp(w.data_ptr()), None) == _lib.APSEP_ENOTSUP
    # n == 0 is a no-op (the area is 0)
    area.fill_(7)
    assert lib.apsep_largest_rectangle(plan._h, vp(x.data_ptr()), 0, vp(area.data_ptr()), vp(w.data_ptr()),
                                       None) == _lib.APSEP_OK
    torch.cuda.synchronize()
    assert int(area.item()) == 0
    with pytest.raises(ValueError):
        consumers.prev_greater(x.cpu())


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
@pytest.mark.parametrize("shift", [0, 1, 3])
def test_flipped_run_and_its_general_route(plans, dtype, shift):
    # keys (and answers) on a 16-byte boundary take the one-run form (keys
    # flipped as they load, spans written as they leave); one or three keys
    # past it, the flip pass and a plain run: both bit-exact, with the
    # extreme keys the flip maps onto the engine's pad value
    rng = np.random.default_rng(40 + shift)
    plan = plans[dtype]
    n = 300_007
    for name in ("uniform", "dup16", "desc", "asc"):
        a = keys(name, n, rng, dtype)
        if dtype == np.int32:
            a[rng.integers(0, n, 200)] = np.iinfo(np.int32).min
            a[rng.integers(0, n, 200)] = np.iinfo(np.int32).max
        else:
            a[rng.integers(0, n, 200)] = -np.inf
            a[rng.integers(0, n, 200)] = np.float32(-0.0)
            a[rng.integers(0, n, 200)] = np.float32(0.0)
        base = torch.zeros(n + shift, dtype=torch.from_numpy(a[:0]).dtype, device="cuda")
        base[shift:] = torch.from_numpy(a).cuda()
        x = base[shift:]
        for le in (False, True):
            check(consumers.prev_greater(x, le, plan=plan).cpu().numpy(), oc.prev_greater(a, le),
                  "prev_greater %s %s" % (name, le))
        check(consumers.stock_span(x, plan=plan).cpu().numpy(), oc.stock_span(a), "stock_span %s" % name)
    plan.check()


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
@pytest.mark.parametrize("name", ["uniform", "dup16", "desc", "asc"])
def test_reversed_run(plans, dtype, name):
    # n a multiple of 32 on a 16-byte boundary: next smaller is one engine run
    # over the reversed array (TMA tiles counted from the end, a partial tile
    # at the array's start when n is not a multiple of 512; below 512 keys
    # plain loads), and the histogram and the Cartesian tree use it
    rng = np.random.default_rng(70 + sum(map(ord, name)))
    plan = plans[dtype]
    for n in (32, 480, 512, 544, 4096, 65536, 1_000_032, 2_000_032):
        a = keys(name, n, rng, dtype)
        x = torch.from_numpy(a).cuda()
        for le in (False, True):
            check(consumers.next_smaller(x, le, plan=plan).cpu().numpy(), oc.next_smaller(a, le),
                  "next_smaller %s %d" % (le, n))
        check(consumers.cartesian_parents(x, plan=plan).cpu().numpy(), oc.cartesian_parents(a), "cartesian %d" % n)
        if dtype == np.int32:
            h = (np.abs(a.astype(np.int64)) % (1 << 20)).astype(np.int32)
            assert consumers.largest_rectangle(torch.from_numpy(h).cuda(), plan=plan) == oc.largest_rectangle(h), n
    plan.check()


def test_answers_over_the_keys_through_the_c_abi(plans):
    # d_out == d_in: the one-run forms step aside (the engine cannot read keys
    # it is overwriting) and the workspace route answers in place
    lib = _lib.load()
    vp = ctypes.c_void_p
    plan = plans[np.int32]
    rng = np.random.default_rng(88)
    n = 65536
    a = rng.integers(-1000, 1000, n).astype(np.int32)
    w = torch.empty(consumers.workspace_bytes(n), dtype=torch.uint8, device="cuda")
    for fn, want in (("apsep_run_prev_greater", oc.prev_greater(a, False)),
                     ("apsep_run_next_smaller", oc.next_smaller(a, False)),
                     ("apsep_stock_span", oc.stock_span(a))):
        buf = torch.from_numpy(a.copy()).cuda()
        args = [plan._h, vp(buf.data_ptr()), vp(buf.data_ptr()), n]
        if fn != "apsep_stock_span":
            args.append(_lib.LT)
        assert getattr(lib, fn)(*args, vp(w.data_ptr()), None) == _lib.APSEP_OK, fn
        torch.cuda.synchronize()
        check(buf.cpu().numpy(), want, fn + " in place")
    plan.check()
