"""GPU parity of 64-bit positions (apsep_run64): an array runs as pieces of the
plan's capacity, and keys that their own piece does not answer are answered
from the hierarchy of minima over the keys before it.  Small plans cut small
arrays into many pieces, so every cross-piece case runs at sizes the CPU
oracle checks in full; arrays beyond 2^31 keys check the int64 positions
themselves."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan, _lib, apse64

pytestmark = pytest.mark.gpu

TYPES = [np.int32, np.float32, np.int64, np.float64]
NAMES = ["uniform", "dup", "desc", "asc", "rising_runs", "valley", "sawtooth", "walk"]


def keys(name, n, rng, dtype, piece):
    i = np.arange(n, dtype=np.int64)
    if name == "uniform":
        a = rng.integers(0, 1 << 30, n)
    elif name == "dup":
        a = rng.integers(0, 4, n)
    elif name == "desc":
        a = -i
    elif name == "asc":
        a = i
    elif name == "rising_runs":  # descending runs, each above the last: every piece start queries
        run = int(rng.integers(max(piece // 3, 1), 3 * piece + 2))
        a = (i // run) * (2 * run) - (i % run)
    elif name == "valley":  # a climb down with a few deep keys
        a = n - i
        a[rng.integers(0, n, 3)] = -5
    elif name == "sawtooth":
        a = i % 257
    else:  # random walk: answers at every distance
        a = np.cumsum(rng.integers(-3, 4, n))
    return a.astype(dtype)


@pytest.fixture(scope="module")
def plans():
    made = {}

    def get(dtype, cap):
        k = (dtype, cap)
        if k not in made:
            made[k] = Plan(cap, torch.from_numpy(np.zeros(0, dtype)).dtype, tuning=None)
        return made[k]

    yield get
    for p in made.values():
        p.close()


def run64(plan, a, le):
    x = torch.from_numpy(a).cuda()
    out = plan.run64(x, inclusive=le)
    plan.check()
    return out.cpu().numpy()


@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: t.__name__)
@pytest.mark.parametrize("name", NAMES)
def test_pieces_against_the_oracle(plans, name, dtype):
    rng = np.random.default_rng(NAMES.index(name) * 10 + TYPES.index(dtype))
    for cap, n in ((32, 5000), (40, 1), (1000, 993), (1000, 60_007), (5003, 200_000)):
        piece = min(n, cap // 32 * 32)
        a = keys(name, n, rng, dtype, piece)
        for le in (False, True):
            got = run64(plans(dtype, cap), a, le)
            want = oracle.apse(a, le).astype(np.int64)
            if not np.array_equal(got, want):
                bad = int(np.flatnonzero(got != want)[0])
                pytest.fail("cap=%d n=%d le=%s: first mismatch at %d: got %d want %d"
                            % (cap, n, le, bad, got[bad], want[bad]))


@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: t.__name__)
def test_pieces_off_a_16_byte_boundary(plans, dtype):
    # keys one element past an aligned base: every piece's tiles come by plain
    # loads instead of TMA; answers to an 8-byte aligned int64 buffer
    rng = np.random.default_rng(90 + TYPES.index(dtype))
    n = 60_007
    for name in ("uniform", "rising_runs", "walk"):
        a = keys(name, n, rng, dtype, 992)
        base = torch.zeros(n + 1, dtype=torch.from_numpy(a[:0]).dtype, device="cuda")
        base[1:] = torch.from_numpy(a).cuda()
        ob = torch.full((n + 2,), -7, dtype=torch.int64, device="cuda")
        for le in (False, True):
            plan = plans(dtype, 1000)
            plan.run64(base[1:], out=ob[1:n + 1], inclusive=le)
            plan.check()
            got = ob.cpu().numpy()
            assert got[0] == -7 and got[n + 1] == -7
            assert np.array_equal(got[1:n + 1], oracle.apse(a, le).astype(np.int64)), (name, le)


def test_one_piece_matches_the_int32_run(plans):
    rng = np.random.default_rng(7)
    plan = plans(np.int32, 300_000)
    a = rng.integers(-1000, 1000, 250_000).astype(np.int32)
    x = torch.from_numpy(a).cuda()
    got = plan.run64(x)
    ref = plan.run(x)
    plan.check()
    assert torch.equal(got, ref.to(torch.int64))


def test_float_zeros_and_extremes(plans):
    plan = plans(np.float32, 64)
    a = np.array([0.0, -0.0, 1e-45, -1e-45, 3e38, -3e38, np.inf, -np.inf] * 200, dtype=np.float32)
    for le in (False, True):
        assert np.array_equal(run64(plan, a, le), oracle.apse(a, le).astype(np.int64))
    plan = plans(np.int64, 64)
    b = np.array([np.iinfo(np.int64).max, np.iinfo(np.int64).min, 0, -1, 1 << 40] * 300, dtype=np.int64)
    for le in (False, True):
        assert np.array_equal(run64(plan, b, le), oracle.apse(b, le).astype(np.int64))


def test_workspace_and_arguments(plans):
    lib = _lib.load()
    small = plans(np.int32, 31)  # too small to cut into 32-key pieces
    assert small.workspace64_bytes(31) > 0
    assert small.workspace64_bytes(32) == -1
    with pytest.raises(ValueError):
        small.run64(torch.zeros(100, dtype=torch.int32, device="cuda"))
    plan = plans(np.int32, 1000)
    assert plan.workspace64_bytes(-1) == -1
    assert plan.workspace64_bytes(_lib.MAX_KEYS64 + 1) == -1
    n = 5000
    x = torch.arange(n, dtype=torch.int32, device="cuda")
    ob = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    work = torch.empty(plan.workspace64_bytes(n) + 16, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    vp = ctypes.c_void_p

    def call(xp, op, wp, nn=n, cmp=_lib.LT):
        return lib.apsep_run64(plan._h, vp(xp), vp(op), nn, cmp, vp(wp), vp(st))

    assert call(x.data_ptr(), ob.data_ptr() + 4, work.data_ptr()) == _lib.APSEP_EINVAL  # misaligned out
    assert call(x.data_ptr(), ob.data_ptr(), work.data_ptr() + 8) == _lib.APSEP_EINVAL  # misaligned work
    assert call(x.data_ptr(), work.data_ptr(), work.data_ptr()) == _lib.APSEP_EINVAL  # overlap
    assert call(x.data_ptr(), ob.data_ptr(), work.data_ptr(), cmp=7) == _lib.APSEP_EINVAL
    assert call(0, ob.data_ptr(), work.data_ptr()) == _lib.APSEP_EINVAL
    assert call(x.data_ptr(), ob.data_ptr(), work.data_ptr(), nn=0) == _lib.APSEP_OK
    assert call(x.data_ptr(), ob.data_ptr(), work.data_ptr()) == _lib.APSEP_OK
    plan.check()
    assert torch.equal(ob[:n], torch.arange(n, dtype=torch.int64, device="cuda") - 1)


def test_one_call_helper():
    a = np.random.default_rng(3).integers(0, 50, 100_000).astype(np.int32)
    got = apse64(torch.from_numpy(a).cuda()).cpu().numpy()
    assert np.array_equal(got, oracle.apse(a, False).astype(np.int64))


# ---- beyond 2^31 keys ------------------------------------------------------
BIG = (1 << 31) + (1 << 22)


def _needs_memory():
    if torch.cuda.get_device_properties(0).total_memory < (80 << 30):
        pytest.skip("needs a GPU with 80 GB or more")


def suffix_min_stack(x, s, chunk=1 << 26):
    """Positions of the strict suffix minima of x[:s] (every key smaller than
    all later keys before s): the only keys before s that can answer a key at
    or after s."""
    parts, m = [], None
    for hi in range(s, 0, -chunk):
        lo = max(0, hi - chunk)
        c = x[lo:hi]
        sm = torch.flip(torch.cummin(torch.flip(c, [0]), 0).values, [0])
        nxt = torch.empty_like(sm)
        nxt[:-1] = sm[1:]
        if m is None:
            keep = c < nxt
            keep[-1] = True
        else:
            nxt[-1] = m
            keep = c < torch.minimum(nxt, m)
        parts.append(torch.nonzero(keep).flatten() + lo)
        m = sm[0] if m is None else torch.minimum(sm[0], m)
    return torch.cat(parts[::-1]).cpu().numpy()


def check_from(x, out, s, le):
    """Every answer at or after s, from the oracle on the keys that can
    answer them: the suffix-minimum stack of x[:s], then x[s:]."""
    st = suffix_min_stack(x, s)
    tail = x[s:].cpu().numpy()
    comp = np.concatenate([x[torch.from_numpy(st).cuda()].cpu().numpy(), tail])
    r = oracle.apse(comp, le).astype(np.int64)
    k = st.shape[0]
    want = np.where(r < 0, -1, np.where(r < k, st[np.minimum(r, max(k - 1, 0))], s + r - k))
    got = out[s:].cpu().numpy()
    assert got.shape == want[k:].shape
    if not np.array_equal(got, want[k:]):
        bad = int(np.flatnonzero(got != want[k:])[0])
        pytest.fail("key %d: got %d want %d" % (s + bad, got[bad], want[k + bad]))


@pytest.mark.parametrize("case", ["uniform", "deep_tail"])
def test_beyond_2p31_keys(case):
    _needs_memory()
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randint(0, (1 << 30), (BIG,), dtype=torch.int32, device="cuda", generator=g)
    if case == "deep_tail":
        # The second piece descends from the top of the first piece's range to
        # below all of it: every key of it is answered from the first piece,
        # further back as the keys fall, and the last ones by nothing.
        t = torch.arange(BIG - _lib.MAX_KEYS, dtype=torch.int64, device="cuda")
        x[_lib.MAX_KEYS:] = ((1 << 30) - 256 * t).to(torch.int32)
    with Plan(_lib.MAX_KEYS, torch.int32, tuning=None) as plan:
        for le in (False, True):
            out = plan.run64(x, inclusive=le)
            plan.check()
            head = 1 << 20
            assert np.array_equal(out[:head].cpu().numpy(), oracle.apse(x[:head].cpu().numpy(), le).astype(np.int64))
            check_from(x, out, _lib.MAX_KEYS - (1 << 20), le)
            del out
    del x
    torch.cuda.empty_cache()


def test_beyond_2p31_keys_ascending():
    _needs_memory()
    x = (torch.arange(BIG, dtype=torch.int64, device="cuda") - (1 << 31)).to(torch.int32)
    with Plan(_lib.MAX_KEYS, torch.int32, tuning=None) as plan:
        out = plan.run64(x)
        plan.check()
    step = 1 << 28
    for lo in range(0, BIG, step):
        hi = min(BIG, lo + step)
        assert torch.equal(out[lo:hi], torch.arange(lo - 1, hi - 1, dtype=torch.int64, device="cuda"))
    del out, x
    torch.cuda.empty_cache()


def test_graph_capture_of_pieces(plans):
    # every piece's engine run, widening pass and level build replay from one graph
    plan = plans(np.int32, 1000)
    n = 60_007
    rng = np.random.default_rng(21)
    x = torch.empty(n, dtype=torch.int32, device="cuda")
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    work = torch.empty(plan.workspace64_bytes(n), dtype=torch.uint8, device="cuda")
    x.copy_(torch.from_numpy(keys("walk", n, rng, np.int32, 992)))
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run64(x, out=out, work=work)  # warm-up outside capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run64(x, out=out, work=work)
    for name in ("uniform", "rising_runs", "desc", "walk"):
        a = keys(name, n, rng, np.int32, 992)
        x.copy_(torch.from_numpy(a))
        out.fill_(-7)
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), oracle.apse(a).astype(np.int64)), name
    plan.check()


def test_run64_while_another_device_is_current():
    """apsep_run64 runs on its plan's device whatever device is current, and
    leaves the caller's device current."""
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    n = 3 * 4096 + 5
    a = np.random.default_rng(12).integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
    with torch.cuda.device(1):
        with Plan(4096, torch.int32, device=1) as plan:
            x = torch.from_numpy(a).to("cuda:1")
            torch.cuda.set_device(0)
            out = plan.run64(x)
            assert torch.cuda.current_device() == 0
            plan.check()
            assert np.array_equal(out.cpu().numpy(), oracle.apse(a).astype(np.int64))
