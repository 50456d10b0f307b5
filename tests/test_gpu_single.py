"""GPU parity of the single-array engine (libapsep.so through its C ABI).

Every check is bit-exact: against the reference's own outputs (golden
hashes, tests/golden/) on the reference harnesses' own inputs, and against
the CPU oracle on seeded inputs.  Outputs are pre-poisoned with 0xAB bytes
as the reference's SPT harness does (src/bench_spt_le.cu:76), so a word the
engine never writes is caught.
"""
import hashlib

import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import ApsepError, Plan, _lib, launch_spt

pytestmark = pytest.mark.gpu

POISON = np.int32(np.uint32(0xABABABAB).view(np.int32))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def run_gpu(plan, a, le=False, poison=True, offset=0):
    """APSE of `a` on the GPU; `offset` shifts both device buffers by that many
    elements off their 16-byte alignment (exercises the non-TMA path)."""
    n = a.shape[0]
    xs = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    if offset:
        xb = torch.empty(n + offset, dtype=xs.dtype, device="cuda")
        xb[offset:] = xs
        xs = xb[offset:]
    ob = torch.full((n + offset,), int(POISON) if poison else 0, dtype=torch.int32, device="cuda")
    out = ob[offset:]
    plan.run(xs, out=out, n=n, inclusive=le)
    plan.check()
    return out.cpu().numpy()


@pytest.fixture(scope="module")
def plans():
    cap = (1 << 25) + 4096
    p = {torch.int32: Plan(cap, torch.int32), torch.float32: Plan(cap, torch.float32)}
    yield p
    for v in p.values():
        v.close()


def test_small_cases_reference(golden):
    # launch_spt: the reference's alloc+run+sync+free entry (main.cu:234-235)
    for c in golden["main_small_cases"]["cases"]:
        a = torch.tensor(c["input"], dtype=torch.int32, device="cuda")
        out = torch.full_like(a, int(POISON))
        launch_spt(a, out, a.numel())
        assert out.cpu().tolist() == c["expected"], c["label"]


@pytest.mark.parametrize("run_idx", [0, 1, 2, 3])
def test_stress_reference(golden, plans, run_idx):
    run = golden["main_stress"]["runs"][run_idx]
    plan = plans[torch.int32]
    for (n, h), a in zip(run["trials_n_sha256"], oracle.main_stress_inputs(run["seed"], run["trials"], run["max_n"])):
        got = run_gpu(plan, a)
        assert sha(got) == h, (run["seed"], n)


def test_spt_le_cases_reference(golden, plans):
    plan = plans[torch.int32]
    full = {}
    for e in golden["spt_le_cases"]["entries"]:
        name = e["case"]
        if name not in full or full[name].shape[0] < e["n"]:
            full[name] = oracle.gen_spt_le_case(name, max(x["n"] for x in golden["spt_le_cases"]["entries"]
                                                          if x["case"] == name))
        a = full[name][: e["n"]]
        got = run_gpu(plan, a, le=e["le"])
        assert sha(got) == e["sha256"], (name, e["n"], e["le"])


EDGE_SIZES = [1, 2, 3, 31, 32, 33, 63, 64, 65, 127, 128, 129, 511, 512, 513, 1023, 1024, 2047, 2048, 2049,
              4095, 4096, 4097, 8191, 8192, 8193, 3 * 4096 + 17, 65536 + 5, 1000003]


def dist(name, n, rng, dtype=np.int32):
    if name == "uniform":
        return rng.integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
    if name == "desc":
        return np.arange(n - 1, -1, -1, dtype=np.int32)
    if name == "asc":
        return np.arange(n, dtype=np.int32)
    if name == "dup16":
        return rng.integers(0, 16, n).astype(np.int32)
    if name == "dup2":
        return rng.integers(0, 2, n).astype(np.int32)
    if name == "saw257":
        return (np.arange(n) % 257).astype(np.int32)
    if name == "valley":  # one tiny key, then a long descent: deep cross-tile answers
        a = np.arange(n + 1000, 1000, -1, dtype=np.int64).astype(np.int32)
        a[0] = -5
        return a
    if name == "intmax":
        a = rng.integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
        a[rng.random(n) < 0.25] = np.iinfo(np.int32).max
        return a
    raise KeyError(name)


DISTS = ["uniform", "desc", "asc", "dup16", "dup2", "saw257", "valley", "intmax"]


@pytest.mark.parametrize("le", [False, True])
@pytest.mark.parametrize("name", DISTS)
def test_edge_sizes_vs_oracle(plans, name, le):
    rng = np.random.default_rng(1000 + DISTS.index(name))
    plan = plans[torch.int32]
    for n in EDGE_SIZES:
        a = dist(name, n, rng)
        got = run_gpu(plan, a, le=le)
        want = oracle.apse(a, le)
        if not np.array_equal(got, want):
            bad = int(np.flatnonzero(got != want)[0])
            pytest.fail("%s n=%d le=%s first mismatch at %d: got %d want %d" % (name, n, le, bad, got[bad],
                                                                               want[bad]))


def near_monotone(n, kind, ipt):
    """Keys that pass a check of a few neighbour pairs per lane (pairs ending at
    k = ipt/4, ipt/2, 3*ipt/4 of each lane's ipt keys) but are not monotone:
    one dip (or bump) at k = 1 of every lane; and monotone runs with ties."""
    i = np.arange(n, dtype=np.int64)
    if kind == "asc_dip":
        a = i * 4
        a[i % ipt == 1] -= 10
    elif kind == "desc_bump":
        a = -i * 4
        a[i % ipt == 1] += 10
    elif kind == "asc_ties":  # non-decreasing: ties every 1000 keys and at every lane start
        a = i - i // 1000
        a[i % 97 == 0] = a[np.maximum(i[i % 97 == 0] - 1, 0)]
    else:  # strictly increasing tiles, one tile in 50 with a tie
        a = i * 2
        a[(i % (50 * 512)) == 300] -= 2
    return a.astype(np.int32)


@pytest.mark.parametrize("config", range(_lib.NUM_CONFIGS))
@pytest.mark.parametrize("kind", ["asc_dip", "desc_bump", "asc_ties", "asc_rare_tie"])
@pytest.mark.parametrize("le", [False, True])
def test_near_monotone_tiles(config, kind, le):
    ipt = 16 if config == 0 else 8
    n = 3_000_017
    a = near_monotone(n, kind, ipt)
    with Plan(n, torch.int32, inclusive=le, tuning=None) as plan:
        plan.set_config(config)
        got = run_gpu(plan, a, le=le)
    want = oracle.apse(a, le)
    if not np.array_equal(got, want):
        bad = int(np.flatnonzero(got != want)[0])
        pytest.fail("first mismatch at %d: got %d want %d" % (bad, got[bad], want[bad]))


@pytest.mark.parametrize("config", range(_lib.NUM_CONFIGS))
def test_every_config(config):
    rng = np.random.default_rng(77 + config)
    with Plan(300000, torch.int32) as plan:
        plan.set_config(config)
        for name in ("uniform", "desc", "asc", "dup16", "valley"):
            for n in (4096 * 3 + 100, 250000):
                a = dist(name, n, rng)
                for le in (False, True):
                    assert np.array_equal(run_gpu(plan, a, le=le), oracle.apse(a, le)), (config, name, n, le)


@pytest.mark.parametrize("le", [False, True])
def test_float_keys(plans, le):
    rng = np.random.default_rng(31)
    plan = plans[torch.float32]
    for n in (1, 33, 4097, 100000, 1 << 20):
        a = (-1e6 + rng.integers(0, 1 << 24, n) * (2e6 / (1 << 24))).astype(np.float32)
        assert np.array_equal(run_gpu(plan, a, le=le), oracle.apse(a, le)), n
        b = (rng.integers(-20, 20, n) * 0.25).astype(np.float32)
        b[rng.random(n) < 0.1] = -0.0
        assert np.array_equal(run_gpu(plan, b, le=le), oracle.apse(b, le)), n
        c = -np.arange(n, dtype=np.float32) * 1.5 + 7.0  # strictly descending through zero
        assert np.array_equal(run_gpu(plan, c, le=le), oracle.apse(c, le)), n


@pytest.mark.parametrize("offset", [1, 2, 3])
def test_unaligned_buffers(plans, offset):
    rng = np.random.default_rng(offset)
    plan = plans[torch.int32]
    for n in (5000, 123457):
        for name in ("uniform", "desc", "asc"):
            a = dist(name, n, rng)
            assert np.array_equal(run_gpu(plan, a, offset=offset), oracle.apse(a)), (name, n)


@pytest.mark.parametrize("oin,oout", [(1, 1), (2, 2), (3, 3), (1, 2), (3, 0), (0, 2)])
@pytest.mark.parametrize("le", [False, True])
def test_misaligned_views(plans, oin, oout, le):
    """Buffers off their 16-byte alignment.  Equal offsets stream through TMA
    behind 1-3 virtual keys (tile 0 takes plain loads and stores); unequal
    offsets take the plain path throughout.  Nothing outside out[0:n] is
    written (the words around it stay poisoned)."""
    rng = np.random.default_rng(oin * 7 + oout + (100 if le else 0))
    plan = plans[torch.int32]
    for n in (1, 511, 5000, 3_000_001):  # 3e6 keys: multi-tile ranges, whole-tile early paths
        for name in ("uniform", "desc", "asc", "dup16"):
            a = dist(name, n, rng)
            xb = torch.zeros(n + 4, dtype=torch.int32, device="cuda")
            xb[oin:oin + n] = torch.from_numpy(a).cuda()
            ob = torch.full((n + 4,), int(POISON), dtype=torch.int32, device="cuda")
            plan.run(xb[oin:oin + n], out=ob[oout:oout + n], n=n, inclusive=le)
            plan.check()
            got = ob.cpu().numpy()
            assert np.array_equal(got[oout:oout + n], oracle.apse(a, le)), (name, n)
            assert (got[:oout] == POISON).all() and (got[oout + n:] == POISON).all(), (name, n)


def test_misaligned_float_view(plans):
    rng = np.random.default_rng(41)
    plan = plans[torch.float32]
    n = 1_000_003
    a = (rng.integers(0, 1 << 24, n) * (2e6 / (1 << 24)) - 1e6).astype(np.float32)
    xb = torch.zeros(n + 4, dtype=torch.float32, device="cuda")
    xb[2:2 + n] = torch.from_numpy(a).cuda()
    ob = torch.full((n + 4,), int(POISON), dtype=torch.int32, device="cuda")
    plan.run(xb[2:2 + n], out=ob[2:2 + n])
    plan.check()
    got = ob.cpu().numpy()
    assert np.array_equal(got[2:2 + n], oracle.apse(a))
    assert (got[:2] == POISON).all() and (got[2 + n:] == POISON).all()


def test_pointer_not_4_byte_aligned_is_einval(plans):
    plan = plans[torch.int32]
    x = torch.zeros(1000, dtype=torch.int32, device="cuda")
    o = torch.zeros(1000, dtype=torch.int32, device="cuda")
    lib = _lib.load()
    assert lib.apsep_run(plan._h, x.data_ptr() + 2, o.data_ptr(), 100, None) == _lib.APSEP_EINVAL
    assert lib.apsep_run(plan._h, x.data_ptr(), o.data_ptr() + 1, 100, None) == _lib.APSEP_EINVAL


@pytest.mark.parametrize("name", ["uniform", "desc", "asc", "dup16"])
def test_full_size_2_25(plans, name):
    n = 1 << 25
    a = dist(name, n, np.random.default_rng(25))
    got = run_gpu(plans[torch.int32], a)
    assert np.array_equal(got, oracle.apse(a))


def test_maximum_size_closed_forms():
    """n = APSEP_MAX_KEYS (2^31 - 4096, the largest n whose tile ends stay in
    int32): ascending keys answer i - 1, descending keys -1, checked on the
    device (the arrays hold 8.6 GB each); then the same n behind a 1-key view
    head (off a 16-byte boundary)."""
    n = _lib.MAX_KEYS
    with Plan(n, torch.int32) as plan:
        x = torch.arange(n, dtype=torch.int32, device="cuda")
        out = torch.empty(n + 1, dtype=torch.int32, device="cuda")
        plan.run(x, out=out[:n])
        plan.check()
        assert int(out[0]) == -1
        assert bool((out[1:n] == x[:n - 1]).all())
        del x
        torch.cuda.empty_cache()
        xd = torch.arange(n, 0, -1, dtype=torch.int32, device="cuda")
        plan.run(xd, out=out[:n])
        plan.check()
        assert bool((out[:n] == -1).all())
        del xd
        torch.cuda.empty_cache()
        xb = torch.empty(n + 1, dtype=torch.int32, device="cuda")
        torch.arange(n, out=xb[1:])
        out.fill_(7)
        plan.run(xb[1:], out=out[1:])
        plan.check()
        assert int(out[0]) == 7 and int(out[1]) == -1
        assert bool((out[2:] == xb[1:n]).all())


def test_repeated_runs_reuse_plan(plans):
    # the run-to-run control block (tile counter, epoch) resets itself
    plan = plans[torch.int32]
    rng = np.random.default_rng(3)
    a = dist("uniform", 300001, rng)
    want = oracle.apse(a)
    x = torch.from_numpy(a).cuda()
    out = torch.empty_like(x)
    for _ in range(50):
        out.fill_(int(POISON))
        plan.run(x, out=out)
    plan.check()
    assert np.array_equal(out.cpu().numpy(), want)


def test_cuda_graph_capture(plans):
    plan = plans[torch.int32]
    n = 200003
    rng = np.random.default_rng(4)
    x = torch.empty(n, dtype=torch.int32, device="cuda")
    out = torch.empty_like(x)
    x.copy_(torch.from_numpy(dist("uniform", n, rng)))
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run(x, out=out)  # warm-up outside capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run(x, out=out)
    for name in ("uniform", "desc", "dup16"):
        a = dist(name, n, rng)
        x.copy_(torch.from_numpy(a))
        out.fill_(int(POISON))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), oracle.apse(a)), name
    plan.check()


def test_lookback_timeout_is_reported_not_hung():
    """A predecessor range that never publishes: the successors' bounded
    waits give up, the run finishes, the host reads APSEP_ETIMEOUT, and the
    next run on the same plan is correct again.  (48 tiles -> 48 one-tile ranges.)"""
    n = 4096 * 6
    a = dist("uniform", n, np.random.default_rng(8))
    with Plan(n, torch.int32) as plan:
        x = torch.from_numpy(a).cuda()
        out = torch.empty_like(x)
        plan.debug_inject(range_index=2, spin_limit=2000)
        plan.run(x, out=out)
        with pytest.raises(ApsepError) as ei:
            plan.check()
        assert ei.value.status == _lib.APSEP_ETIMEOUT
        plan.run(x, out=out)
        plan.check()
        assert np.array_equal(out.cpu().numpy(), oracle.apse(a))


def test_invalid_arguments_are_statuses(plans):
    plan = plans[torch.int32]
    x = torch.zeros(100, dtype=torch.int32, device="cuda")
    lib = _lib.load()
    # n beyond capacity
    with Plan(50, torch.int32) as small:
        st = lib.apsep_run(small._h, x.data_ptr(), x.data_ptr() + 4096, 100, None)
        assert st == _lib.APSEP_EINVAL
    # overlapping in/out
    st = lib.apsep_run(plan._h, x.data_ptr(), x.data_ptr() + 8, 100, None)
    assert st == _lib.APSEP_EINVAL
    # n == 0 no-op
    assert lib.apsep_run(plan._h, x.data_ptr(), x.data_ptr(), 0, None) == _lib.APSEP_OK
