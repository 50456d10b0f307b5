"""GPU parity of the batched segmented run (apsep_run_segmented).

Every array of the batch is checked bit-exactly against the CPU oracle's
per-segment APSE (answers relative to the segment start).  Segment lengths
cover the shapes that stress the segment cursor: empty segments, one-key
segments, many segment starts inside one warp tile, segments exactly one tile
long, and segments spanning many ranges (so deferred keys search earlier
ranges of their own segment and must not see the previous segment).
"""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import ApsepError, Plan, _lib, apse_segmented

pytestmark = pytest.mark.gpu

POISON = int(np.uint32(0xABABABAB).view(np.int32))


def keys(dist, n, rng):
    if dist == "uniform":
        return rng.integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
    if dist == "desc":
        return np.arange(n - 1, -1, -1, dtype=np.int32)
    if dist == "asc":
        return np.arange(n, dtype=np.int32)
    if dist == "dup16":
        return rng.integers(0, 16, n).astype(np.int32)
    if dist == "saw":
        return (np.arange(n) % 257).astype(np.int32)
    if dist == "runs":  # strictly descending runs of random length, random starts
        out = np.empty(n, dtype=np.int32)
        i = 0
        while i < n:
            L = int(rng.integers(1, 4097))
            start = int(rng.integers(L, 1 << 30))
            m = min(L, n - i)
            out[i:i + m] = start - np.arange(m)
            i += m
        return out
    raise KeyError(dist)


def batch(lengths, dists, rng):
    parts = [keys(dists[i % len(dists)], int(L), rng) for i, L in enumerate(lengths)]
    a = np.concatenate(parts) if parts else np.zeros(0, np.int32)
    offs = np.zeros(len(lengths) + 1, dtype=np.int64)
    offs[1:] = np.cumsum(lengths)
    return a, offs


def run(plan, a, offs, out_poison=True):
    x = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    o = torch.from_numpy(offs).cuda()
    out = torch.full((a.shape[0],), POISON if out_poison else 0, dtype=torch.int32, device="cuda")
    plan.run_segmented(x, o, out=out)
    plan.check()
    return out.cpu().numpy()


def check(plan, a, offs, le=False):
    got = run(plan, a, offs)
    want = oracle.apse_segmented(a, offs, le)
    if not np.array_equal(got, want):
        bad = int(np.flatnonzero(got != want)[0])
        seg = int(np.searchsorted(offs, bad, side="right") - 1)
        pytest.fail("first mismatch at %d (segment %d [%d, %d)): got %d want %d" %
                    (bad, seg, offs[seg], offs[seg + 1], got[bad], want[bad]))


EDGE_LENGTHS = [0, 1, 2, 3, 31, 32, 33, 63, 64, 65, 255, 256, 257, 511, 512, 513, 1000, 1023, 1024, 1025, 4096,
                5000, 0, 0, 1, 17]


@pytest.mark.parametrize("le", [False, True])
@pytest.mark.parametrize("dist", ["uniform", "desc", "asc", "dup16", "saw"])
def test_edge_lengths(dist, le):
    rng = np.random.default_rng(11)
    lengths = list(EDGE_LENGTHS) * 3
    rng.shuffle(lengths)
    a, offs = batch(lengths, [dist], rng)
    with Plan(a.shape[0], torch.int32, inclusive=le) as plan:
        check(plan, a, offs, le)


@pytest.mark.parametrize("dist", ["uniform", "dup16", "asc", "desc"])
def test_many_tiny_segments(dist):
    # tens of segment starts inside every warp tile
    rng = np.random.default_rng(12)
    lengths = rng.integers(0, 9, 60000)
    a, offs = batch(lengths, [dist], rng)
    with Plan(a.shape[0], torch.int32) as plan:
        check(plan, a, offs)


def test_log_uniform_mixed_batch():
    # the batched benchmark's shape, smaller: log-uniform lengths, segment s
    # uniform / descending runs / sawtooth by s % 3
    rng = np.random.default_rng(13)
    lengths = np.round(np.exp(rng.uniform(np.log(32), np.log(1 << 16), 600))).astype(np.int64)
    a, offs = batch(lengths, ["uniform", "runs", "saw"], rng)
    for le in (False, True):
        with Plan(a.shape[0], torch.int32, inclusive=le) as plan:
            check(plan, a, offs, le)


@pytest.mark.parametrize("dist", ["uniform", "dup16", "runs"])
def test_segments_spanning_many_ranges(dist):
    # a few huge segments: deferred keys of later ranges search earlier ranges
    # of their own segment, and must stop at its start
    rng = np.random.default_rng(14)
    lengths = [3 << 20, 1 << 20, 77777, 5 << 20, 1]
    a, offs = batch(lengths, [dist], rng)
    with Plan(a.shape[0], torch.int32) as plan:
        check(plan, a, offs)


@pytest.mark.parametrize("shift", [1, 2, 3])
def test_misaligned_batch_base(shift):
    """A batch whose keys and answers start 4*shift bytes past a 16-byte
    boundary (the view adds virtual keys in front; offsets stay relative to
    the batch).  The words before the answers stay untouched."""
    rng = np.random.default_rng(shift)
    lengths = np.array([int(x) for x in np.exp(rng.uniform(np.log(1), np.log(300000), 60))], dtype=np.int64)
    lengths[:5] = [0, 1, 2, 3, 5]
    a, offs = batch(lengths, ["uniform", "desc", "asc", "runs", "dup16"], rng)
    n = a.shape[0]
    xb = torch.zeros(n + 4, dtype=torch.int32, device="cuda")
    xb[shift:shift + n] = torch.from_numpy(a).cuda()
    for le in (False, True):
        ob = torch.full((n + 4,), POISON, dtype=torch.int32, device="cuda")
        with Plan(n, torch.int32, inclusive=le) as plan:
            plan.run_segmented(xb[shift:shift + n], torch.from_numpy(offs).cuda(), out=ob[shift:shift + n])
            plan.check()
        got = ob.cpu().numpy()
        assert np.array_equal(got[shift:shift + n], oracle.apse_segmented(a, offs, le))
        assert (got[:shift] == POISON).all() and (got[shift + n:] == POISON).all()


def test_one_segment_equals_single_run():
    rng = np.random.default_rng(15)
    a = keys("uniform", 1000003, rng)
    offs = np.array([0, a.shape[0]], dtype=np.int64)
    with Plan(a.shape[0], torch.int32) as plan:
        assert np.array_equal(run(plan, a, offs), oracle.apse(a))


@pytest.mark.parametrize("le", [False, True])
def test_float_segments(le):
    rng = np.random.default_rng(16)
    lengths = rng.integers(0, 3000, 400)
    parts = [(-1e6 + rng.integers(0, 1 << 24, int(L)) * (2e6 / (1 << 24))).astype(np.float32) for L in lengths]
    a = np.concatenate(parts)
    a[rng.random(a.shape[0]) < 0.05] = -0.0
    offs = np.zeros(len(lengths) + 1, dtype=np.int64)
    offs[1:] = np.cumsum(lengths)
    with Plan(a.shape[0], torch.float32, inclusive=le) as plan:
        check(plan, a, offs, le)


@pytest.mark.parametrize("config", range(_lib.NUM_CONFIGS))
def test_every_config(config):
    rng = np.random.default_rng(17 + config)
    lengths = list(rng.integers(0, 40000, 60)) + EDGE_LENGTHS
    a, offs = batch(lengths, ["uniform", "runs", "saw", "dup16"], rng)
    with Plan(a.shape[0], torch.int32) as plan:
        plan.set_config(config)
        check(plan, a, offs)


def test_convenience_call_and_repeats():
    rng = np.random.default_rng(18)
    lengths = rng.integers(1, 20000, 50)
    a, offs = batch(lengths, ["uniform"], rng)
    x = torch.from_numpy(a).cuda()
    o = torch.from_numpy(offs).cuda()
    want = oracle.apse_segmented(a, offs)
    for _ in range(5):
        got = apse_segmented(x, o)
        torch.cuda.synchronize()
        assert np.array_equal(got.cpu().numpy(), want)


def test_segmented_graph_capture():
    rng = np.random.default_rng(19)
    lengths = rng.integers(0, 5000, 300)
    a, offs = batch(lengths, ["uniform"], rng)
    n = a.shape[0]
    with Plan(n, torch.int32) as plan:
        x = torch.from_numpy(a).cuda()
        o = torch.from_numpy(offs).cuda()
        out = torch.empty(n, dtype=torch.int32, device="cuda")
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            plan.run_segmented(x, o, out=out)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            plan.run_segmented(x, o, out=out)
        for dist in ("dup16", "runs", "uniform"):
            b, _ = batch(lengths, [dist], rng)
            x.copy_(torch.from_numpy(b))
            out.fill_(POISON)
            g.replay()
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy(), oracle.apse_segmented(b, offs)), dist
        plan.check()


def test_bad_offsets_are_reported():
    rng = np.random.default_rng(20)
    a, offs = batch([100, 200, 300], ["uniform"], rng)
    with Plan(a.shape[0], torch.int32) as plan:
        b1 = offs.copy()
        b1[-1] = a.shape[0] - 1  # does not end at n
        b2 = offs.copy()
        b2[0] = 1  # does not start at 0
        for b in (b1, b2):
            x = torch.from_numpy(a).cuda()
            o = torch.from_numpy(b).cuda()
            plan.run_segmented(x, o)
            with pytest.raises(ApsepError) as ei:
                plan.check()
            assert ei.value.status == _lib.APSEP_EINVAL
        check(plan, a, offs)  # the plan still works


def test_invalid_segmented_arguments():
    lib = _lib.load()
    x = torch.zeros(100, dtype=torch.int32, device="cuda")
    out = torch.zeros(100, dtype=torch.int32, device="cuda")
    o = torch.tensor([0, 50, 100], dtype=torch.int64, device="cuda")
    with Plan(100, torch.int32) as plan:
        assert lib.apsep_run_segmented(plan._h, x.data_ptr(), out.data_ptr(), 100, o.data_ptr(), 0,
                                       None) == _lib.APSEP_EINVAL  # nseg < 1
        assert lib.apsep_run_segmented(plan._h, x.data_ptr(), out.data_ptr(), 100, None, 2,
                                       None) == _lib.APSEP_EINVAL  # no offsets
        assert lib.apsep_run_segmented(plan._h, x.data_ptr(), out.data_ptr(), 100, o.data_ptr() + 4, 2,
                                       None) == _lib.APSEP_EINVAL  # misaligned offsets
        assert lib.apsep_run_segmented(plan._h, x.data_ptr(), out.data_ptr(), 0, o.data_ptr(), 2,
                                       None) == _lib.APSEP_OK  # n == 0 no-op
