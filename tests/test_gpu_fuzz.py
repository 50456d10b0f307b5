"""Randomised differential test across the engine's forms: single arrays,
segmented batches and arrays off a 16-byte boundary, for every key type and
both comparators, against the CPU oracle.  Seeded: each case prints its
parameters on failure, so it replays exactly."""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan

pytestmark = pytest.mark.gpu

POISON = int(np.uint32(0xABABABAB).view(np.int32))
TYPES = [np.int32, np.float32, np.int64, np.float64]


def draw_keys(rng, n, dtype):
    kind = rng.integers(0, 6)
    if kind == 0:  # full range
        if dtype in (np.int32, np.int64):
            info = np.iinfo(dtype)
            return rng.integers(info.min, info.max, n, dtype=dtype, endpoint=True)
        return (rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30)).astype(dtype)
    if kind == 1:  # few distinct values (ties)
        return rng.integers(-3, 3, n).astype(dtype)
    if kind == 2:  # descending runs
        run = int(rng.integers(1, 5000))
        return (-(np.arange(n) % run) + rng.integers(0, 4, n)).astype(dtype)
    if kind == 3:  # ascending with noise
        return (np.arange(n) + rng.integers(-50, 50, n)).astype(dtype)
    if kind == 4:  # valley: one small key then a long climb down
        a = np.arange(n, 0, -1).astype(dtype)
        if n:
            a[int(rng.integers(0, n))] = -5
        return a
    return rng.integers(0, 1 << 20, n).astype(dtype)  # plain uniform


def run_case(rng, case):
    dtype = TYPES[int(rng.integers(0, 4))]
    le = bool(rng.integers(0, 2))
    n = int(np.exp(rng.uniform(0, np.log(400000))))
    a = np.ascontiguousarray(draw_keys(rng, n, dtype))
    segmented = bool(rng.integers(0, 2))
    off_in = int(rng.integers(0, 4)) if dtype in (np.int32, np.float32) else 2 * int(rng.integers(0, 2))
    off_out = off_in if rng.integers(0, 4) else int(rng.integers(0, 4))
    tdt = torch.from_numpy(a[:0]).dtype
    unit = 4 if dtype in (np.int32, np.float32) else 8
    elems_in = off_in * 4 // unit  # keys of offset (8-byte keys move by whole keys)
    xb = torch.zeros(n + 4, dtype=tdt, device="cuda")
    xb[elems_in:elems_in + n] = torch.from_numpy(a).cuda()
    ob = torch.full((n + 4,), POISON, dtype=torch.int32, device="cuda")
    x, out = xb[elems_in:elems_in + n], ob[off_out:off_out + n]
    what = "case %d: %s n=%d le=%s seg=%s off_in=%d off_out=%d" % (case, dtype.__name__, n, le, segmented,
                                                                   elems_in, off_out)
    with Plan(max(n, 1), tdt, inclusive=le) as plan:
        if segmented and n:
            cuts = np.sort(rng.integers(0, n + 1, int(rng.integers(1, 60))))
            offs = np.concatenate([[0], cuts, [n]]).astype(np.int64)
            plan.run_segmented(x, torch.from_numpy(offs).cuda(), out=out)
            want = np.concatenate([oracle.apse(np.ascontiguousarray(a[s0:s1]), le) if s1 > s0
                                   else np.zeros(0, np.int32) for s0, s1 in zip(offs[:-1], offs[1:])])
        else:
            plan.run(x, out=out, n=n)
            want = oracle.apse(a, le)
        plan.check()
    got = ob.cpu().numpy()
    body = got[off_out:off_out + n]
    if not np.array_equal(body, want):
        bad = int(np.flatnonzero(body != want)[0])
        pytest.fail("%s: first mismatch at %d: got %d want %d" % (what, bad, body[bad], want[bad]))
    assert (got[:off_out] == POISON).all() and (got[off_out + n:] == POISON).all(), what


@pytest.mark.parametrize("seed", range(40))
def test_random_forms_against_the_oracle(seed):
    rng = np.random.default_rng(1000 + seed)
    for case in range(12):
        run_case(rng, case)
