"""The engine sharing the GPU: runs on one stream while another stream keeps
the SMs busy with long matrix products, and runs of two plans on two streams
at once.  The persistent launch is sized from occupancy as if it had the
device to itself, so here part of its grid may start only after other work
leaves; the look-back falls back to waiting on earlier ranges, which have all
started (range ids go out in start order), so the answers stay exact and no
wait can depend on a CTA that has not started."""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan

pytestmark = pytest.mark.gpu

N = 1 << 24


def keys(seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 1 << 31, N).astype(np.int32)


def test_runs_beside_a_busy_stream():
    a = keys(1)
    want = oracle.apse(a)
    x = torch.from_numpy(a).cuda()
    m = torch.randn(6144, 6144, device="cuda")
    side = torch.cuda.Stream()
    with Plan(N, torch.int32, tuning=None) as plan:
        outs = []
        side.wait_stream(torch.cuda.current_stream())
        for _ in range(4):
            with torch.cuda.stream(side):
                m = (m @ m).clamp_(-1, 1)
            outs.append(plan.run(x))
        plan.check()
        torch.cuda.synchronize()
        for o in outs:
            assert np.array_equal(o.cpu().numpy(), want)


def test_two_plans_on_two_streams():
    a, b = keys(2), keys(3)
    wa, wb = oracle.apse(a), oracle.apse(b, True)
    xa, xb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    s1.wait_stream(torch.cuda.current_stream())
    s2.wait_stream(torch.cuda.current_stream())
    with Plan(N, torch.int32, tuning=None) as pa, Plan(N, torch.int32, inclusive=True, tuning=None) as pb:
        oa, ob = [], []
        for _ in range(4):
            with torch.cuda.stream(s1):
                oa.append(pa.run(xa))
            with torch.cuda.stream(s2):
                ob.append(pb.run(xb))
        pa.check(s1)
        pb.check(s2)
        torch.cuda.synchronize()
        for o in oa:
            assert np.array_equal(o.cpu().numpy(), wa)
        for o in ob:
            assert np.array_equal(o.cpu().numpy(), wb)
