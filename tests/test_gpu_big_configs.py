"""GPU parity at the full sizes of the benchmark configurations, checked
against the CPU oracle key by key (not only through properties):

  - the batch of the batched bench leg: 4096 segments with log-uniform lengths
    in [32, 2^20] (4.1e8 keys; uniform / descending runs / sawtooth), every
    segment;
  - uniform keys at N = 2^30, the top of the size sweep (4 GiB in, 4 GiB out);

(the served stream at its full length range, up to 2^24 keys and both key
types, is in test_gpu_pool_serve.py)."""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan
from apsep_gb300.workloads import batch_workload

pytestmark = pytest.mark.gpu


def test_bench_batch_every_segment():
    x, offs = batch_workload(4096, seed=7)
    n = x.numel()
    assert n > 4 * 10**8
    with Plan(n, torch.int32) as plan:
        d_offs = torch.from_numpy(offs).cuda()
        out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        plan.run_segmented(x, d_offs, out=out)
        plan.check()
        got = out.cpu().numpy()
    want = oracle.apse_segmented(x.cpu().numpy(), offs)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, "first mismatch at %d of %d" % (bad[0], n)


def test_uniform_2p30():
    n = 1 << 30
    g = torch.Generator(device="cuda")
    g.manual_seed(30)
    x = torch.randint(0, 1 << 31, (n,), generator=g, device="cuda", dtype=torch.int64).to(torch.int32)
    with Plan(n, torch.int32) as plan:
        out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        plan.run(x, out=out)
        plan.check()
        got = out.cpu().numpy()
    a = x.cpu().numpy()
    del x, out
    torch.cuda.empty_cache()
    want = oracle.apse(a)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, "first mismatch at %d of %d" % (bad[0], n)
