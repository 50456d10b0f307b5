"""GPU: continuous batching over device-resident pools (PoolServer).

The served workload's mixed stream (int32 / float32 50/50, lengths
log-uniform up to 2^24) through rings much smaller than the stream, so ring
space is reclaimed and reused while requests keep arriving.  Every answer is
checked bit-exactly against the CPU oracle, and a sample of requests is run
again alone (one apsep_run each) to show that a result is the same alone and
in the mix."""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan
from apsep_gb300.serve import PoolServer, device_loop
from apsep_gb300.workloads import pool_requests

pytestmark = pytest.mark.gpu


def host_keys(r):
    return r.keys.cpu().numpy() if r.keys.is_cuda else r.keys.numpy()


@pytest.mark.parametrize("realtime", [False, True])
def test_mixed_stream_through_small_rings(realtime):
    reqs = pool_requests(48, rate=4000.0, seed=31, hi=1 << 24)
    ring = 3 << 20
    srv = PoolServer(budget_bytes=1 << 30, max_batch_keys=1 << 24, ring_keys=ring, direct_min_keys=2 << 20)
    try:
        st = srv.serve(reqs, keep_answers=True, realtime=realtime)
    finally:
        srv.close()
    assert st.requests == 48 and st.device_bytes <= 1 << 30
    batched = [r for r in reqs if r.n < (2 << 20)]
    direct = [r for r in reqs if r.n >= (2 << 20)]
    assert direct and sum(r.n for r in batched) > 2 * ring  # the rings were reused
    assert {r.keys.dtype for r in reqs} == {torch.int32, torch.float32}
    for r in reqs:
        assert not r.failed and r.t_done is not None
        assert np.array_equal(r.answers, oracle.apse(host_keys(r))), r.rid
    for r in reqs[::6]:  # alone: one single-array run each
        with Plan(r.n, r.keys.dtype) as p:
            alone = p.run(r.keys).cpu().numpy()
            p.check()
        assert np.array_equal(alone, r.answers), r.rid


def test_everything_batched_and_the_plain_loop_agree():
    reqs = pool_requests(60, rate=0.0, seed=32, hi=1 << 20)
    srv = PoolServer(budget_bytes=256 << 20, max_batch_keys=1 << 21, ring_keys=1 << 21)
    try:
        st = srv.serve(reqs, keep_answers=True, realtime=False)
    finally:
        srv.close()
    got = {r.rid: r.answers for r in reqs}
    assert st.batches < 60
    for r in reqs:
        r.out.fill_(-7)
    device_loop(reqs, realtime=False)
    for r in reqs:
        assert np.array_equal(r.out.cpu().numpy(), got[r.rid]), r.rid
        assert np.array_equal(got[r.rid], oracle.apse(host_keys(r))), r.rid


def test_host_keys_and_host_answers():
    reqs = pool_requests(30, rate=0.0, seed=33, hi=1 << 19, device_keys=False)
    srv = PoolServer(budget_bytes=128 << 20, max_batch_keys=1 << 20, ring_keys=1 << 20)
    try:
        srv.serve(reqs, keep_answers=True, realtime=False)
    finally:
        srv.close()
    for r in reqs:
        assert np.array_equal(r.answers, oracle.apse(host_keys(r))), r.rid


def test_a_failed_batch_is_marked_and_the_rest_stand():
    """A device-side wait that gives up (host-armed injection on one lane's
    plan, bounded waits) marks exactly the requests of that launch failed."""
    reqs = [r for r in pool_requests(40, rate=0.0, seed=34, lo=1 << 15, hi=1 << 17)
            if r.keys.dtype == torch.int32][:12]
    srv = PoolServer(budget_bytes=128 << 20, kinds=((torch.int32, False),), lanes_per_kind=1,
                     max_batch_keys=1 << 18, ring_keys=1 << 18)
    try:
        srv.lanes[(torch.int32, False)][0].plan.debug_inject(range_index=2, spin_limit=2000)
        srv.serve(reqs, keep_answers=True, realtime=False)
        failed = [r for r in reqs if r.failed]
        assert failed and len(failed) < len(reqs)
        assert failed == reqs[:len(failed)]  # the first launch
        for r in reqs[len(failed):]:
            assert np.array_equal(r.answers, oracle.apse(host_keys(r))), r.rid
        srv.serve(reqs, keep_answers=True, realtime=False)  # the plan was re-armed
        for r in reqs:
            assert not r.failed and np.array_equal(r.answers, oracle.apse(host_keys(r))), r.rid
    finally:
        srv.close()


def test_copy_spans_every_alignment_and_size():
    from apsep_gb300 import _lib
    src = torch.randint(0, 255, (1 << 22,), dtype=torch.uint8, device="cuda")
    dst = torch.zeros_like(src)
    rng = np.random.default_rng(3)
    spans, o = [], 0
    for n in [0, 1, 3, 15, 16, 17, 4096, 16384, 16385, 100000, 1 << 20]:
        # source and destination at independent offsets within 16 bytes
        spans.append((o + int(rng.integers(0, 16)), o + int(rng.integers(0, 16)), n))
        o += n + 64
    srcs = [src.data_ptr() + a for a, _, n in spans]
    dsts = [dst.data_ptr() + b for _, b, n in spans]
    _lib.copy_spans(srcs, dsts, [n for _, _, n in spans], torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    want = torch.zeros_like(src)
    for a, b, n in spans:
        want[b:b + n] = src[a:a + n]
    assert torch.equal(dst, want)
    # more spans than one launch carries, to pinned host memory
    host = torch.zeros(600 * 64, dtype=torch.uint8).pin_memory()
    _lib.copy_spans([src.data_ptr() + 64 * i + 3 for i in range(600)], [host.data_ptr() + 64 * i for i in range(600)],
                    [61] * 600, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h = host.numpy().reshape(600, 64)
    s2 = src.cpu().numpy()
    for i in range(600):
        assert np.array_equal(h[i, :61], s2[64 * i + 3:64 * i + 64])


def test_direct_runs_answer_into_the_ring():
    """Large requests run from their own keys (no copy into the pool); with no
    output buffer their answers land in a span of the answer ring, handed to
    on_done, while the small ones are batched around them."""
    reqs = pool_requests(32, rate=0.0, seed=35, hi=1 << 22)
    for r in reqs:
        r.out = None
    got = {}

    def done(r, answers):
        got[r.rid] = answers.cpu().numpy()

    srv = PoolServer(budget_bytes=1 << 30, max_batch_keys=1 << 22, ring_keys=5 << 20, direct_min_keys=1 << 20)
    try:
        st = srv.serve(reqs, realtime=False, on_done=done)
    finally:
        srv.close()
    assert st.requests == 32 and any(r.n >= 1 << 20 for r in reqs) and any(r.n < 1 << 20 for r in reqs)
    for r in reqs:
        assert not r.failed
        assert np.array_equal(got[r.rid], oracle.apse(host_keys(r))), r.rid
