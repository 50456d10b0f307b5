"""GPU: the serving loop and the autotuner.  Every answer the server returns
is checked bit-exactly against the CPU oracle."""
import numpy as np
import pytest
import torch

import oracle
from apsep_gb300 import Plan, autotune
from apsep_gb300.serve import ResidentServer, Server, plain_loop, resident_loop
from apsep_gb300.workloads import resident_requests, serve_requests

pytestmark = pytest.mark.gpu


def oracle_of(r):
    return oracle.apse(r.keys.numpy(), r.inclusive)


@pytest.fixture(scope="module")
def server():
    s = Server(budget_bytes=1 << 30, slot_keys=4 << 20, max_segments=256)
    yield s
    s.close()


def test_served_answers_match_oracle(server):
    reqs = serve_requests(80, rate=2000.0, seed=5, hi=1 << 20)
    st = server.serve(reqs, keep_answers=True)
    assert st.requests == 80 and st.batches >= 1
    assert st.device_bytes <= server.budget_bytes
    for r in reqs:
        assert r.t_done is not None and r.t_done >= r.arrival
        assert np.array_equal(r.answers, oracle_of(r)), r.rid
    assert st.p99_ms >= st.p50_ms > 0


def test_saturated_batches_and_plain_loop_agree(server):
    reqs = serve_requests(60, rate=0.0, seed=6, hi=1 << 19)
    st = server.serve(reqs, keep_answers=True, realtime=False)
    got = {r.rid: r.answers for r in reqs}
    base = serve_requests(60, rate=0.0, seed=6, hi=1 << 19)
    plain_loop(base, keep_answers=True, realtime=False)
    for r in base:
        assert np.array_equal(got[r.rid], r.answers), r.rid
    assert st.batches < 60  # saturation packs several requests per launch


def test_budget_and_capacity_are_enforced():
    with pytest.raises(ValueError):
        Server(budget_bytes=1 << 10)
    s = Server(budget_bytes=256 << 20, slot_keys=1 << 16, max_segments=16)
    try:
        big = serve_requests(1, rate=0.0, seed=7, lo=1 << 17, hi=1 << 18)
        with pytest.raises(ValueError):
            s.serve(big)
    finally:
        s.close()


def test_autotune_table_and_tuned_plan():
    table = autotune.tune(dtype=torch.int32, classes=[14, 16], reps=1)
    assert set(table.entries) == {14, 16}
    assert all(0 <= c < autotune.num_configs() for c in table.entries.values())
    rng = np.random.default_rng(3)
    with Plan(1 << 17, torch.int32, tuning=table) as p:
        for n in (1 << 14, 1 << 16, 100003):
            a = rng.integers(0, 1 << 31, n, dtype=np.int64).astype(np.int32)
            out = p.run(torch.from_numpy(a).cuda())
            p.check()
            assert np.array_equal(out.cpu().numpy(), oracle.apse(a))


@pytest.mark.parametrize("dtype", [torch.int32, torch.float32])
def test_resident_server_matches_oracle_and_loop(dtype):
    keys, answers, reqs = resident_requests(120, rate=0.0, seed=9, hi=1 << 18, dtype=dtype)
    srv = ResidentServer(keys, answers, max_batch_keys=1 << 20, max_segments=64)
    try:
        st = srv.serve(reqs, realtime=False)
    finally:
        srv.close()
    assert st.requests == 120 and st.batches < 120
    got = answers.cpu().numpy()
    k = keys.cpu().numpy()
    for r in reqs[::7]:  # a sample of the requests, each checked in full
        assert np.array_equal(got[r.start:r.start + r.n], oracle.apse(k[r.start:r.start + r.n])), r.rid
    answers.fill_(-7)
    resident_loop(keys, answers, reqs, realtime=False)
    loop = answers.cpu().numpy()
    for r in reqs:
        assert r.start % 4 == 0
        assert np.array_equal(loop[r.start:r.start + r.n], got[r.start:r.start + r.n]), r.rid
