"""Host logic of the serving loop (no GPU): FIFO admission by slot capacity
and segment count, and the latency statistics."""
import collections

import pytest

torch = pytest.importorskip("torch")

from apsep_gb300.serve import BatchPlanner, Request, ServeStats  # noqa: E402


def req(i, n):
    return Request(rid=i, keys=torch.empty(n, dtype=torch.int32))


def test_takes_longest_fitting_prefix_in_arrival_order():
    p = BatchPlanner(capacity_keys=100, max_segments=10)
    q = collections.deque([req(0, 40), req(1, 50), req(2, 20), req(3, 5)])
    b = p.take(q)
    assert [r.rid for r in b] == [0, 1]          # 90 keys; request 2 would overflow
    assert [r.rid for r in q] == [2, 3]          # FIFO order kept, no overtaking
    assert [r.rid for r in p.take(q)] == [2, 3]


def test_segment_limit_and_empty_requests():
    p = BatchPlanner(capacity_keys=1000, max_segments=3)
    q = collections.deque([req(i, 0 if i % 2 else 7) for i in range(7)])
    assert [r.rid for r in p.take(q)] == [0, 1, 2]
    assert len(q) == 4


def test_oversized_request_is_not_admissible():
    p = BatchPlanner(capacity_keys=64, max_segments=8)
    assert p.fits(64) and not p.fits(65)
    q = collections.deque([req(0, 65), req(1, 1)])
    assert p.take(q) == []                       # the head does not fit: nothing overtakes it
    assert len(q) == 2


def test_stats():
    s = ServeStats(requests=4, keys=400, makespan_s=2.0, latencies_ms=[1.0, 2.0, 3.0, 100.0], batches=2,
                   device_bytes=10)
    assert s.requests_per_s == 2.0 and s.keys_per_s == 200.0
    assert s.p50_ms == pytest.approx(2.5)
    assert s.p99_ms > 90.0
    d = s.as_dict()
    assert d["useful_gbs"] == round(8 * 200 / 1e9, 2) and d["batches"] == 2
