"""Host logic of the serving loop (no GPU): the ring allocator of the pools
(spans, wrap-around, reclamation from the tail) and the latency statistics."""
import pytest

torch = pytest.importorskip("torch")

from apsep_gb300.serve import ServeStats  # noqa: E402


def test_stats():
    s = ServeStats(requests=4, keys=400, makespan_s=2.0, latencies_ms=[1.0, 2.0, 3.0, 100.0], batches=2,
                   device_bytes=10)
    assert s.requests_per_s == 2.0 and s.keys_per_s == 200.0
    assert s.p50_ms == pytest.approx(2.5)
    assert s.p99_ms > 90.0
    d = s.as_dict()
    assert d["useful_gbs"] == round(8 * 200 / 1e9, 2) and d["batches"] == 2


def test_ring_pool_allocates_wraps_and_reclaims():
    from apsep_gb300.serve import RingPool
    p = RingPool(100, align=4)
    assert p.capacity == 100
    a = p.alloc(30)   # 32 slots
    b = p.alloc(50)   # 52
    assert (a, b) == (0, 32)
    assert p.alloc(20) is None          # 84 + 20 > 100 and nothing free at the tail yet
    c = p.alloc(13)                     # 16 -> 84..100
    assert c == 84 and p.used == 100
    assert p.alloc(1) is None           # full
    p.free(b)                           # out of order: the tail stays at 0
    assert p.used == 100 and p.alloc(4) is None
    p.free(a)                           # tail reclaimed up to c
    assert p.used == 16
    d = p.alloc(60)                     # wraps to the start
    assert d == 0
    assert p.alloc(30) is None          # only 84 - 60 = 24 free before the tail
    e = p.alloc(24)
    assert e == 60 and p.used == 100
    p.free(c)
    p.free(d)
    p.free(e)
    assert p.used == 0 and p.alloc(100) == 0


def test_ring_pool_spans_are_aligned_and_never_overlap():
    import random
    from apsep_gb300.serve import RingPool
    rnd = random.Random(5)
    p = RingPool(1000, align=4)
    live = {}
    for _ in range(5000):
        if live and (rnd.random() < 0.45 or len(live) > 20):
            s = rnd.choice(list(live))
            p.free(s)
            del live[s]
        else:
            n = rnd.randint(0, 300)
            s = p.alloc(n)
            if s is not None:
                size = p.span_size(n)
                assert s % 4 == 0 and s + size <= 1000
                for t, z in live.items():
                    assert s + size <= t or t + z <= s
                live[s] = size
    assert p.alloc(2000) is None
