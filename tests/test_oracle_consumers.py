"""The consumer oracles pinned against each other (CPU): the monotone-stack
restatements fix each definition, ties included; the compositions with the
C oracle's APSE (used for the large GPU parity cases) must agree with them."""
import numpy as np
import pytest

from oracle import consumers as oc


def arrays(rng):
    yield np.array([], dtype=np.int32)
    yield np.array([5], dtype=np.int32)
    yield np.array([1, 1, 1, 1], dtype=np.int32)
    yield np.array([3, 1, 3, 1, 3], dtype=np.int32)
    yield np.arange(50, dtype=np.int32)
    yield np.arange(50, 0, -1, dtype=np.int32)
    for n in (17, 200, 3001):
        yield rng.integers(0, 4, n).astype(np.int32)           # heavy ties
        yield rng.integers(-(1 << 31), 1 << 31, n, dtype=np.int64).astype(np.int32)
        yield (rng.integers(-8, 8, n) * 0.5).astype(np.float32)  # float ties, both zeros
    yield np.array([0.0, -0.0, 0.0, -0.0], dtype=np.float32)
    yield np.array([-(1 << 31), (1 << 31) - 1, -(1 << 31)], dtype=np.int32)


@pytest.mark.parametrize("le", [False, True])
def test_prev_greater_and_next_smaller(le):
    for a in arrays(np.random.default_rng(1)):
        assert np.array_equal(oc.prev_greater(a, le), oc.prev_greater_stack(list(a), le)), a
        assert np.array_equal(oc.next_smaller(a, le), oc.next_smaller_stack(list(a), le)), a


def test_stock_span_and_cartesian():
    for a in arrays(np.random.default_rng(2)):
        assert np.array_equal(oc.stock_span(a), oc.stock_span_stack(list(a))), a
        assert np.array_equal(oc.cartesian_parents(a), oc.cartesian_parents_stack(list(a))), a


def test_largest_rectangle():
    rng = np.random.default_rng(3)
    cases = [np.array([], np.int32), np.array([0], np.int32), np.array([2, 1, 5, 6, 2, 3], np.int32),
             np.array([4, 4, 4], np.int32), np.arange(30, dtype=np.int32)]
    cases += [rng.integers(0, k, n).astype(np.int32) for k in (2, 10, 1 << 20) for n in (1, 50, 2000)]
    for h in cases:
        assert oc.largest_rectangle(h) == oc.largest_rectangle_stack(list(h)), h
    assert oc.largest_rectangle(np.array([2, 1, 5, 6, 2, 3], np.int32)) == 10  # the textbook case


def test_cartesian_tie_rule():
    # a later equal key is the right child of an earlier one
    assert oc.cartesian_parents_stack([1, 1]).tolist() == [-1, 0]
    assert oc.cartesian_parents_stack([1, 3, 1]).tolist() == [-1, 2, 0]
    assert oc.cartesian_parents_stack([2, 3, 1]).tolist() == [2, 0, -1]
