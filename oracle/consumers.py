"""CPU oracles for the consumers of APSE -- TEST INFRASTRUCTURE ONLY.

Two independent restatements of each consumer the reference names for its
output (README.md:3, src/bench_spt_le.cu:1-3):
  *_stack   the textbook one-pass monotone-stack algorithms, pure Python
            (small inputs only: they pin the definitions, ties included);
  the rest  compositions of the C oracle's APSE with numpy (order reversal,
            array reversal), for inputs the size of the engine's tests.
"""
from __future__ import annotations

import numpy as np

from . import apse


# ---- monotone-stack restatements (pure Python) -----------------------------
def prev_greater_stack(a, le: bool = False) -> np.ndarray:
    """max{j < i : a[j] > a[i]} (>= when le), else -1."""
    out, st = [], []
    for i, x in enumerate(a):
        while st and (a[st[-1]] < x if le else a[st[-1]] <= x):
            st.pop()
        out.append(st[-1] if st else -1)
        st.append(i)
    return np.array(out, dtype=np.int32)


def next_smaller_stack(a, le: bool = False) -> np.ndarray:
    """min{j > i : a[j] < a[i]} (<= when le), else -1."""
    n = len(a)
    out = [-1] * n
    st = []
    for j in range(n):
        while st and (a[j] <= a[st[-1]] if le else a[j] < a[st[-1]]):
            out[st.pop()] = j
        st.append(j)
    return np.array(out, dtype=np.int32)


def stock_span_stack(a) -> np.ndarray:
    """The number of consecutive keys ending at i that are <= a[i]."""
    out, st = [], []
    for i, x in enumerate(a):
        while st and a[st[-1]] <= x:
            st.pop()
        out.append(i - (st[-1] if st else -1))
        st.append(i)
    return np.array(out, dtype=np.int32)


def largest_rectangle_stack(h) -> int:
    """Largest rectangle under the histogram of non-negative heights."""
    best, st = 0, []
    for i in range(len(h) + 1):
        x = h[i] if i < len(h) else -1
        while st and h[st[-1]] >= x:
            top = st.pop()
            left = st[-1] if st else -1
            best = max(best, int(h[top]) * (i - left - 1))
        st.append(i)
    return best


def cartesian_parents_stack(a) -> np.ndarray:
    """Min-rooted Cartesian tree by the stack construction (pop keys greater
    than the new one; the last popped becomes its left child; it becomes the
    right child of the new top): a later equal key is the right child of an
    earlier one.  -1 at the root."""
    n = len(a)
    parent = [-1] * n
    st = []
    for i in range(n):
        last = -1
        while st and a[st[-1]] > a[i]:
            last = st.pop()
        if last != -1:
            parent[last] = i
        if st:
            parent[i] = st[-1]
        st.append(i)
    return np.array(parent, dtype=np.int32)


# ---- compositions with the C oracle (any size) -----------------------------
def _flip(a: np.ndarray) -> np.ndarray:
    return ~a if np.issubdtype(a.dtype, np.integer) else -a


def prev_greater(a: np.ndarray, le: bool = False) -> np.ndarray:
    return apse(_flip(np.ascontiguousarray(a)), le)


def next_smaller(a: np.ndarray, le: bool = False) -> np.ndarray:
    n = a.shape[0]
    r = apse(np.ascontiguousarray(a[::-1]), le)[::-1]
    return np.where(r >= 0, n - 1 - r, -1).astype(np.int32)


def stock_span(a: np.ndarray) -> np.ndarray:
    return (np.arange(a.shape[0], dtype=np.int64) - prev_greater(a, False)).astype(np.int32)


def largest_rectangle(h: np.ndarray) -> int:
    n = h.shape[0]
    if n == 0:
        return 0
    left = apse(np.ascontiguousarray(h), False).astype(np.int64)
    right = next_smaller(h, False).astype(np.int64)
    right = np.where(right < 0, n, right)
    return int(max(0, (h.astype(np.int64) * (right - left - 1)).max()))


def cartesian_parents(a: np.ndarray) -> np.ndarray:
    left = apse(np.ascontiguousarray(a), True).astype(np.int64)
    right = next_smaller(a, False).astype(np.int64)
    lv = a[np.maximum(left, 0)]
    rv = a[np.maximum(right, 0)]
    p = np.where(right < 0, left, np.where(left < 0, right, np.where(rv >= lv, right, left)))
    return p.astype(np.int32)
