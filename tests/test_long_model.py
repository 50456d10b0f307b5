"""CPU model of the int64-position algorithm (apsep_gb300/csrc/apsep_long.cu):
pieces answered on their own, then every key its piece leaves unanswered
answered from the hierarchy of minima before the piece -- the nearest
frontier whose minimum qualifies, the last qualifying entry there, then one
32-wide step per level down to the key.  Checked against the oracle on small
arrays cut into many pieces, so the frontier tiling and the descent are
pinned without a GPU (the GPU tests run the CUDA code itself)."""
import numpy as np
import pytest

import oracle


def top_level(n):
    level, size = 1, -(-n // 32)
    while size > 31:
        size = -(-size // 32)
        level += 1
    return level


def levels_of(a):
    """lv[0] = keys; lv[l][e] = min of keys [e*32^l, (e+1)*32^l) (l >= 1)."""
    lv = [a]
    for _ in range(top_level(len(a))):
        prev = lv[-1]
        pad = (-len(prev)) % 32
        big = np.iinfo(a.dtype).max if np.issubdtype(a.dtype, np.integer) else np.inf
        lv.append(np.concatenate([prev, np.full(pad, big, prev.dtype)]).reshape(-1, 32).min(axis=1))
    return lv


def answer_before(lv, q, b0, le):
    lt = (lambda x, y: x <= y) if le else (lambda x, y: x < y)
    top = len(lv) - 1
    # frontiers: at level l the entries [g*32, idx) with idx = b0 >> 5l, g = idx >> 5
    for lev in range(top + 1):
        idx = b0 >> (5 * lev)
        g0 = (idx >> 5) << 5
        run = lv[lev][g0:idx]
        hits = np.flatnonzero(lt(run, q)) if len(run) else []
        if len(hits):
            f = g0 + int(hits[-1])
            for d in range(lev, 0, -1):  # descend: last qualifying entry of each group
                grp = lv[d - 1][f * 32:f * 32 + 32]
                f = f * 32 + int(np.flatnonzero(lt(grp, q))[-1])
            return f
    return -1


def model(a, piece, le):
    n = len(a)
    lv = levels_of(a)
    out = np.empty(n, dtype=np.int64)
    for b0 in range(0, n, piece):
        b1 = min(n, b0 + piece)
        r = oracle.apse(np.ascontiguousarray(a[b0:b1]), le).astype(np.int64)
        out[b0:b1] = np.where(r >= 0, b0 + r, -1)
        if b0:
            for i in np.flatnonzero(r < 0):
                out[b0 + i] = answer_before(lv, a[b0 + i], b0, le)
    return out


@pytest.mark.parametrize("le", [False, True])
@pytest.mark.parametrize("piece,n", [(32, 3000), (992, 40_000), (4096, 70_001)])
def test_model_matches_the_oracle(piece, n, le):
    rng = np.random.default_rng(piece + n)
    i = np.arange(n)
    for a in (rng.integers(0, 1 << 20, n).astype(np.int32),
              rng.integers(0, 5, n).astype(np.int32),
              (-(i % 777) + (i // 777) * 900).astype(np.int32),  # descending runs, rising
              np.cumsum(rng.integers(-3, 4, n)).astype(np.int32)):
        assert np.array_equal(model(a, piece, le), oracle.apse(a, le).astype(np.int64))


def test_frontiers_tile_the_prefix():
    # the frontier runs of all levels cover [0, b0) exactly, nearest first
    n = 1 << 22
    top = top_level(n)
    for b0 in (32, 992, 1024, 33 * 1024 + 64, (1 << 21) + 96, n - 32):
        covered, hi = 0, b0
        for lev in range(top + 1):
            idx = b0 >> (5 * lev)
            g0 = (idx >> 5) << 5
            lo = g0 << (5 * lev)
            assert (idx << (5 * lev)) == hi or lev == 0 and idx == b0
            covered += hi - lo
            hi = lo
        assert hi == 0 and covered == b0
