"""CPU oracle for APSE -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only to verify the engine's answers / as the timed CPU
baseline.  The product
(apsep_gb300, libapsep.so) never imports, links or calls it.

Contents
  apse(a, le)                 sequential monotone stack (apsep_oracle.c),
                              restating cpuApsep (src/main.cu:102-113) and
                              cpuPSE (src/bench_spt_le.cu:24-35)
  apse_segmented(a, offs, le) the same per segment, answers segment-relative
  ref_available(), ref_apse   the reference's own cpuApsep / cpuPSE compiled
                              from its sources (oracle/build_ref.py), when the
                              reference tree is present
  mt19937_raw, glibc_rand     the PRNG streams the reference harnesses draw
                              their test inputs from (main.cu:145-175,
                              bench_spt_le.cu:93-127), regenerated without the
                              reference so golden inputs can be rebuilt anywhere
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None
_ref = None


def build(force: bool = False) -> str:
    """Compile apsep_oracle.c with gcc into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "apsep_oracle.c")
    if (not force and os.path.isfile(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    tmp = _LIB_PATH + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-shared", "-fPIC",
                           "-o", tmp, src])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        i64, i32, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
        for name in ("oracle_apse_i32", "oracle_apse_f32", "oracle_apse_i64", "oracle_apse_f64"):
            f = getattr(lib, name)
            f.argtypes = [vp, i64, i32, vp]
            f.restype = i32
        for name in ("oracle_apse_segmented_i32", "oracle_apse_segmented_f32"):
            f = getattr(lib, name)
            f.argtypes = [vp, vp, i64, i32, vp]
            f.restype = i32
        _lib = lib
    return _lib


def _fn(a: np.ndarray, seg: bool):
    lib = _load()
    if a.dtype == np.int32:
        return lib.oracle_apse_segmented_i32 if seg else lib.oracle_apse_i32
    if a.dtype == np.float32:
        return lib.oracle_apse_segmented_f32 if seg else lib.oracle_apse_f32
    if a.dtype == np.int64 and not seg:
        return lib.oracle_apse_i64
    if a.dtype == np.float64 and not seg:
        return lib.oracle_apse_f64
    raise TypeError("oracle supports int32 / float32 keys (and int64 / float64 single arrays), got %s" % a.dtype)


def apse(a: np.ndarray, le: bool = False) -> np.ndarray:
    """out[i] = max{j < i : a[j] < a[i]} (<= when le), else -1."""
    a = np.ascontiguousarray(a)
    out = np.empty(a.shape[0], dtype=np.int32)
    rc = _fn(a, False)(a.ctypes.data, a.shape[0], int(bool(le)), out.ctypes.data)
    if rc:
        raise RuntimeError("oracle_apse failed: %d" % rc)
    return out


def apse_segmented(a: np.ndarray, offsets: np.ndarray, le: bool = False) -> np.ndarray:
    """Per-segment APSE; segment s is a[offsets[s]:offsets[s+1]], answers
    relative to offsets[s]."""
    a = np.ascontiguousarray(a)
    offs = np.ascontiguousarray(offsets, dtype=np.int64)
    out = np.full(a.shape[0], -1, dtype=np.int32)
    rc = _fn(a, True)(a.ctypes.data, offs.ctypes.data, offs.shape[0] - 1,
                      int(bool(le)), out.ctypes.data)
    if rc:
        raise RuntimeError("oracle_apse_segmented failed: %d" % rc)
    return out


# --------------------------------------------------------------------------
# The reference's own CPU oracles (compiled from its sources), when present.
# --------------------------------------------------------------------------
def ref_available() -> bool:
    return _load_ref() is not None


def _load_ref():
    global _ref
    if _ref is None:
        from . import build_ref
        p = build_ref.build()
        if p is None:
            _ref = False
        else:
            lib = ctypes.CDLL(p)
            vp, i32 = ctypes.c_void_p, ctypes.c_int
            lib.ref_cpu_apsep.argtypes = [vp, i32, vp]
            lib.ref_cpu_pse.argtypes = [vp, i32, i32, vp]
            lib.ref_mt19937_raw.argtypes = [ctypes.c_uint, vp, ctypes.c_longlong]
            lib.ref_glibc_rand.argtypes = [ctypes.c_uint, vp, ctypes.c_longlong]
            _ref = lib
    return _ref or None


def ref_apse(a: np.ndarray, le: bool | None = None) -> np.ndarray:
    """Run the reference's cpuApsep (le is None) or cpuPSE (le given)."""
    lib = _load_ref()
    if lib is None:
        raise RuntimeError("reference CPU oracle unavailable")
    a = np.ascontiguousarray(a, dtype=np.int32)
    out = np.empty(a.shape[0], dtype=np.int32)
    if le is None:
        lib.ref_cpu_apsep(a.ctypes.data, a.shape[0], out.ctypes.data)
    else:
        lib.ref_cpu_pse(a.ctypes.data, a.shape[0], int(bool(le)), out.ctypes.data)
    return out


# --------------------------------------------------------------------------
# PRNG streams of the reference harnesses, reproducible without it.
# --------------------------------------------------------------------------
def mt19937_raw(seed: int, count: int) -> np.ndarray:
    """First `count` outputs of std::mt19937(seed) (numpy's legacy MT19937
    seeding is the same init_genrand routine)."""
    bg = np.random.MT19937()
    bg._legacy_seeding(int(seed))
    return bg.random_raw(int(count)).astype(np.uint32)


class MT19937Stream:
    """Sequential draws from std::mt19937(seed), like `rng()` calls."""

    def __init__(self, seed: int):
        self._bg = np.random.MT19937()
        self._bg._legacy_seeding(int(seed))

    def draw(self, count: int) -> np.ndarray:
        return self._bg.random_raw(int(count)).astype(np.uint32)


SPT_LE_CASES = ("random", "dup16", "dup2", "all-equal", "descending",
                "ascending", "intmax")
SPT_LE_FULL_N = 32 * 1024 * 1024


def gen_spt_le_case(name: str, n: int, full_n: int = SPT_LE_FULL_N) -> np.ndarray:
    """Prefix of length n of the input the reference's SPT </<= harness
    builds for case `name` (src/bench_spt_le.cu:93-127)."""
    lib = _load()
    f = lib.oracle_gen_spt_le_case
    f.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    out = np.empty(int(n), dtype=np.int32)
    if f(SPT_LE_CASES.index(name), int(full_n), int(n), out.ctypes.data):
        raise ValueError(name)
    return out


def main_small_cases() -> list[tuple[str, np.ndarray]]:
    """The structured cases of the reference harness (src/main.cu:181-199)."""
    B = 128 * 4
    cases = [
        ("single element", [42]),
        ("two ascending", [1, 2]),
        ("two descending", [2, 1]),
        ("all equal", [5, 5, 5, 5, 5]),
        ("ascending", [1, 2, 3, 4, 5, 6, 7, 8]),
        ("descending", [8, 7, 6, 5, 4, 3, 2, 1]),
        ("alternating", [3, 1, 4, 1, 5, 9, 2, 6]),
        ("exact block (B=512)", list(range(B))),
        ("two full blocks", [(i % 7) * 13 for i in range(2 * B)]),
        ("non-power-of-two", [i % 17 for i in range(B + 13)]),
    ]
    return [(lab, np.asarray(v, dtype=np.int32)) for lab, v in cases]


def main_stress_inputs(seed: int, trials: int, max_n: int):
    """Yield the inputs of the reference's random stress loop
    (src/main.cu:145-175): per trial n = 1 + rng() % maxN, then n values
    rng() % 1000000, all from one std::mt19937(seed) stream."""
    s = MT19937Stream(seed)
    for _ in range(trials):
        n = 1 + int(s.draw(1)[0] % np.uint32(max_n))
        yield (s.draw(n) % np.uint32(1000000)).astype(np.int32)


def glibc_rand(seed: int, count: int) -> np.ndarray:
    """`count` successive glibc rand() values after srand(seed)."""
    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    libc.rand.restype = ctypes.c_int
    # Fast path: a small C loop would need a compiler; rand() through ctypes
    # is ~10 M calls/s, enough for the fixture sizes used in the tests.
    libc.srand(int(seed))
    out = np.empty(int(count), dtype=np.int32)
    r = libc.rand
    for i in range(int(count)):
        out[i] = r()
    return out
