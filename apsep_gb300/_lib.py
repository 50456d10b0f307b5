"""ctypes binding of libapsep.so (include/apsep.h).

Loading fails loudly: there is no CPU or pure-PyTorch fallback for any entry
point.  If the library is missing, build it with
`python -m apsep_gb300.build` (or `__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libapsep.so")

# Every function include/apsep.h declares, with its ctypes signature.
_vp, _i32, _i64, _u32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32
SIGNATURES = {
    "apsep_version": ([], ctypes.c_int),
    "apsep_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "apsep_plan_create": ([ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, _i64], ctypes.c_int),
    "apsep_plan_destroy": ([_vp], ctypes.c_int),
    "apsep_run": ([_vp, _vp, _vp, _i64, _vp], ctypes.c_int),
    "apsep_run_cmp": ([_vp, _vp, _vp, _i64, ctypes.c_int, _vp], ctypes.c_int),
    "apsep_plan_check": ([_vp, _vp], ctypes.c_int),
    "apsep_plan_error_async": ([_vp, _vp, _vp], ctypes.c_int),
    "apsep_copy_spans": ([_vp, _vp, _vp, _i32, _vp], ctypes.c_int),
    "apsep_plan_get_info": ([_vp, _vp], ctypes.c_int),
    "apsep_plan_set_config": ([_vp, _i32], ctypes.c_int),
    "apsep_num_configs": ([], _i32),
    "apsep_config_shape": ([_i32, ctypes.POINTER(_i32), ctypes.POINTER(_i32)], ctypes.c_int),
    "apsep_launch": ([_vp, _vp, _i64, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "apsep_debug_inject": ([_vp, _i32, _u32], ctypes.c_int),
    "apsep_run_noalloc": ([_vp, _vp, _i64, ctypes.c_int, ctypes.c_int, _vp], ctypes.c_int),
    "apsep_noalloc_check": ([_vp], ctypes.c_int),
    "apsep_run_segmented": ([_vp, _vp, _vp, _i64, _vp, _i32, _vp], ctypes.c_int),
    "apsep_consumer_workspace_bytes": ([_i64], _i64),
    "apsep_run_prev_greater": ([_vp, _vp, _vp, _i64, ctypes.c_int, _vp, _vp], ctypes.c_int),
    "apsep_run_next_smaller": ([_vp, _vp, _vp, _i64, ctypes.c_int, _vp, _vp], ctypes.c_int),
    "apsep_stock_span": ([_vp, _vp, _vp, _i64, _vp, _vp], ctypes.c_int),
    "apsep_largest_rectangle": ([_vp, _vp, _i64, _vp, _vp, _vp], ctypes.c_int),
    "apsep_cartesian_parents": ([_vp, _vp, _vp, _i64, _vp, _vp], ctypes.c_int),
    "apsep_run64_workspace_bytes": ([_vp, _i64], _i64),
    "apsep_run64": ([_vp, _vp, _vp, _i64, ctypes.c_int, _vp, _vp], ctypes.c_int),
}

NOALLOC_MAX_KEYS = 4194304  # APSEP_NOALLOC_MAX_KEYS in include/apsep.h
NUM_CONFIGS = 6  # kernel configurations of the 4-byte key engine (apsep_num_configs)
MAX_KEYS = 2147479552  # APSEP_MAX_KEYS in include/apsep.h (2^31 - 4096)
MAX_KEYS64 = 1 << 40  # APSEP_MAX_KEYS64 in include/apsep.h

APSEP_OK, APSEP_EINVAL, APSEP_ENOMEM, APSEP_ECUDA, APSEP_ETIMEOUT, APSEP_EINTERNAL, APSEP_ENOTSUP = range(7)
INT32, FLOAT32, INT64, FLOAT64 = 0, 1, 2, 3
LT, LE = 0, 1


class PlanInfo(ctypes.Structure):
    _fields_ = [("capacity", _i64), ("scratch_bytes", _i64), ("tile_keys", _i32), ("config", _i32),
                ("device", _i32), ("dtype", _i32), ("cmp", _i32), ("reserved", _i32)]


class ApsepError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status)
        super().__init__("%s: %s (status %d)" % (what, msg, status) if what else msg)


_lib = None
_lock = threading.Lock()


def load() -> ctypes.CDLL:
    """Load libapsep.so; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.isfile(LIB_PATH):
                raise ImportError(
                    "libapsep.so is not built at %s; run `python -m apsep_gb300.build`" % LIB_PATH)
            lib = ctypes.CDLL(LIB_PATH)
            for name, (argtypes, restype) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = argtypes
                fn.restype = restype
            _lib = lib
    return _lib


def status_string(status: int) -> str:
    try:
        return load().apsep_status_string(int(status)).decode()
    except ImportError:
        return "status %d" % status


def check(status: int, what: str = "") -> None:
    if status != APSEP_OK:
        raise ApsepError(status, what)


def copy_spans(srcs, dsts, nbytes, stream_handle: int) -> None:
    """apsep_copy_spans over Python lists of addresses and byte counts."""
    n = len(srcs)
    if n == 0:
        return
    a = (ctypes.c_void_p * n)(*srcs)
    b = (ctypes.c_void_p * n)(*dsts)
    c = (ctypes.c_int64 * n)(*nbytes)
    check(load().apsep_copy_spans(a, b, c, n, ctypes.c_void_p(stream_handle)), "apsep_copy_spans")
