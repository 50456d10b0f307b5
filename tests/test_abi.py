"""The C-ABI library: it builds, loads without a GPU, exports every entry
point include/apsep.h declares, and rejects bad arguments with status codes
(no call exits the process).  No compute call is made here."""
import ctypes
import os
import re

import pytest

from apsep_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(apsep_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_the_api():
    names = declared_functions()
    for must in ("apsep_plan_create", "apsep_plan_destroy", "apsep_run", "apsep_launch", "apsep_plan_check"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert set(_lib.SIGNATURES) >= declared_functions()


def test_status_strings_and_configs(built_lib):
    lib = _lib.load()
    assert lib.apsep_version() >= 10000
    assert lib.apsep_status_string(_lib.APSEP_OK) == b"ok"
    assert lib.apsep_status_string(_lib.APSEP_ETIMEOUT) == b"device-side wait timed out"
    n = lib.apsep_num_configs()
    assert n == _lib.NUM_CONFIGS
    for c in range(n):
        t, k = ctypes.c_int32(), ctypes.c_int32()
        assert lib.apsep_config_shape(c, ctypes.byref(t), ctypes.byref(k)) == _lib.APSEP_OK
        assert t.value % 32 == 0 and k.value in (4, 8, 16)
    assert lib.apsep_config_shape(n, None, None) == _lib.APSEP_EINVAL


def test_argument_validation_without_device(built_lib):
    lib = _lib.load()
    assert lib.apsep_plan_create(None, 0, 0, 10) == _lib.APSEP_EINVAL
    h = ctypes.c_void_p()
    assert lib.apsep_plan_create(ctypes.byref(h), 7, 0, 10) == _lib.APSEP_EINVAL
    assert lib.apsep_plan_create(ctypes.byref(h), 0, 5, 10) == _lib.APSEP_EINVAL
    assert lib.apsep_plan_create(ctypes.byref(h), 0, 0, -1) == _lib.APSEP_EINVAL
    assert lib.apsep_plan_create(ctypes.byref(h), 0, 0, 1 << 40) == _lib.APSEP_EINVAL
    # int32 positions: the largest capacity keeps the last whole tile below 2^31
    assert lib.apsep_plan_create(ctypes.byref(h), 0, 0, 2147479552 + 1) == _lib.APSEP_EINVAL
    assert lib.apsep_run(None, None, None, 5, None) == _lib.APSEP_EINVAL
    assert lib.apsep_plan_destroy(None) == _lib.APSEP_OK
    assert lib.apsep_plan_check(None, None) == _lib.APSEP_EINVAL
    assert lib.apsep_plan_error_async(None, None, None) == _lib.APSEP_EINVAL
    assert lib.apsep_copy_spans(None, None, None, -1, None) == _lib.APSEP_EINVAL
    assert lib.apsep_copy_spans(None, None, None, 3, None) == _lib.APSEP_EINVAL
    assert lib.apsep_plan_set_config(None, 0) == _lib.APSEP_EINVAL
    assert lib.apsep_debug_inject(None, -2, 0) == _lib.APSEP_EINVAL
    assert lib.apsep_debug_inject(None, -1, 0) == _lib.APSEP_OK  # (no plan: the no-alloc path, disarmed)
    assert lib.apsep_launch(None, None, 0, 0, 0) == _lib.APSEP_OK  # n == 0 is a no-op
    assert lib.apsep_run64_workspace_bytes(None, 10) == -1
    assert lib.apsep_run64(None, None, None, 5, 0, None, None) == _lib.APSEP_EINVAL


def test_no_device_is_a_status_not_a_crash(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    h = ctypes.c_void_p()
    st = lib.apsep_plan_create(ctypes.byref(h), 0, 0, 1000)
    assert st in (_lib.APSEP_ECUDA, _lib.APSEP_ENOTSUP)
    assert not h.value
