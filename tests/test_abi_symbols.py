"""The C ABI library loads and exports every function include/*.h declares.

Runs without a GPU: loading the library and resolving symbols makes no CUDA
call.  The library is built first if it is missing (nvcc cross-compiles).
"""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for path in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(path).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:unsigned\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, re.M):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from tupan_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for k in ("phi", "acc", "acc_jerk", "snap_crackle", "tstep", "pnacc", "sakura"):
        assert k + "_kernel" in names      # libtupan.h signatures
        assert "tg_" + k in names          # device-pointer forms
    assert "tg_last_error" in names and "tg_sync_status" in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_precision_without_gpu(lib):
    lib.tg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.tg_version()
    lib.tg_set_host_precision.argtypes = [ctypes.c_int]
    assert lib.tg_set_host_precision(7) == -1          # TG_EINVAL
    assert lib.tg_set_host_precision(1) == 0
    assert lib.tg_get_host_precision() == 1
    assert lib.tg_set_host_precision(0) == 0


def test_invalid_precision_is_rejected_before_any_cuda_call(lib):
    lib.tg_acc.restype = ctypes.c_int
    args = [ctypes.c_size_t(0)] + [None] * 5 + [ctypes.c_size_t(0)] + [None] * 5 + [None] * 3
    assert lib.tg_acc(*args, ctypes.c_int(9), None) == -1
    lib.tg_last_error.restype = ctypes.c_char_p
    assert b"precision" in lib.tg_last_error()
