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


def test_ds32x_refused_for_kernels_without_it_before_any_cuda_call(lib):
    lib.tg_phi.restype = ctypes.c_int
    lib.tg_last_error.restype = ctypes.c_char_p
    args = [ctypes.c_size_t(0)] + [None] * 5 + [ctypes.c_size_t(0)] + [None] * 5 + [None]
    assert lib.tg_phi(*args, ctypes.c_int(2), None) == -1          # TG_PREC_DS32X
    assert b"DS32X" in lib.tg_last_error()
    lib.tg_set_host_precision.argtypes = [ctypes.c_int]
    assert lib.tg_set_host_precision(2) == -1                       # host drop-ins: FP64 or DS32 only


def test_sia_h_step_validates_its_arguments_before_any_cuda_call(lib):
    f = lib.tg_sia_h_step
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                  ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                  ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    lib.tg_last_error.restype = ctypes.c_char_p
    kinds = (ctypes.c_int * 3)(0, 1, 0)
    coefs = (ctypes.c_double * 3)(0.5, 1.0, 0.5)
    rows = (ctypes.c_int * 15)(*range(14), 1)     # nstep: row 1 of the int block
    t = ctypes.c_double(0.25)
    fake = ctypes.c_void_p(4096)      # never dereferenced: every case fails its checks first

    def call(nops=3, k=kinds, n=8, real=fake, ld_real=8, rows_real=20, ints=fake, ld_int=8, rows_int=2, rw=rows):
        return f(nops, k, coefs, 1, 0.01, 0.01, 0, 0, n, real, ld_real, rows_real, ints, ld_int, rows_int, rw,
                 ctypes.byref(t), None)

    assert call(nops=0) == -1 and b"scheme" in lib.tg_last_error()
    assert call(nops=65) == -1
    assert call(n=0) == 0 and t.value == 0.25            # empty set: nothing to do
    assert call(ld_real=4) == -1 and b"blocks" in lib.tg_last_error()
    assert call(real=None) == -1
    bad = (ctypes.c_int * 15)(*range(14), 2)             # nstep row 2 of a 2-row int block
    assert call(rw=bad) == -1 and b"row" in lib.tg_last_error()
    neg = (ctypes.c_int * 15)(-1, *range(1, 15))
    assert call(rw=neg) == -1
    odd = (ctypes.c_int * 3)(0, 2, 0)
    assert call(k=odd) == -1 and b"kinds" in lib.tg_last_error()
    assert call(n=0, k=odd) == -1                          # the scheme is checked even for an empty set


def test_recompute_threshold_setting_without_gpu(lib):
    f = lib.tg_set_recompute_threshold
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double]
    prev = f(12.5)
    assert prev == 20.0                      # the default
    assert f(0.5) == -1.0 and f(float("nan")) == -1.0 and f(2e6) == -1.0
    assert f(prev) == 12.5                   # restored
