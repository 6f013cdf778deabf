"""tg_acc_jerk_noalloc: split-FP32 AccJerk without any GPU allocation.

Some programs cannot let a library allocate GPU memory: those whose own
memory pool claims the GPU at start-up (a library cudaMalloc would then fail
or fragment the pool) and time-stepping loops that must not stall their
other streams on cudaMalloc/cudaFree.  For them the library has one entry
point whose scratch is a fixed 24 MiB __device__ array.  These tests call it
through the C ABI and check it against the allocating entry point
tg_acc_jerk(..., TG_PREC_DS32, ...) on two calls in a row, with the same
per-particle relative tolerance the split-FP32 parity tests use for AccJerk.

This file is collected last on purpose (test_zz_*), so a run that stops at
the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 4e-6          # split-FP32 AccJerk tolerance of tests/test_gpu_parity.py
P8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")


def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    fn = _native.lib.tg_acc_jerk_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = ([ctypes.c_size_t] + [ctypes.c_void_p] * 8) * 2 + [ctypes.c_void_p] * 7
    return _native, fn


def _particles(n, seed):
    rng = np.random.default_rng(seed)
    d = {"mass": rng.random(n) / n, "eps2": np.full(n, 5e-5)}
    for c in "xyz":
        d["r" + c] = rng.normal(size=n)
        d["v" + c] = rng.normal(size=n) * 0.3
    return {k: torch.tensor(v, dtype=torch.float64, device="cuda") for k, v in d.items()}


def _outputs(n):
    return [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(6)]


def _rel_err(got, want):
    worst = 0.0
    for g in ((0, 1, 2), (3, 4, 5)):
        d = torch.sqrt(sum((got[k] - want[k]) ** 2 for k in g))
        n = torch.sqrt(sum(want[k] ** 2 for k in g))
        worst = max(worst, float((d / n).max()))
    return worst


def test_noalloc_matches_allocating_entry_point_twice():
    native, fn = _lib()
    n = 5000                      # ragged: partial i- and j-tiles, several CTAs per i-tile
    T = _particles(n, seed=11)
    ptr = [T[k].data_ptr() for k in P8]
    stream = torch.cuda.current_stream().cuda_stream

    want = _outputs(n)
    native.call_device("acc_jerk", n, ptr, n, ptr, (), [o.data_ptr() for o in want],
                       native.PREC_DS32, stream)

    results = []
    for _ in range(2):            # the shared scratch keeps the previous call's contents
        got = _outputs(n)
        rc = fn(n, *ptr, n, *ptr, *[o.data_ptr() for o in got], stream)
        assert rc == 0, native.last_error()
        torch.cuda.synchronize()
        assert _rel_err(got, want) <= TOL
        results.append(got)
    for a, b in zip(*results):
        assert torch.equal(a, b)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    native, fn = _lib()
    null = [None] * 8
    rc = fn((1 << 20) + 1, *null, 16, *null, *([None] * 6), None)
    assert rc == native.EINVAL
    assert "1048576" in native.last_error()
    rc = fn(16, *null, (1 << 17) + 1, *null, *([None] * 6), None)
    assert rc == native.EINVAL
    assert "131072" in native.last_error()
