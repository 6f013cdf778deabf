"""tg_acc_jerk_noalloc: split-FP32 AccJerk without any GPU allocation.

Some programs cannot let a library allocate GPU memory: those whose own
memory pool claims the GPU at start-up (a library cudaMalloc would then fail
or fragment the pool) and time-stepping loops that must not stall their
other streams on cudaMalloc/cudaFree.  For them the library has one entry
point whose scratch is a fixed 24 MiB __device__ array.  These tests call it
through the C ABI:

  * against the CPU oracle (the reference algorithm in FP64) on two calls in
    a row, within the split-FP32 bounds of the parity tests (acceleration
    1e-6, jerk 1e-5 per particle), the two calls bit-identical;
  * at the largest j-set it accepts (2^17, the most CTAs it runs) against
    the FP64 kernel, which is bit-identical to the reference;
  * in a fresh process, that its calls leave the device's free memory
    unchanged (after a first call: with the CUDA runtime's lazy loading that
    first call is when the library's GPU image, static scratch included,
    gets loaded);
  * that sizes beyond its scratch are refused with a clear error.

This file is collected last on purpose (test_zz_*), so a run that stops at
the first failure has run every other test before it.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = (1e-6, 1e-5)  # acceleration, jerk: the split-FP32 bounds of tests/test_gpu_parity.py
P8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    fn = _native.lib.tg_acc_jerk_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = ([ctypes.c_size_t] + [ctypes.c_void_p] * 8) * 2 + [ctypes.c_void_p] * 7
    return _native, fn


def _arrays(n, seed):
    rng = np.random.default_rng(seed)
    d = {"mass": rng.random(n) / n, "eps2": np.full(n, 5e-5)}
    for c in "xyz":
        d["r" + c] = rng.normal(size=n)
        d["v" + c] = rng.normal(size=n) * 0.3
    return d


def _dev(d):
    return {k: torch.tensor(v, dtype=torch.float64, device="cuda") for k, v in d.items()}


def _outputs(n):
    return [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(6)]


def _errs(got, want):
    """Max per-particle relative error of the acceleration and of the jerk."""
    out = []
    for g in ((0, 1, 2), (3, 4, 5)):
        d = np.sqrt(sum((got[k] - want[k]) ** 2 for k in g))
        n = np.sqrt(sum(want[k] ** 2 for k in g))
        out.append(float((d / n).max()))
    return out


def test_noalloc_matches_oracle_twice():
    from oracle.oracle import Oracle
    native, fn = _lib()
    n = 5000                      # ragged: partial i- and j-tiles, several CTAs per i-tile
    d = _arrays(n, seed=11)
    want = np.stack(Oracle().calc("acc_jerk", d, d, nthreads=8))
    T = _dev(d)
    ptr = [T[k].data_ptr() for k in P8]
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):            # the shared scratch keeps the previous call's contents
        got = _outputs(n)
        rc = fn(n, *ptr, n, *ptr, *[o.data_ptr() for o in got], stream)
        assert rc == 0, native.last_error()
        assert native.last_error() == ""
        torch.cuda.synchronize()
        host = np.stack([o.cpu().numpy() for o in got])
        errs = _errs(host, want)
        assert errs[0] <= TOL[0] and errs[1] <= TOL[1], errs
        results.append(host)
    assert np.array_equal(results[0], results[1])
    assert native.sync_status(stream) == 0


def test_noalloc_largest_j_set():
    """nj = 2^17: the scratch's largest j-set, and more units than the 320
    CTAs the entry point runs, so its grid cap is in play."""
    native, fn = _lib()
    ni, nj = 4096, 1 << 17
    d = _arrays(nj, seed=12)
    T = _dev(d)
    jp = [T[k].data_ptr() for k in P8]
    ip = [T[k][:ni].data_ptr() for k in P8]
    stream = torch.cuda.current_stream().cuda_stream
    want = _outputs(ni)
    native.call_device("acc_jerk", ni, ip, nj, jp, (), [o.data_ptr() for o in want], native.PREC_FP64, stream)
    got = _outputs(ni)
    rc = fn(ni, *ip, nj, *jp, *[o.data_ptr() for o in got], stream)
    assert rc == 0, native.last_error()
    torch.cuda.synchronize()
    errs = _errs(np.stack([o.cpu().numpy() for o in got]), np.stack([o.cpu().numpy() for o in want]))
    assert errs[0] <= TOL[0] and errs[1] <= TOL[1], errs


CHILD = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, %r)
from tupan_gb300 import _native
fn = _native.lib.tg_acc_jerk_noalloc
fn.restype = ctypes.c_int
fn.argtypes = ([ctypes.c_size_t] + [ctypes.c_void_p] * 8) * 2 + [ctypes.c_void_p] * 7
n = 3000
rng = np.random.default_rng(3)
T = [torch.tensor(rng.normal(size=n) if k else rng.random(n) / n, dtype=torch.float64, device="cuda")
     for k in range(8)]
T[4] = torch.full((n,), 5e-5, dtype=torch.float64, device="cuda")
out = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(6)]
ptr = [t.data_ptr() for t in T]
s = torch.cuda.current_stream().cuda_stream
torch.cuda.synchronize()
free = []
for _ in range(3):
    free.append(torch.cuda.mem_get_info()[0])
    assert fn(n, *ptr, n, *ptr, *[o.data_ptr() for o in out], s) == 0, _native.last_error()
    torch.cuda.synchronize()
free.append(torch.cuda.mem_get_info()[0])
print("FREE", *free)
"""


def test_noalloc_allocates_nothing():
    """Free device memory before and after each of three calls, in a fresh
    process, from the second call on (the first may load the library's GPU
    image, which holds the static scratch)."""
    _lib()
    out = subprocess.run([sys.executable, "-c", CHILD % ROOT], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    free = [int(x) for x in out.stdout.split("FREE", 1)[1].split()]
    assert len(set(free[1:])) == 1, free


def test_noalloc_rejects_sizes_beyond_its_scratch():
    native, fn = _lib()
    null = [None] * 8
    rc = fn((1 << 20) + 1, *null, 16, *null, *([None] * 6), None)
    assert rc == native.EINVAL
    assert "1048576" in native.last_error()
    rc = fn(16, *null, (1 << 17) + 1, *null, *([None] * 6), None)
    assert rc == native.EINVAL
    assert "131072" in native.last_error()
