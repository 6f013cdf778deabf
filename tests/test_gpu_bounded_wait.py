"""Failure detection without a GPU fault: the bounded shared-memory barrier
wait of the split-FP32 kernels gives up, raises TG_ST_MBAR_TIMEOUT and
returns, and the CUDA context stays usable for the next call.

The wait runs on a barrier that nothing arrives at (tg_check_bounded_wait
with arrive = 0), which is how a j-tile copy that never completes looks to
the kernels; no copy is in flight, nothing faults or traps."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TG_ST_MBAR_TIMEOUT = 1


@pytest.fixture(scope="module")
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    return _native


def wait(native, polls, arrive):
    ms = ctypes.c_double(0.0)
    rc = native.lib.tg_check_bounded_wait(polls, arrive, ctypes.byref(ms))
    assert rc >= 0, native.last_error()
    return rc, ms.value


def test_wait_that_never_completes_gives_up_with_a_status(native):
    rc, ms = wait(native, 4096, 0)
    assert rc == TG_ST_MBAR_TIMEOUT
    assert ms < 1000.0


def test_completed_barrier_raises_nothing(native):
    rc, _ = wait(native, 4096, 1)
    assert rc == 0


def test_context_usable_after_a_timeout(native):
    from oracle.oracle import Oracle
    from tupan_gb300.lib import extensions
    from tupan_gb300.particles import ParticleSystem
    assert wait(native, 4096, 0)[0] == TG_ST_MBAR_TIMEOUT
    rng = np.random.default_rng(11)
    n = 700
    d = {"mass": rng.random(n) / n, "eps2": np.full(n, 1e-4)}
    for c in "xyz":
        d["r" + c] = rng.normal(size=n)
        d["v" + c] = rng.normal(size=n)
    ps = ParticleSystem.from_arrays(**d)
    got = np.stack([o.cpu().numpy() for o in extensions.Acc("CUDA", "ds32").calc(ps, ps)])
    want = np.stack(Oracle().calc("acc", d, d, nthreads=4))
    err = np.sqrt(((got - want) ** 2).sum(0)) / np.sqrt((want ** 2).sum(0))
    assert err.max() < 4e-6
    assert native.sync_status() == 0   # the pairwise call itself raised nothing
