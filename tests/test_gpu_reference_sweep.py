"""The reference's own kernel test at full length: every prefix 1..256 of a
256-particle set as the j-set (i = all) and as the i-set (j = all), for every
hot-path kernel (tupan/tests/test_extensions.py:45-85, whose particle
set is U(0,1) masses, zero softening and U(0,10) positions and velocities,
lines 28-36).  The reference test prints deviations; this one asserts them
against the CPU oracle (the reference algorithm, pinned bit-exact to the
reference C backend): FP64 bit-identical for Phi, Acc, AccJerk,
SnapCrackle, Tstep; PNAcc (order 7, c = 128) to 1e-13 of the largest
component; Sakura (dt = 1/64, flags -1 and +1) to 1e-9 (CUDA's
transcendentals); split FP32 within the parity test's bounds for the
synthetic sets."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from test_gpu_parity import DS32_TOL, KCLASS, PS, within  # noqa: E402

N = 256
PN = (7, 128.0)


def particles(seed=2024):
    rng = np.random.default_rng(seed)
    d = {"mass": rng.random(N), "eps2": np.zeros(N)}
    for c in "xyz":
        d["r" + c] = rng.random(N) * 10
        d["v" + c] = rng.random(N) * 10
    for k in ("ax", "ay", "az", "jx", "jy", "jz"):
        d[k] = rng.random(N)
    return d


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle.oracle import Oracle
    from tupan_gb300.lib import extensions
    return extensions, Oracle()


def gpu(ext, name, prec, I, J, sc):
    k = getattr(ext, KCLASS[name])("CUDA", prec)
    if name == "pnacc":
        c = ext.clight
        c.pn_order, c.clight = PN
        out = k.calc(PS(I), PS(J))
    else:
        out = k.calc(PS(I), PS(J), *sc)
    torch.cuda.synchronize()
    return np.stack([o.cpu().numpy() for o in out])


def oracle_scalars(ext, name, sc):
    if name != "pnacc":
        return sc
    c = ext.clight
    c.pn_order, c.clight = PN
    return (c.pn_order,) + tuple(getattr(c, "inv%d" % q) for q in range(1, 8))


CALLS = [("phi", ()), ("acc", ()), ("acc_jerk", ()), ("snap_crackle", ()), ("tstep", (1.0 / 64,)),
         ("pnacc", ()), ("sakura", (1.0 / 64, -1)), ("sakura", (1.0 / 64, 1))]


@pytest.mark.parametrize("name,sc", CALLS, ids=["phi", "acc", "acc_jerk", "snap_crackle", "tstep", "pnacc",
                                               "sakura-1", "sakura+1"])
def test_reference_prefix_sweep(env, name, sc):
    ext, orc = env
    d = particles()
    osc = oracle_scalars(ext, name, sc)
    for p in range(1, N + 1):
        S = {f: v[:p] for f, v in d.items()}
        for I, J in ((d, S), (S, d)):
            want = np.stack(orc.calc(name, I, J, *osc))
            got = gpu(ext, name, "float64", I, J, sc)
            if name in ("pnacc", "sakura"):
                tol = 1e-13 if name == "pnacc" else 1e-9
                assert np.abs(got - want).max() <= tol * max(np.abs(want).max(), 1e-300), (name, p)
            else:
                assert np.array_equal(got, want), (name, p)
            if name != "sakura":
                ok, err = within(name, gpu(ext, name, "ds32", I, J, sc), want, DS32_TOL[name])
                assert ok, (name, p, err)
