"""Split-FP32 Acc and AccJerk (the ordered path) on particle distributions
other than the benchmark's Plummer-Salpeter sphere, against the FP64
kernels (bit-identical to the reference C backend), per particle:
acceleration within 1e-6, jerk within 1e-5.

* a central massive particle (5% of the mass), coincident particles (pairs
  at one position, softened), zero softening, a uniform cube: with the
  default recompute threshold;
* two clusters 100 length units apart and masses spread over six decades:
  with tg_set_recompute_threshold(10) (the default, 20, leaves these at
  1.2-1.4e-6 in the acceleration at N = 65536);
* a flat disk of equal masses (every particle's forces cancel in the
  plane): with tg_set_recompute_threshold(5) (20 leaves it at 2.5e-6, 10
  at 1.4e-6);
* all at N = 16384 and 65536.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

P5 = ("mass", "rx", "ry", "rz", "eps2")
P8 = P5 + ("vx", "vy", "vz")


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    from tupan_gb300.ics import Salpeter, plummer_arrays
    return _native, Salpeter, plummer_arrays


def make(mods, name, n):
    _, Salpeter, plummer_arrays = mods
    rng = np.random.default_rng(n)
    if name == "central_mass":
        d = plummer_arrays(n, 1e-3, imf=Salpeter(0.1, 100.0), seed=1)
        d["mass"] = d["mass"] * 0.95
        d["mass"][0] = 0.05
        for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
            d[k][0] = 0.0
    elif name == "two_clusters":
        d = plummer_arrays(n, 1e-3, imf=Salpeter(0.1, 100.0), seed=2)
        d["rx"][n // 2:] += 100.0
        d["vx"][n // 2:] -= 0.5
    elif name == "disk":
        d = plummer_arrays(n, 1e-3, seed=3)
        d["rz"][:] = 0.0
        d["vz"][:] = 0.0
    elif name == "coincident":
        d = plummer_arrays(n, 1e-3, seed=4)
        for k in ("rx", "ry", "rz"):
            d[k][1::7] = d[k][0::7][:len(d[k][1::7])]
    elif name == "no_softening":
        d = plummer_arrays(n, 0.0, seed=5)
        d["eps2"] = np.zeros(n)
    elif name == "mass_range":
        d = plummer_arrays(n, 1e-3, seed=6)
        m = np.exp(rng.uniform(np.log(1e-4), np.log(100.0), n))
        d["mass"] = m / m.sum()
    else:   # cube
        d = plummer_arrays(n, 1e-3, seed=7)
        for k in ("rx", "ry", "rz"):
            d[k] = rng.uniform(-1.0, 1.0, n)
    return {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device="cuda") for k, v in d.items()}


def run(native, name, I, prec, nout):
    f = P5 if name == "acc" else P8
    n = len(I["mass"])
    outs = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(nout)]
    p = [I[k].data_ptr() for k in f]
    native.call_device(name, n, p, n, p, (), [o.data_ptr() for o in outs], prec, native.current_stream())
    return torch.stack(outs)


def worst(got, want):
    e = torch.linalg.norm(got - want, dim=0) / torch.linalg.norm(want, dim=0)
    return float(e.max())


def check(mods, case, n):
    native = mods[0]
    I = make(mods, case, n)
    for name, nout in (("acc", 3), ("acc_jerk", 6)):
        want = run(native, name, I, native.PREC_FP64, nout)
        got = run(native, name, I, native.PREC_DS32, nout)
        assert worst(got[:3], want[:3]) <= 1e-6, (case, n, name)
        if nout == 6:
            assert worst(got[3:], want[3:]) <= 1e-5, (case, n, "jerk")
    assert native.sync_status() == 0


@pytest.mark.parametrize("n", [16384, 65536])
@pytest.mark.parametrize("case", ["central_mass", "coincident", "no_softening", "cube"])
def test_default_threshold(mods, case, n):
    check(mods, case, n)


@pytest.mark.parametrize("n", [16384, 65536])
@pytest.mark.parametrize("case,tau", [("two_clusters", 10.0), ("mass_range", 10.0), ("disk", 5.0)])
def test_lower_threshold(mods, case, tau, n):
    native = mods[0]
    prev = native.set_recompute_threshold(tau)
    try:
        check(mods, case, n)
    finally:
        native.set_recompute_threshold(prev)
