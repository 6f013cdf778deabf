"""GPU NREG_X / NREG_V kernels, the batched Kepler pair solver and the
numpy-order reduction, called through the C ABI (extensions layer, device
entry points and drop-in host entry points).

* NREG_X / NREG_V (FP64 whatever the requested precision): bit-identical to
  the reference C backend (golden_nreg.npz), including prefix sweeps.
* Kepler pair solver: within 1e-9 of the largest |component| of the
  reference (golden_kepler.npz) -- the universal-variable solve uses CUDA's
  cos/sin/cosh/sinh/log, which differ from glibc by an ulp, so the Laguerre
  iteration may stop on a neighbouring iterate within its 2^-42 tolerance.
  A softened close pair that needs more sub-steps than the solver's bounds
  raises TG_ST_KEPLER_CAP and stays finite.
* tg_sum equals numpy.sum bit for bit; tg_div3 equals numpy division.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from golden_io import CASES, FIELDS, PREFIXES, load  # noqa: E402
from test_oracle_pin import (KEPLER_DTS, KEPLER_KINDS, NREG_DTS, P8, load_kepler,  # noqa: E402
                             load_nreg)

KEPLER_TOL = 1e-9


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    from tupan_gb300.lib import extensions
    return _native, extensions


class PS(object):
    def __init__(self, d, fields=FIELDS):
        self.n = len(d["mass"])
        for f in fields:
            setattr(self, f, torch.as_tensor(np.ascontiguousarray(d[f]), dtype=torch.float64, device="cuda"))

    def register_auxiliary_attribute(self, name, sctype):
        setattr(self, name, torch.zeros(self.n, dtype=torch.float64, device="cuda"))


def calc(ext, name, prec, ips, jps, dt):
    k = {"nreg_x": ext.NREG_X, "nreg_v": ext.NREG_V}[name]("CUDA", prec)
    out = k.calc(ips, jps, dt)
    torch.cuda.synchronize()
    return np.stack([o.cpu().numpy() for o in out])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("prec", ["float64", "ds32"])
def test_nreg_matches_golden(mods, case, prec):
    _, ext = mods
    g = load_nreg()
    _, ps, _ = load(case)
    for dt in NREG_DTS:
        for name in ("nreg_x", "nreg_v"):
            P = PS(ps)
            got = calc(ext, name, prec, P, P, dt)
            want = g["%s_%s_%r" % (case, name, dt)]
            assert np.array_equal(got, want), (case, name, dt)


def test_nreg_prefix_sweeps(mods):
    _, ext = mods
    g = load_nreg()
    _, ps, _ = load("sweep")
    for name in ("nreg_x", "nreg_v"):
        key = "sweep_%s_%r" % (name, 1.0 / 64)
        for p in PREFIXES:
            sub = {f: ps[f][:p] for f in FIELDS}
            assert np.array_equal(calc(ext, name, "float64", PS(ps), PS(sub), 1.0 / 64), g["J%d_" % p + key])
            assert np.array_equal(calc(ext, name, "float64", PS(sub), PS(ps), 1.0 / 64), g["I%d_" % p + key])


def test_nreg_host_drop_ins(mods):
    native, _ = mods
    g = load_nreg()
    _, ps, _ = load("plummer")
    n = len(ps["mass"])
    D = ctypes.POINTER(ctypes.c_double)
    arr = {f: np.ascontiguousarray(ps[f]) for f in FIELDS}
    p = lambda a: a.ctypes.data_as(D)  # noqa: E731
    dt = 1.0 / 64
    out = [np.zeros(n) for _ in range(7)]
    fx = native.lib.nreg_Xkernel
    fx(n, *[p(arr[f]) for f in P8], n, *[p(arr[f]) for f in P8], dt, *[p(o) for o in out])
    assert np.array_equal(np.stack(out), g["plummer_nreg_x_%r" % dt])
    v7 = ("mass", "vx", "vy", "vz", "ax", "ay", "az")
    out = [np.zeros(n) for _ in range(4)]
    native.lib.nreg_Vkernel(n, *[p(arr[f]) for f in v7], n, *[p(arr[f]) for f in v7], dt, *[p(o) for o in out])
    assert np.array_equal(np.stack(out), g["plummer_nreg_v_%r" % dt])


def test_nreg_empty_j(mods):
    _, ext = mods
    _, ps, _ = load("edge")
    empty = {f: ps[f][:0] for f in FIELDS}
    got = calc(ext, "nreg_x", "float64", PS(ps), PS(empty), 0.1)
    assert np.array_equal(got, np.zeros((7, 5)))


def kepler_close(got, want):
    scale = max(np.abs(want).max(), 1e-300)
    return np.abs(got - want).max() <= KEPLER_TOL * scale


@pytest.mark.parametrize("kind", KEPLER_KINDS)
def test_kepler_batched_matches_golden(mods, kind):
    """All pairs of a set in one tg_kepler_solver call, in place on torch
    tensors through extensions.Kepler."""
    native, ext = mods
    z, sets = load_kepler()
    for dt in KEPLER_DTS:
        P = PS(sets[kind], P8)
        ext.Kepler("CUDA").calc(P, P, dt)
        torch.cuda.synchronize()
        got = np.stack([getattr(P, f).cpu().numpy() for f in ("rx", "ry", "rz", "vx", "vy", "vz")])
        assert kepler_close(got, z["out_%s_%r" % (kind, dt)]), (kind, dt)
        assert native.sync_status() == 0


def test_kepler_host_drop_in_one_pair_in_place(mods):
    native, _ = mods
    z, sets = load_kepler()
    D = ctypes.POINTER(ctypes.c_double)
    dt = 0.37
    want = z["out_bound_%r" % dt]
    for p in range(3):
        arr = {f: np.ascontiguousarray(sets["bound"][f][2 * p:2 * p + 2]) for f in P8}
        ptr = {f: arr[f].ctypes.data_as(D) for f in P8}
        native.lib.kepler_solver_kernel(*[ptr[f] for f in P8], dt,
                                        *[ptr[f] for f in ("rx", "ry", "rz", "vx", "vy", "vz")])
        got = np.stack([arr[f] for f in ("rx", "ry", "rz", "vx", "vy", "vz")])
        assert kepler_close(got, want[:, 2 * p:2 * p + 2])


def test_kepler_bound_reached_is_reported(mods):
    native, ext = mods
    d = {f: np.zeros(2) for f in P8}
    d["mass"][:] = [0.5, 0.5]
    d["rx"][:] = [1e-3, -1e-3]
    d["vy"][:] = [10.0, -10.0]
    d["eps2"][:] = [1e-7, 1e-7]
    P = PS(d, P8)
    native.sync_status()
    with pytest.warns(RuntimeWarning, match="retry bound"):
        ext.Kepler("CUDA").calc(P, P, 0.37)
    assert all(torch.isfinite(getattr(P, f)).all() for f in P8)


def test_kepler_odd_count_rejected(mods):
    _, ext = mods
    d = {f: np.ones(3) for f in P8}
    P = PS(d, P8)
    with pytest.raises(ValueError):
        ext.Kepler("CUDA").calc(P, P, 0.1)


@pytest.mark.parametrize("n", [0, 1, 5, 7, 8, 9, 127, 128, 129, 136, 255, 256, 264, 1000, 4097, 65537, 300001])
def test_sum_equals_numpy(mods, n):
    native, _ = mods
    rng = np.random.default_rng(n)
    a = rng.normal(size=n) * np.exp(rng.normal(size=n) * 6)
    t = torch.tensor(a, dtype=torch.float64, device="cuda")
    assert native.psum(t) == float(np.sum(a))


def test_sum_negative_zero(mods):
    native, _ = mods
    t = torch.tensor([-0.0, -0.0, -0.0], dtype=torch.float64, device="cuda")
    got = native.psum(t)
    assert got == 0.0 and np.copysign(1.0, got) == np.copysign(1.0, float(np.sum(np.array([-0.0] * 3))))


def test_div3_is_ieee_division(mods):
    native, _ = mods
    rng = np.random.default_rng(1)
    m = [rng.normal(size=1001) for _ in range(3)]
    d = 0.7300000000000001
    T = [torch.tensor(x, dtype=torch.float64, device="cuda") for x in m]
    O = [torch.empty_like(x) for x in T]
    native.check(native.lib.tg_div3(1001, *[o.data_ptr() for o in O], *[t.data_ptr() for t in T], d,
                                    torch.cuda.current_stream().cuda_stream), "tg_div3")
    for o, x in zip(O, m):
        assert np.array_equal(o.cpu().numpy(), x / d)
