"""The hierarchical SIA step driven natively (tg_sia_h_step) against the same
recursion driven from Python over the extension calls
(tupan_gb300.integrator.sia.SIA.recurse, which follows
tupan/integrator/sia.py:24-57, 175-230, 1092-1123 and fewbody.py:13-57).

Both make the same kernel calls with the same arguments in the same order,
so every attribute that the step reads or writes -- positions, velocities,
per-particle time, step and step count, ids (the particle order after the
slow/fast splits and joins) -- and the integrator's current time must agree
bit for bit, in FP64 and in split FP32.  Sizes: 200 particles (one
partition chunk, several hundred levels per step, Kepler pairs at the
leaves) and 2500 (three chunks, so the partition's cross-chunk prefix is
used).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

STATE = ("rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep", "nstep", "id")


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300.ics import plummer_arrays
    from tupan_gb300.integrator import Integrator, sia
    from tupan_gb300.lib import extensions
    from tupan_gb300.particles import ParticleSystem
    return plummer_arrays, Integrator, sia, extensions, ParticleSystem


def run(mods, n, method, native, steps, eta=1.0 / 64):
    plummer_arrays, Integrator, sia, _, ParticleSystem = mods
    d = plummer_arrays(n, 0.0, seed=n)
    d["eps2"] = np.zeros(n)
    ps = ParticleSystem.from_arrays(**d)
    integ = Integrator(eta, 0.0, ps, method=method)
    integ.integrator.native_h = native
    for k in range(steps):
        integ.evolve_step((k + 1) * eta)
    out = integ.particle_system
    return integ.time, {f: getattr(out, f).cpu().numpy() for f in STATE}


@pytest.mark.parametrize("prec", ["float64", "ds32"])
@pytest.mark.parametrize("method", ["sia21h.dkd", "sia21h.kdk", "sia22h.dkd", "sia44h.kdk"])
def test_native_h_step_equals_python_recursion(mods, method, prec):
    ext = mods[3]
    ext.set_precision(prec)
    try:
        t_py, py = run(mods, 200, method, native=False, steps=2)
        t_nat, nat = run(mods, 200, method, native=True, steps=2)
    finally:
        ext.set_precision("float64")
    assert t_nat == t_py
    for f in STATE:
        assert np.array_equal(nat[f], py[f]), (method, prec, f)
    assert not np.array_equal(nat["id"], np.arange(200))   # the splits did reorder


def test_native_h_step_multi_chunk_partition(mods):
    mods[3].set_precision("float64")
    t_py, py = run(mods, 2500, "sia21h.dkd", native=False, steps=1)
    t_nat, nat = run(mods, 2500, "sia21h.dkd", native=True, steps=1)
    assert t_nat == t_py
    for f in STATE:
        assert np.array_equal(nat[f], py[f]), f


def test_native_h_step_rejects_bad_rows(mods):
    import ctypes
    from tupan_gb300 import _native
    kinds = (ctypes.c_int * 3)(0, 1, 0)
    coefs = (ctypes.c_double * 3)(0.5, 1.0, 0.5)
    rows = (ctypes.c_int * 15)(*range(14), 5)    # nstep row 5 of a 2-row int block
    buf = torch.zeros(20, 4, dtype=torch.float64, device="cuda")
    ib = torch.zeros(2, 4, dtype=torch.int64, device="cuda")
    t = ctypes.c_double(0.0)
    rc = _native.lib.tg_sia_h_step(3, kinds, coefs, 1, 0.01, 0.01, 0, 0, 4, buf.data_ptr(), 4, 20,
                                   ib.data_ptr(), 4, 2, rows, ctypes.byref(t), None)
    assert rc == -1 and "row" in _native.last_error()
