"""Snapshot and worldline files from GPU-resident particle sets.

* Snapshots of a 65536-particle Plummer-Salpeter set round-trip bit-exactly,
  through the synchronous path and through the background writer (pinned
  copies, encoding on the writer thread); a PSDF stream of a set with its
  potential does too.
* Worldlines: the GPU integrators with a dumpper write the rows the
  reference's dumpper receives -- the whole set before the first step, then
  per step the particles whose time is a multiple of dump_freq * tau
  (tupan/integrator/hermite.py:318-327, 402-405; sia.py:1114-1117 for the
  slow part of every level of the h. recursion) -- compared with the CPU
  restatement of the reference integrators run with the same dump_freq:
  ids, times, step counts and steps exact, positions and velocities exact
  for the FP64 runs and within 1e-9 of their scale for the runs whose
  two-body subsets use the Kepler solver (CUDA's transcendentals).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from golden_traj import KEPLER_RUNS, initial_state, load, run_config  # noqa: E402

FIELDS = ("id", "mass", "eps2", "rx", "ry", "rz", "vx", "vy", "vz", "time", "nstep", "tstep")


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import integrator, io
    from tupan_gb300.lib import extensions
    from tupan_gb300.particles import ParticleSystem
    extensions.set_precision("float64")
    return integrator, io, ParticleSystem


@pytest.mark.parametrize("background", [False, True])
def test_snapshot_round_trip_65536(mods, tmp_path, background):
    _integ, io, ParticleSystem = mods
    from tupan_gb300 import ics
    d = ics.plummer_arrays(65536, 1e-3, ics.Salpeter(0.1, 100.0), seed=20261203)
    ps = ParticleSystem.from_arrays(**d)
    ps.time.fill_(0.25)
    ps.nstep.copy_(torch.arange(ps.n, device=ps.time.device) % 7)
    path = str(tmp_path / "snap.hdf5")
    w = io.IO(path, "a", background=background)
    w.dump_snapshot(ps, 3)
    w.dump_worldline(ps[:1000])
    w.close()
    r = io.IO(path, "r")
    back = r.load_snapshot(3)
    assert back.n == ps.n and back.time.device.type == "cuda"
    for k in FIELDS:
        assert torch.equal(getattr(back, k), getattr(ps, k)), k
    wl = r.load_worldline()
    assert torch.equal(wl.rx, ps.rx[:1000])


def test_psdf_round_trip_from_the_device(mods, tmp_path):
    _integ, io, ParticleSystem = mods
    from tupan_gb300 import ics
    from tupan_gb300.lib import extensions
    ps = ParticleSystem.from_arrays(**ics.plummer_arrays(1000, 1e-2, seed=3))
    extensions.phi.calc(ps, ps)                     # registers phi on the set
    path = str(tmp_path / "s.psdf")
    io.IO(path, "w", background=True).dump_snapshot(ps)
    back = io.IO(path, "r").load_snapshot()
    for k in FIELDS[:10] + ("phi",):
        assert torch.equal(getattr(back, k), getattr(ps, k)), k


@pytest.mark.parametrize("method,dump_freq", [("ahermite4", 1), ("ahermite4", 4), ("sia21s.kdk", 2),
                                              ("sia21h.dkd", 1), ("nreg", 1), ("sakura", 1)])
def test_worldline_matches_oracle(mods, tmp_path, method, dump_freq):
    integrator, io, ParticleSystem = mods
    from oracle import integrators as oi
    z = load()
    eta, t_end, eps2, steps, _t = run_config(z, method)
    d = initial_state(z, eps2)
    path = str(tmp_path / "wl.hdf5")
    dumpper = io.IO(path, "a", background=True)
    integ = integrator.Integrator(eta, 0.0, ParticleSystem.from_arrays(**d), method=method,
                                  dumpper=dumpper, dump_freq=dump_freq)
    n = 0
    while abs(integ.time) < abs(t_end):
        integ.evolve_step(t_end)
        n += 1
    dumpper.close()
    ref = oi.integrator(method, eta, oi.make_ps(d), oi.Kernels(nthreads=2), dump_freq=dump_freq)
    while abs(ref.t_curr) < abs(t_end):
        ref.evolve_step(t_end)
    assert n == steps
    want = {k: np.concatenate([p[k] for p in ref.worldline]) for k in FIELDS if k in ref.worldline[0]}
    got = io.IO(path, "r").load_worldline()
    assert got.n == len(want["id"]) >= 48 + (48 if dump_freq == 1 else 0)
    for k in ("id", "time", "nstep", "tstep", "mass"):
        assert np.array_equal(getattr(got, k).cpu().numpy(), want[k]), k
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        g, w = getattr(got, k).cpu().numpy(), want[k]
        if method in KEPLER_RUNS:
            assert np.abs(g - w).max() <= 1e-9 * np.abs(w).max(), k
        else:
            assert np.array_equal(g, w), k
