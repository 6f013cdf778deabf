"""Run diagnostics (tupan_gb300.diagnostic.Diagnostic, after
tupan/simulation.py:39-129) on a GPU-resident Plummer sphere advanced by the
GPU leapfrog: the report file has the reference's header and one line per
report; the energies equal the host recomputation from the same arrays bit
for bit (numpy-order sums; potential from the oracle's Phi, which the FP64
kernel reproduces exactly); eerr, geerr and the drifts follow their
definitions."""
import math

import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle.oracle import Oracle
    from tupan_gb300 import diagnostic, integrator
    from tupan_gb300.ics import plummer_arrays
    from tupan_gb300.lib import extensions
    from tupan_gb300.particles import ParticleSystem
    extensions.set_precision("float64")
    return diagnostic, integrator, plummer_arrays, ParticleSystem, Oracle()


def host_energies(ps, orc):
    d = {f: getattr(ps, f).cpu().numpy() for f in ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")}
    ke = (0.5 * d["mass"] * (d["vx"] ** 2 + d["vy"] ** 2 + d["vz"] ** 2)).sum()
    phi = orc.calc("phi", d, d, nthreads=4)[0]
    pe = 0.5 * (d["mass"] * phi).sum()
    return float(ke), float(pe)


def test_diagnostic_report_follows_the_reference(mods, tmp_path):
    diagnostic, integrator, plummer_arrays, ParticleSystem, orc = mods
    ps = ParticleSystem.from_arrays(**plummer_arrays(512, 0.01, seed=3))
    fname = str(tmp_path / "diag.txt")
    integ = integrator.Integrator(1.0 / 256, 0.0, ps, method="sia21s.kdk")
    diag = diagnostic.Diagnostic(fname, 0.0, integ.particle_system, report_freq=2)
    ke0, pe0 = host_energies(integ.particle_system, orc)
    eerrs = []
    for step in range(6):
        diag.diagnostic_report(integ.particle_system)
        if step % 2 == 0:
            ke, pe = host_energies(integ.particle_system, orc)
            last = diag.last
            assert last["ke"] == ke and last["pe"] == pe and last["te"] == ke + pe
            eerr = ((ke + pe) - (ke0 + pe0)) / (-pe)
            assert last["eerr"] == eerr
            eerrs.append(eerr)
            assert last["geerr"] == math.sqrt(sum(e * e for e in eerrs) / len(eerrs))
            assert last["virial"] == 2 * ke + pe
            assert last["time"] == integ.time
        integ.evolve_step(1.0)
    lines = open(fname).read().splitlines()
    assert lines[0].split() == list(diagnostic.COLUMNS)
    assert len(lines) == 1 + 3
    cols = [float(x) for x in lines[-1].split()]
    assert len(cols) == len(diagnostic.COLUMNS)
    assert abs(cols[6] - eerrs[-1]) <= 1e-3 * abs(eerrs[-1]) + 1e-300   # printed to 4 digits
    assert 0 < abs(eerrs[-1]) < 1e-4    # a short, smooth leapfrog run
    # the sphere starts with its centre of mass at rest at the origin
    assert diag.last["com_v"] < 1e-12 and diag.last["lmom"] < 1e-12
