"""The reference's own integrators, unmodified, on this backend.

tupan's integrators reach the pairwise kernels only through
tupan/lib/extensions.py: `extensions.<kernel>.calc(ips, jps, ...)` on their
numpy particle sets (tupan/particles/body.py:324-361, integrator/sakura.py:30-38,
fewbody.py:41, nreg.py:27-53; the post-Newtonian switch through
`extensions.clight`, integrator/__init__.py:33-35).  Here, in a fresh
process, the reference tree installed in baseline/_ref is put on sys.path
and `tupan.lib.extensions` is pointed at tupan_gb300.lib.extensions before
anything of tupan.integrator is imported; the reference's Integrator and
ParticleSystem then run as they are.  Their final states are compared with
the trajectories the reference itself produced with its C backend
(tests/golden/golden_integrators.npz): Hermite and SIA bit-identical,
Sakura within 1e-9 of the state's scale (CUDA's transcendentals differ from
glibc by an ulp in the Kepler solve).  Step counts and final times exact.
The reference's ahermite4 also runs once with tupan_gb300.io.IO as its
dumpper (dump_freq 1): the worldline it writes through the reference's own
hooks (hermite.py:318-327, 402-405) equals, row for row, the one the CPU
restatement of the integrator collects.

Skipped when no installed reference tree is present.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from golden_traj import KEPLER_RUNS, RV, final_state, load, run_config  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")
METHODS = ("ahermite4", "sia21s.kdk", "sakura", "hermite6", "nreg")

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(ref)r)
sys.path.insert(1, %(root)r)
import tupan.lib
import tupan_gb300.lib.extensions as backend
tupan.lib.extensions = backend
sys.modules["tupan.lib.extensions"] = backend
from tupan.integrator import Integrator
from tupan.particles.allparticles import ParticleSystem
assert sys.modules["tupan.lib.extensions"] is backend
z = np.load(%(golden)r)
ics = {k[3:]: z[k] for k in z.files if k.startswith("ic_")}
out = {}
for method in %(methods)r:
    eta, t_end, eps2, steps, t_final = [float(x) for x in z["cfg_" + method.replace(".", "_")]]
    ps = ParticleSystem(len(ics["mass"]))
    for k, v in ics.items():
        getattr(ps, k)[...] = v
    ps.eps2[...] = eps2
    integ = Integrator(eta, 0.0, ps, method=method)
    n = 0
    while abs(integ.time) < abs(t_end):
        integ.evolve_step(t_end)
        n += 1
    p = integ.particle_system
    out[method] = {"steps": n, "time": integ.time, "state": [np.asarray(getattr(p, f)).tolist() for f in %(rv)r],
                   "backend": type(backend.acc_jerk.kernel).__module__}
from tupan_gb300.io import IO
eta, t_end, eps2, steps, t_final = [float(x) for x in z["cfg_ahermite4"]]
ps = ParticleSystem(len(ics["mass"]))
for k, v in ics.items():
    getattr(ps, k)[...] = v
ps.eps2[...] = eps2
io = IO(%(wl)r, "a")
integ = Integrator(eta, 0.0, ps, method="ahermite4", dumpper=io, dump_freq=1)
while abs(integ.time) < abs(t_end):
    integ.evolve_step(t_end)
print("RESULT" + json.dumps(out))
"""


@pytest.fixture(scope="module")
def runs():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.isdir(os.path.join(REF, "tupan", "integrator")):
        pytest.skip("no installed reference tree (baseline/_ref)")
    from golden_io import GOLDEN
    home = tempfile.mkdtemp(prefix="tupan_home_")
    wl = os.path.join(home, "worldline.hdf5")
    code = CHILD % {"ref": REF, "root": ROOT, "golden": os.path.join(GOLDEN, "golden_integrators.npz"),
                    "methods": METHODS, "rv": RV, "wl": wl}
    env = dict(os.environ, HOME=home, TUPAN_GB300_PREC="float64")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.split("RESULT", 1)[1])
    out["worldline_file"] = wl
    return out


@pytest.mark.parametrize("method", METHODS)
def test_reference_integrator_runs_unchanged_on_this_backend(runs, method):
    z = load()
    eta, t_end, eps2, steps, t_final = run_config(z, method)
    r = runs[method]
    assert r["backend"] == "tupan_gb300.lib.extensions"
    assert r["steps"] == steps and r["time"] == t_final, (r["steps"], steps, r["time"], t_final)
    got, want = np.array(r["state"]), final_state(z, method)
    if method in KEPLER_RUNS:
        assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max()
    else:
        assert np.array_equal(got, want), method


def test_reference_integrator_dumps_through_this_io(runs):
    from golden_traj import initial_state
    from oracle import integrators as oi
    from tupan_gb300.io import IO
    z = load()
    eta, t_end, eps2, _steps, _t = run_config(z, "ahermite4")
    ref = oi.integrator("ahermite4", eta, oi.make_ps(initial_state(z, eps2)), oi.Kernels(nthreads=2), dump_freq=1)
    while abs(ref.t_curr) < abs(t_end):
        ref.evolve_step(t_end)
    got = IO(runs["worldline_file"], "r").load_worldline()
    assert got.n == sum(p.n for p in ref.worldline) > 48
    for k in ("id", "mass", "rx", "ry", "rz", "vx", "vy", "vz", "time", "nstep", "tstep"):
        want = np.concatenate([p[k] for p in ref.worldline])
        assert np.array_equal(getattr(got, k).cpu().numpy(), want), k
