"""GPU integrators (tupan_gb300.integrator, FP64 kernels + fused FP64
updates) against the reference integrators' trajectories.

* Hermite, SIA21 and NREG: bit-identical final states and step counts (the FP64
  kernels, the fused updates and the numpy-order sums keep the reference's
  operation order).
* Sakura and the hierarchical SIA runs (whose two-body subsystems use the
  Kepler pair solver): the Kepler branch uses CUDA's transcendental
  functions, which differ from glibc by an ulp, so final states agree to
  1e-9 of their scale; step counts, final time and particle order are exact.
* Configuration 1 at full size: adaptive 4th-order Hermite, Plummer N=4096,
  eps2 = 1e-4, eta = 0.01, to t = 1/8, against the CPU restatement of the
  reference integrator: bit-identical.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from golden_traj import (KEPLER_RUNS, RUNS, RV, final_ids, final_state, initial_state, load,  # noqa: E402
                         run_config)


@pytest.fixture(scope="module")
def modules():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import integrator
    from tupan_gb300.lib import extensions
    from tupan_gb300.particles import ParticleSystem
    extensions.set_precision("float64")
    return integrator, ParticleSystem


def run_gpu(modules, d, method, eta, t_end):
    integrator, ParticleSystem = modules
    ps = ParticleSystem.from_arrays(**d)
    integ = integrator.Integrator(eta, 0.0, ps, method=method)
    steps = 0
    while abs(integ.time) < abs(t_end):
        integ.evolve_step(t_end)
        steps += 1
    out = integ.particle_system
    return steps, integ.time, np.stack([getattr(out, f).cpu().numpy() for f in RV]), out.id.cpu().numpy()


@pytest.mark.parametrize("method", RUNS)
def test_gpu_integrator_matches_reference_trajectory(modules, method):
    z = load()
    eta, t_end, eps2, steps, t_final = run_config(z, method)
    n, t, got, ids = run_gpu(modules, initial_state(z, eps2), method, eta, t_end)
    want = final_state(z, method)
    assert n == steps and t == t_final
    want_ids = final_ids(z, method)
    if want_ids is not None:
        assert np.array_equal(ids, want_ids), method
    if method in KEPLER_RUNS:
        assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max()
    else:
        assert np.array_equal(got, want), method


def test_config1_ahermite4_plummer_4096_full_run(modules):
    """Configuration 1 at full size against tests/golden/golden_config1.npz
    (made by tests/golden/make_config1.py with the CPU restatement of the
    reference integrator): same step count, bit-identical final state."""
    import os
    from golden_io import GOLDEN
    g = np.load(os.path.join(GOLDEN, "golden_config1.npz"))
    d = {k[3:]: g[k] for k in g.files if k.startswith("ic_")}   # stored: see make_config1.py
    n, t, got, _ = run_gpu(modules, d, "ahermite4", float(g["eta"]), float(g["t_end"]))
    assert n == int(g["steps"]) and t == float(g["t_final"])
    assert np.array_equal(got, np.stack([g[f] for f in RV]))
