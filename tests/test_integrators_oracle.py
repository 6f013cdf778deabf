"""The CPU restatement of the reference integrators (oracle/integrators.py)
reproduces the reference integrators' trajectories (golden fixtures made by
running tupan/integrator/{hermite,sia,sakura,nreg}.py with the reference C
kernels): bit-identical final states, particle order and step counts."""
import numpy as np
import pytest

from golden_traj import RUNS, RV, final_ids, final_state, initial_state, load, run_config
from oracle import integrators as oi


@pytest.mark.parametrize("method", RUNS)
def test_oracle_integrator_matches_reference(method):
    z = load()
    eta, t_end, eps2, steps, t_final = run_config(z, method)
    ps = oi.make_ps(initial_state(z, eps2))
    integ = oi.integrator(method, eta, ps, oi.Kernels(nthreads=2))
    n = 0
    while abs(integ.t_curr) < abs(t_end):
        integ.evolve_step(t_end)
        n += 1
    assert n == steps and integ.t_curr == t_final
    got = np.stack([integ.ps[f] for f in RV])
    ids = final_ids(z, method)
    if ids is not None:
        assert np.array_equal(integ.ps["id"], ids), method
    assert np.array_equal(got, final_state(z, method)), method
