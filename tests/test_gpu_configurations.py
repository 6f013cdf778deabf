"""Configuration runs under test (tupan_gb300.runs, seeded synthetic inputs).

* Precision form, shortened: Plummer N = 65536 with Salpeter masses on
  [0.1, 100], pair softening 1e-6, shared-step SIA21 kdk leapfrog with
  dt = 1/1024 (Tstep each step), 8 steps, split FP32 against FP64: the
  per-particle acceleration error at step 0 and at steps 4 and 8 within 1e-6,
  and |dE/E| of the split-FP32 run within twice the FP64 run's.
* Compact-binary-rich cluster, shortened: 2048 Plummer particles plus 64
  hard binaries (a log-uniform on [1e-4, 1e-3], thermal e on [0, 0.9]), PN
  kicks to 2.5PN (c = 1e4, split FP32) around FP64 Sakura steps, dt = 1/1024,
  to t = 1/128: no Kepler retry bound reached, every binary still bound
  within [0.05, 2] of its initial semi-major axis, energy finite.
"""
import math

import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def runs():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import runs as r
    return r


def test_precision_configuration_short(runs):
    out = runs.precision_run(n=65536, steps=8, dt=1.0 / 1024, probe_every=4)
    assert out["force_error_step0"]["max"] <= 1e-6, out["force_error_step0"]
    for p in out["ds32"]["force_error_probes"]:
        assert p["force_error"]["max"] <= 1e-6, p
    e32, e64 = out["ds32"]["rel_energy_error"], out["float64"]["rel_energy_error"]
    assert math.isfinite(e32) and e32 <= 2.0 * e64, (e32, e64)


def test_binaries_configuration_short(runs):
    out = runs.binaries_run(t_end=1.0 / 128)
    assert out["kepler_status"] == 0, out
    sep = out["binary_separation_over_a"]
    assert 0.05 <= sep["min"] and sep["max"] <= 2.0, sep
    assert math.isfinite(out["rel_energy_error_newtonian"])
