"""Initial conditions against the reference's own generators (run from the
installed reference tree in child processes):

* the mass functions (tupan/ics/imf.py:20-112) restated in
  tupan_gb300.ics.IMF: the same normalisation, peak and, drawn from
  numpy's global random state with the same seed, the same samples bit for
  bit; a Generator draws from the same distribution;
* plummer_reference (tupan/ics/plummer.py:22-133, 213-221): the same
  particle set bit for bit for three mass functions, sizes, seeds and
  softening types, with the potential from the CPU oracle on both sides
  (on the GPU the FP64 Phi kernel gives the oracle's bits)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tupan_gb300.ics import IMF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")
CASES = [("equalmass", ()), ("salpeter1955", (0.5, 100.0)), ("padoan2007", (0.1, 10.0)),
         ("parravano2011", (0.01, 50.0))]

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(ref)r)
from tupan.ics.imf import IMF
out = {}
for name, args in %(cases)r:
    np.random.seed(20261204)
    s = getattr(IMF, name)(*args)
    out[name] = {"peak": s.peak, "mpeak": s.mpeak, "sample": s.sample(700).tolist()}
print("RESULT" + json.dumps(out))
"""


def test_imf_samples_equal_the_reference():
    if not os.path.isdir(os.path.join(REF, "tupan", "ics")):
        pytest.skip("no installed reference tree (baseline/_ref)")
    r = subprocess.run([sys.executable, "-c", CHILD % {"ref": REF, "cases": CASES}], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    ref = json.loads(r.stdout.split("RESULT", 1)[1])
    for name, args in CASES:
        np.random.seed(20261204)
        s = getattr(IMF, name)(*args)
        assert s.peak == ref[name]["peak"] and s.mpeak == ref[name]["mpeak"], name
        assert np.array_equal(s.sample(700), np.array(ref[name]["sample"])), name


def test_imf_ranges_and_generators():
    with pytest.raises(ValueError, match="Mass range outer of limits"):
        IMF.salpeter1955(0.1, 100.0)
    s = IMF.padoan2007(0.1, 10.0)
    m = s.sample(20000, np.random.default_rng(3))
    assert m.shape == (20000,) and m.min() >= 0.1 and m.max() <= 10.0
    # log-uniform proposals accepted with probability f(m) / peak: the
    # accepted masses' density per unit ln m follows f, within noise
    h, edges = np.histogram(np.log(m), bins=8, range=(np.log(0.1), np.log(10.0)))
    mid = np.exp(0.5 * (edges[1:] + edges[:-1]))
    want = s.func(mid) / s.func(mid).sum() * len(m)
    assert np.all(np.abs(h - want) < 5 * np.sqrt(want) + 0.02 * want)
    assert np.array_equal(IMF.equalmass().sample(10, np.random.default_rng(0)), np.ones(10))


PLUMMER_CHILD = r"""
import json, sys, types
import numpy as np
sys.path.insert(0, %(ref)r)
sys.path.insert(1, %(root)r)
from oracle.oracle import Oracle
orc = Oracle()


class _Phi(object):
    def calc(self, ips, jps):
        if not hasattr(ips, "phi"):
            ips.register_auxiliary_attribute("phi", "real")
        d = lambda p: {k: np.asarray(getattr(p, k)) for k in ("mass", "rx", "ry", "rz", "eps2")}
        ips.phi[...] = orc.calc("phi", d(ips), d(jps))[0]


import tupan.lib
fake = types.ModuleType("tupan.lib.extensions")
fake.phi = _Phi()
tupan.lib.extensions = fake
sys.modules["tupan.lib.extensions"] = fake
from tupan.ics.plummer import make_plummer
out = {}
for key, (n, eps, imf, seed, st) in %(cases)r.items():
    ps = make_plummer(n, eps, tuple(imf), seed=seed, softening_type=st)
    out[key] = {k: np.asarray(getattr(ps, k)).tolist()
                for k in ("id", "mass", "eps2", "rx", "ry", "rz", "vx", "vy", "vz")}
print("RESULT" + json.dumps(out))
"""
PLUMMER_CASES = {"equal": (300, 0.01, ["equalmass"], 5, 0),
                 "padoan": (257, 1e-3, ["padoan2007", 0.1, 10.0], 11, 2),
                 "salpeter": (64, 0.05, ["salpeter1955", 0.5, 100.0], 3, 3)}


def test_plummer_reference_equals_the_reference_model():
    # the reference's make_plummer run from its installed tree, its Phi
    # calls answered by the CPU oracle (bit-identical to its C backend),
    # against plummer_reference with the same oracle Phi: equal bit for bit
    from oracle.oracle import Oracle
    from tupan_gb300.ics import plummer_reference
    if not os.path.isdir(os.path.join(REF, "tupan", "ics")):
        pytest.skip("no installed reference tree (baseline/_ref)")
    import tempfile
    r = subprocess.run([sys.executable, "-c", PLUMMER_CHILD % {"ref": REF, "root": ROOT, "cases": PLUMMER_CASES}],
                       capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, HOME=tempfile.mkdtemp(prefix="tupan_home_")))
    assert r.returncode == 0, r.stderr[-2000:]
    ref = json.loads(r.stdout.split("RESULT", 1)[1])
    orc = Oracle()

    def phi(mass, rx, ry, rz, eps2):
        d = {"mass": mass, "rx": rx, "ry": ry, "rz": rz, "eps2": eps2}
        return orc.calc("phi", d, d)[0]
    for key, (n, eps, imf, seed, st) in PLUMMER_CASES.items():
        ps = plummer_reference(n, eps, tuple(imf), seed=seed, softening_type=st, device="cpu", phi=phi)
        for k, v in ref[key].items():
            assert np.array_equal(getattr(ps, k).numpy(), np.array(v)), (key, k)
