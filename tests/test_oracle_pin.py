"""Pin the CPU oracle (oracle/tupan_oracle.c) to the reference.

1. Against the committed golden fixtures (made from the reference C backend by
   tests/golden/make_golden.py): bit-identical for Phi, Acc, AccJerk,
   SnapCrackle, Tstep and Sakura (same per-pair operation order, IEEE double,
   no contraction); PNAcc to 1e-13 of the largest |component| (the oracle
   evaluates the PN polynomial from a monomial table, not in the reference's
   nested order).
2. Where the reference tree has been built into oracle/_ref (this container),
   against the reference itself on fresh seeded inputs.
"""
import numpy as np
import pytest

from golden_io import CASES, FIELDS, PREFIXES, load, typed_scalars
from oracle.oracle import Oracle, ReferenceLib, reference_available

PN_TOL = 1e-13


@pytest.fixture(scope="module")
def orc():
    return Oracle()


def _check(name, got, want):
    got = np.stack(got)
    if name == "pnacc":
        scale = max(np.abs(want).max(), 1e-300)
        assert np.abs(got - want).max() <= PN_TOL * scale
    else:
        assert np.array_equal(got, want), name


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_golden(orc, case):
    z, ps, calls = load(case)
    for key, name, sc in calls:
        sc = typed_scalars(name, sc)
        _check(name, orc.calc(name, ps, ps, *sc, nthreads=2), z["out_" + key])


def test_oracle_prefix_sweeps(orc):
    """i=all vs j=prefix and i=prefix vs j=all (test_extensions.py:45-85)."""
    z, ps, calls = load("sweep")
    for key, name, sc in calls:
        if name == "sakura":
            continue
        sc = typed_scalars(name, sc)
        for p in PREFIXES:
            sub = {f: ps[f][:p] for f in FIELDS}
            _check(name, orc.calc(name, ps, sub, *sc), z["outJ%d_" % p + key])
            _check(name, orc.calc(name, sub, ps, *sc), z["outI%d_" % p + key])


def test_threads_do_not_change_results(orc):
    _, ps, _ = load("plummer")
    a = orc.calc("acc_jerk", ps, ps, nthreads=1)
    b = orc.calc("acc_jerk", ps, ps, nthreads=7)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_empty_sets(orc):
    _, ps, _ = load("edge")
    empty = {f: ps[f][:0] for f in FIELDS}
    assert all(len(x) == 0 for x in orc.calc("acc", empty, ps))
    out = orc.calc("acc", ps, empty)
    assert all(np.array_equal(x, np.zeros(5)) for x in out)


@pytest.mark.skipif(not reference_available(), reason="reference not built here")
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_matches_reference_build(orc, seed):
    ref = ReferenceLib()
    rng = np.random.default_rng(seed)
    n = 150
    ps = {f: rng.normal(size=n) for f in FIELDS}
    ps["mass"] = rng.random(n)
    ps["eps2"] = rng.random(n) * 1e-3
    for name, sc in [("phi", ()), ("acc", ()), ("acc_jerk", ()), ("snap_crackle", ()),
                     ("tstep", (0.01,)), ("pnacc", (7,) + tuple(0.05 ** k for k in range(1, 8)))]:
        _check(name, orc.calc(name, ps, ps, *sc), np.stack(ref.calc(name, ps, ps, *sc)))
    ps["eps2"][:] = 0.0     # Sakura's Kepler branch only terminates unsoftened
    for flag in (-2, -1, 1, 2):
        _check("sakura", orc.calc("sakura", ps, ps, 0.01, flag),
               np.stack(ref.calc("sakura", ps, ps, 0.01, flag)))


# ---------------------------------------------------------------------------
# NREG_X / NREG_V and the Kepler pair solver (golden_nreg.npz,
# golden_kepler.npz from tests/golden/make_golden.py --nreg-kepler).
# ---------------------------------------------------------------------------
NREG_DTS = (0.0, 1.0 / 64, -0.3)
KEPLER_DTS = (1.0 / 64, 0.37, -0.5)
KEPLER_KINDS = ("bound", "hyper", "soft", "edge")
P8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")


def load_nreg():
    import os
    from golden_io import GOLDEN
    return np.load(os.path.join(GOLDEN, "golden_nreg.npz"))


def load_kepler():
    import os
    from golden_io import GOLDEN
    z = np.load(os.path.join(GOLDEN, "golden_kepler.npz"))
    sets = {k: {f: z["in_%s_%s" % (k, f)] for f in P8} for k in KEPLER_KINDS}
    return z, sets


@pytest.mark.parametrize("case", CASES)
def test_oracle_nreg_matches_golden(orc, case):
    g = load_nreg()
    _, ps, _ = load(case)
    for dt in NREG_DTS:
        for name in ("nreg_x", "nreg_v"):
            key = "%s_%s_%r" % (case, name, dt)
            assert np.array_equal(np.stack(orc.calc(name, ps, ps, dt, nthreads=3)), g[key]), key


def test_oracle_nreg_prefix_sweeps(orc):
    g = load_nreg()
    _, ps, _ = load("sweep")
    for name in ("nreg_x", "nreg_v"):
        key = "sweep_%s_%r" % (name, 1.0 / 64)
        for p in PREFIXES:
            sub = {f: ps[f][:p] for f in FIELDS}
            assert np.array_equal(np.stack(orc.calc(name, ps, sub, 1.0 / 64)), g["J%d_" % p + key])
            assert np.array_equal(np.stack(orc.calc(name, sub, ps, 1.0 / 64)), g["I%d_" % p + key])


@pytest.mark.parametrize("kind", KEPLER_KINDS)
def test_oracle_kepler_matches_golden(orc, kind):
    z, sets = load_kepler()
    for dt in KEPLER_DTS:
        capped = []
        got = np.stack(orc.kepler(sets[kind], dt, nthreads=2, capped=capped))
        assert not any(capped), (kind, dt)
        assert np.array_equal(got, z["out_%s_%r" % (kind, dt)]), (kind, dt)


def test_oracle_kepler_reports_bounds(orc):
    """A softened close pair whose energy test cannot pass within the bounds
    (the reference keeps halving its sub-steps for millions of solves)."""
    ps = {f: np.zeros(2) for f in P8}
    ps["mass"][:] = [0.5, 0.5]
    ps["rx"][:] = [1e-3, -1e-3]
    ps["vy"][:] = [10.0, -10.0]
    ps["eps2"][:] = [1e-7, 1e-7]
    capped = []
    out = np.stack(orc.kepler(ps, 0.37, capped=capped))
    assert capped == [True]
    assert np.all(np.isfinite(out))


@pytest.mark.skipif(not reference_available(), reason="reference not built here")
def test_oracle_nreg_kepler_match_reference_build(orc):
    ref = ReferenceLib()
    rng = np.random.default_rng(3)
    n = 120
    ps = {f: rng.normal(size=n) for f in FIELDS}
    ps["mass"] = rng.random(n)
    ps["eps2"] = rng.random(n) * 1e-3
    for name in ("nreg_x", "nreg_v"):
        for dt in (0.01, -0.07):
            assert np.array_equal(np.stack(orc.calc(name, ps, ps, dt)), np.stack(ref.calc(name, ps, ps, dt)))
    from golden.make_golden import kepler_pairs
    pairs = kepler_pairs(np.random.default_rng(11), 6, "bound")
    capped = []
    got = np.stack(orc.kepler(pairs, 0.2, capped=capped))
    assert not any(capped)
    assert np.array_equal(got, np.stack(ref.kepler(pairs, 0.2)))
