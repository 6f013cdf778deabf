"""Initial-condition generators on the CPU (tupan_gb300.ics): the Salpeter
sampler's range and slope, the triangular velocity fraction, the Plummer
arrays' normalisation and Henon-unit energies, and the two-body orbit of
tupan/ics/fewbody.py:13-50."""
import numpy as np

from tupan_gb300.ics import EqualMass, Salpeter, make_binary, plummer_arrays, triangular


def test_salpeter_range_and_slope():
    rng = np.random.default_rng(1)
    m = Salpeter(0.1, 100.0).sample(200000, rng)
    assert m.min() >= 0.1 and m.max() <= 100.0
    # maximum-likelihood slope of a power law truncated to [0.1, 100]
    slopes = np.linspace(-2.6, -2.1, 501)
    ll = []
    for a in slopes:
        b = a + 1
        norm = (100.0 ** b - 0.1 ** b) / b
        ll.append(a * np.log(m).sum() - m.size * np.log(norm))
    assert abs(slopes[int(np.argmax(ll))] + 2.35) < 0.01
    assert np.array_equal(EqualMass().sample(5, rng), np.ones(5))


def test_triangular_density():
    q = triangular(400000, np.random.default_rng(2))
    assert q.min() >= 0 and q.max() <= 1
    assert abs(q.mean() - 1 / 3) < 3e-3            # density 2(1 - q): mean 1/3
    assert abs((q < 0.5).mean() - 0.75) < 3e-3      # P(q < 1/2) = 3/4


def test_plummer_arrays_units():
    d = plummer_arrays(20000, 1e-3, imf=Salpeter(0.1, 100.0), seed=3)
    m = d["mass"]
    assert abs(m.sum() - 1) < 1e-12
    assert np.allclose(d["eps2"], 0.5e-6)
    for c in "xyz":    # centre of mass at rest at the origin
        assert abs(np.dot(m, d["r" + c])) < 1e-12
        assert abs(np.dot(m, d["v" + c])) < 1e-12
    ke = 0.5 * (m * (d["vx"] ** 2 + d["vy"] ** 2 + d["vz"] ** 2)).sum()
    assert abs(ke - 0.25) < 1e-12                   # Henon units: K = 1/4 for a virialised sphere
    r = np.sqrt(d["rx"] ** 2 + d["ry"] ** 2 + d["rz"] ** 2)
    # half-mass radius of a Plummer sphere in Henon units: 0.769
    order = np.argsort(r)
    rh = r[order][np.searchsorted(np.cumsum(m[order]), 0.5)]
    assert abs(rh - 0.769) < 0.05
    e = plummer_arrays(100, 0.01, seed=3)
    assert np.array_equal(e["rx"], plummer_arrays(100, 0.01, seed=3)["rx"])   # seeded


def test_binary_orbit():
    m1, m2, a, e = 0.3, 0.7, 1e-3, 0.6
    m, r, v = make_binary(m1, m2, a, e, np.random.default_rng(4))
    assert np.allclose(m @ r, 0, atol=1e-18) and np.allclose(m @ v, 0, atol=1e-15)
    dr, dv = r[0] - r[1], v[0] - v[1]
    M = m1 + m2
    energy = 0.5 * dv @ dv - M / np.linalg.norm(dr)
    assert abs(-M / (2 * energy) - a) < 1e-12 * a * 1e3          # semi-major axis
    h = np.cross(dr, dv)
    ecc = np.linalg.norm(np.cross(dv, h) / M - dr / np.linalg.norm(dr))
    assert abs(ecc - e) < 1e-9
    assert abs(np.linalg.norm(dr) - a * (1 - e)) < 1e-15          # starts at pericentre
