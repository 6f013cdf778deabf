"""Physical invariants of the batched Kepler pair solver (tg_kepler_solver
through extensions.Kepler, the two-body step of FewBody and of the Sakura
kernel's pairs): 64 unsoftened bound binaries built like
tupan/ics/fewbody.py:13-50 (pericentre start, random orientation,
eccentricities up to 0.9) that share one orbital period P.  Three calls of
P/3 each bring every pair back to its initial state, and every call keeps
each pair's energy and angular momentum.

Tolerances: closure 1e-10 of the semi-major axis and of the pericentre
speed (the CPU oracle of the same algorithm closes to 2e-13 / 1e-12);
energy and angular momentum 1e-11 relative (oracle: 4e-14 and 1e-15)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

F8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")


class PS(object):
    def __init__(self, d):
        self.n = len(d["mass"])
        for f in F8:
            setattr(self, f, torch.as_tensor(d[f], dtype=torch.float64, device="cuda"))


def binaries(nb, period, seed):
    from tupan_gb300.ics import make_binary
    rng = np.random.default_rng(seed)
    d = {f: np.zeros(2 * nb) for f in F8}
    a_s, vp_s = np.zeros(nb), np.zeros(nb)
    for b in range(nb):
        m1, m2 = rng.uniform(0.1, 1.0, 2) / 1000
        e = 0.9 * np.sqrt(rng.random())
        M = m1 + m2
        a = (M * (period / (2 * np.pi)) ** 2) ** (1.0 / 3.0)
        m, r, v = make_binary(m1, m2, a, e, rng)
        a_s[b], vp_s[b] = a, np.sqrt(M * (1 + e) / (a * (1 - e)))
        d["mass"][2 * b:2 * b + 2] = m
        for k, c in enumerate("xyz"):
            d["r" + c][2 * b:2 * b + 2] = r[:, k]
            d["v" + c][2 * b:2 * b + 2] = v[:, k]
    return d, a_s, vp_s


def state(P):
    return {f: getattr(P, f).cpu().numpy() for f in F8}


def invariants(s):
    """Per pair: relative-orbit energy and angular momentum vector."""
    m = s["mass"].reshape(-1, 2)
    r = np.stack([s["r" + c].reshape(-1, 2) for c in "xyz"])
    v = np.stack([s["v" + c].reshape(-1, 2) for c in "xyz"])
    dr, dv = r[:, :, 0] - r[:, :, 1], v[:, :, 0] - v[:, :, 1]
    M = m.sum(1)
    E = 0.5 * (dv * dv).sum(0) - M / np.sqrt((dr * dr).sum(0))
    L = np.cross(dr.T, dv.T)
    return E, L


def test_kepler_pairs_close_after_one_period_and_conserve():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    from tupan_gb300.lib import extensions
    period = 2 * np.pi * 1e-5
    d, a_s, vp_s = binaries(64, period, seed=64)
    P = PS(d)
    E0, L0 = invariants(d)
    _native.sync_status()
    for _ in range(3):
        extensions.Kepler("CUDA").calc(P, P, period / 3)
        torch.cuda.synchronize()
        E, L = invariants(state(P))
        assert np.abs((E - E0) / E0).max() < 1e-11
        assert (np.linalg.norm(L - L0, axis=1) / np.linalg.norm(L0, axis=1)).max() < 1e-11
    assert _native.sync_status() == 0
    s = state(P)
    dr = np.sqrt(sum((s["r" + c] - d["r" + c]) ** 2 for c in "xyz")).reshape(-1, 2).max(1) / a_s
    dv = np.sqrt(sum((s["v" + c] - d["v" + c]) ** 2 for c in "xyz")).reshape(-1, 2).max(1) / vp_s
    assert dr.max() < 1e-10 and dv.max() < 1e-10, (dr.max(), dv.max())
