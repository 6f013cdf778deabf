"""The particle container's storage on the CPU (no GPU needed): attributes
are rows of one float64 and one int64 block; selection, concatenation,
copies and attribute registration keep the reference's semantics
(tupan/particles/body.py:26-39, 641-645; allparticles.py:64-76)."""
import numpy as np
import pytest
import torch

from tupan_gb300.particles import REAL_ATTRS, ParticleSystem


def system(n=6):
    return ParticleSystem.from_arrays(device="cpu", mass=np.arange(n) + 1.0, rx=np.arange(n) * 2.0,
                                      vy=-np.arange(n) * 1.0)


def test_rows_and_defaults():
    ps = system()
    assert ps.n == 6 and torch.equal(ps.id, torch.arange(6))
    assert torch.equal(ps.rx, torch.arange(6, dtype=torch.float64) * 2)
    for a in REAL_ATTRS:
        assert getattr(ps, a).shape == (6,)
    assert torch.equal(ps.nstep, torch.zeros(6, dtype=torch.int64))
    # assignment copies into the attribute's row; in-place updates stay in it
    ps.rx = ps.rx + 1
    ps.mass *= 2
    assert torch.equal(ps._real[REAL_ATTRS.index("rx")], ps.rx)
    assert torch.equal(ps.mass, 2 * (torch.arange(6, dtype=torch.float64) + 1))
    with pytest.raises(ValueError):
        ps.rx = torch.zeros(5, dtype=torch.float64)


def test_selection_keeps_order_and_all_attributes():
    ps = system()
    ps.register_auxiliary_attribute("ax", "real")
    ps.ax += torch.arange(6, dtype=torch.float64)
    mask = ps.rx > 5
    slow, fast = ps[mask], ps[~mask]
    assert slow.n == 3 and fast.n == 3
    assert slow.id.tolist() == [3, 4, 5] and fast.id.tolist() == [0, 1, 2]
    assert slow.ax.tolist() == [3.0, 4.0, 5.0]
    idx = torch.tensor([5, 0, 2])
    t = ps.take(idx)
    assert t.id.tolist() == [5, 0, 2] and t.rx.tolist() == [10.0, 0.0, 4.0]
    s = ps[1:3]
    assert s.n == 2 and s.id.tolist() == [1, 2]
    # a selection is a copy
    slow.rx.zero_()
    assert ps.rx[3] == 6.0


def test_append_and_copy():
    ps = system()
    a, b = ps[ps.id < 2], ps[ps.id >= 2]
    b.register_auxiliary_attribute("phi", "real")
    b.phi += 7
    a.append(b)      # attribute present on one side only: zero-filled on the other
    assert a.n == 6 and a.id.tolist() == list(range(6))
    assert a.phi.tolist() == [0, 0, 7, 7, 7, 7]
    c = a.copy()
    c.vy += 100
    assert a.vy.tolist() == (-np.arange(6.0)).tolist()
    e = ParticleSystem(0, device="cpu")
    a.append(e)
    assert a.n == 6


def test_registration():
    ps = system()
    ps.register_auxiliary_attribute("ax", "real")
    with pytest.raises(ValueError):
        ps.register_auxiliary_attribute("ax", "real")
    sub = ps[ps.id > 2]              # row views are made on first use
    with pytest.raises(ValueError):
        sub.register_auxiliary_attribute("ax", "real")
    for k in range(40):              # more than the spare rows: the block grows
        ps.register_auxiliary_attribute("x%d" % k, "real")
    ps.x39 += 1
    assert ps.x39.tolist() == [1.0] * 6 and ps.rx.tolist() == [0.0, 2.0, 4.0, 6.0, 8.0, 10.0]
    assert not hasattr(ps, "nonexistent")
