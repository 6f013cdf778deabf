"""Sakura with its Kepler pairs solved apart (the default evaluation) against
the one-pass evaluation (tg_set_sakura_split(0)): the same bits for every
output and the same status, for flags -1 and +1.  Inputs: the binary-rich
golden set (Kepler and leapfrog pairs), a Plummer-Salpeter sphere, the
uniform test set of the reference (tupan/tests/test_extensions.py:28-36)
and a cold compact cluster whose pairs all take the Kepler solver -- more
than the term buffer holds, so the excess is evolved in the fold pass."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from golden_io import load  # noqa: E402

F8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")


class PS(object):
    def __init__(self, d):
        self.n = len(d["mass"])
        for f in F8:
            setattr(self, f, torch.as_tensor(np.ascontiguousarray(d[f]), dtype=torch.float64, device="cuda"))

    def register_auxiliary_attribute(self, name, sctype):
        setattr(self, name, torch.zeros(self.n, dtype=torch.float64, device="cuda"))


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native
    from tupan_gb300.lib import extensions
    yield _native, extensions
    _native.lib.tg_set_sakura_split(1)


def sets():
    from tupan_gb300.ics import Salpeter, plummer_arrays
    out = {"binary": load("binary")[1], "sweep": load("sweep")[1]}
    out["plummer"] = plummer_arrays(1500, 1e-3, imf=Salpeter(0.1, 100.0), seed=5)
    rng = np.random.default_rng(8)
    n = 400
    cold = {"mass": np.full(n, 1.0 / n), "eps2": np.zeros(n)}
    for c in "xyz":
        cold["r" + c] = rng.normal(size=n)
        cold["v" + c] = rng.normal(size=n) * 1e-3
    out["cold"] = cold
    return out


def run(native, ext, d, dt, flag, split):
    native.lib.tg_set_sakura_split(split)
    native.sync_status()
    P = PS({f: np.asarray(d[f], dtype=np.float64) for f in F8})
    out = ext.Sakura("CUDA", "float64").calc(P, P, dt, flag)
    torch.cuda.synchronize()
    status = native.sync_status()
    return np.stack([o.cpu().numpy() for o in out]), status


@pytest.mark.filterwarnings("ignore:sakura. Kepler retry bound")
@pytest.mark.parametrize("name", ["binary", "sweep", "plummer", "cold"])
@pytest.mark.parametrize("flag", [-1, 1])
def test_split_sakura_is_bit_identical_to_one_pass(mods, name, flag):
    native, ext = mods
    d = sets()[name]
    for dt in (1.0 / 64, 1.0 / 1024):
        one, s1 = run(native, ext, d, dt, flag, 0)
        two, s2 = run(native, ext, d, dt, flag, 1)
        assert s1 == s2, (name, flag, dt)
        bad = np.argwhere(one.view(np.int64) != two.view(np.int64))
        assert bad.size == 0, (name, flag, dt, bad[:3].tolist())


@pytest.mark.filterwarnings("ignore:sakura. Kepler retry bound")
@pytest.mark.parametrize("flag", [-1, 1])
def test_split_sakura_with_distinct_i_and_j_sets(mods, flag):
    """i-set a prefix of the j-set, and the reverse (ragged bitmap rows,
    rows shorter and longer than the j-range of a word)."""
    native, ext = mods
    from tupan_gb300.ics import Salpeter, plummer_arrays
    d = plummer_arrays(700, 1e-3, imf=Salpeter(0.1, 100.0), seed=13)
    for ni, nj in ((70, 700), (700, 45), (33, 33)):
        I = {f: np.asarray(d[f][:ni]) for f in F8}
        J = {f: np.asarray(d[f][:nj]) for f in F8}
        outs = []
        for split in (0, 1):
            native.lib.tg_set_sakura_split(split)
            native.sync_status()
            out = ext.Sakura("CUDA", "float64").calc(PS(I), PS(J), 1.0 / 256, flag)
            torch.cuda.synchronize()
            outs.append((np.stack([o.cpu().numpy() for o in out]), native.sync_status()))
        assert outs[0][1] == outs[1][1]
        assert np.array_equal(outs[0][0].view(np.int64), outs[1][0].view(np.int64)), (ni, nj)
