"""Non-finite inputs, injected on the host: a NaN position in one particle
and an infinite velocity in another.  Every kernel returns and raises no
status bit.  FP64 reproduces the CPU oracle (the reference algorithm)
exactly: the same non-finite outputs and the same bits elsewhere.  Split
FP32 (for these small sets the double-single kernel of Acc and AccJerk, the
unordered split-FP32 kernels of Phi and Tstep) is non-finite at least
wherever the reference is."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

F8 = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")
KCLASS = {"phi": "Phi", "acc": "Acc", "acc_jerk": "AccJerk", "tstep": "Tstep"}
SCALARS = {"tstep": (1.0 / 64,)}


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
    from oracle.oracle import Oracle
    from tupan_gb300 import _native
    from tupan_gb300.lib import extensions
    return _native, extensions, Oracle()


def particles(n, seed):
    rng = np.random.default_rng(seed)
    d = {"mass": rng.random(n) / n, "eps2": np.full(n, 1e-4)}
    for c in "xyz":
        d["r" + c] = rng.normal(size=n)
        d["v" + c] = rng.normal(size=n) * 0.3
    return d


@pytest.mark.parametrize("name", ["phi", "acc", "acc_jerk", "tstep"])
@pytest.mark.parametrize("prec", ["float64", "ds32"])
def test_nonfinite_inputs_follow_the_reference(mods, name, prec):
    native, ext, orc = mods
    d = particles(300, seed=21)
    d["rx"][5] = np.nan
    d["vy"][17] = np.inf
    native.sync_status()
    sc = SCALARS.get(name, ())
    got = np.stack([o.cpu().numpy() for o in getattr(ext, KCLASS[name])("CUDA", prec).calc(PS(d), PS(d), *sc)])
    torch.cuda.synchronize()
    assert native.sync_status() == 0
    want = np.stack(orc.calc(name, d, d, *sc, nthreads=4))
    if prec == "float64":
        assert np.array_equal(np.isfinite(got), np.isfinite(want)), name
        ok = np.isfinite(want)
        assert np.array_equal(got[ok], want[ok])
    else:
        assert not np.isfinite(got[~np.isfinite(want)]).any(), name


@pytest.mark.parametrize("name", ["acc", "acc_jerk"])
def test_nonfinite_inputs_on_the_ordered_path(mods, name):
    """4096 particles take the ordered split-FP32 path (Hilbert sort, block
    records, recompute): a NaN position and an infinite velocity still give
    non-finite results wherever the FP64 kernels (the reference's
    arithmetic) do, and no status bit."""
    native, ext, _ = mods
    d = particles(4096, seed=22)
    d["rx"][100] = np.nan
    d["vy"][3000] = np.inf
    native.sync_status()
    got = np.stack([o.cpu().numpy() for o in getattr(ext, KCLASS[name])("CUDA", "ds32").calc(PS(d), PS(d))])
    want = np.stack([o.cpu().numpy() for o in getattr(ext, KCLASS[name])("CUDA", "float64").calc(PS(d), PS(d))])
    torch.cuda.synchronize()
    assert native.sync_status() == 0
    assert not np.isfinite(got[~np.isfinite(want)]).any(), name
