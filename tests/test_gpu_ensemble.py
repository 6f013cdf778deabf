"""Segmented (ensemble) kernels and the graph-captured ensemble Hermite step.

* FP64 segmented Phi/Acc/AccJerk/SnapCrackle: each cluster's results equal
  the single-set FP64 calls bit for bit (sizes 0, 1, 2, ... 1300, ragged).
* Split-FP32 segmented kernels against the CPU oracle per cluster.
* Determinism after the first-call autotune; a captured CUDA graph of one
  6th-order Hermite step reproduces the eager step exactly.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SIZES = [5, 0, 1, 2, 63, 64, 65, 255, 256, 511, 1000, 1300]
OUTS = {"phi": ("phi",), "acc": ("ax", "ay", "az"), "acc_jerk": ("ax", "ay", "az", "jx", "jy", "jz"),
        "snap_crackle": ("sx", "sy", "sz", "cx", "cy", "cz")}
TOL = {"phi": 2e-6, "acc": 4e-6, "acc_jerk": 4e-6, "snap_crackle": 5e-5}


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import ensemble
    from tupan_gb300.lib import extensions
    return ensemble, extensions


def clusters(seed=9):
    rng = np.random.default_rng(seed)
    out = []
    for n in SIZES:
        d = {"mass": rng.random(n) / max(n, 1), "eps2": np.full(n, 5e-5)}
        for c in "xyz":
            d["r" + c] = rng.normal(size=n)
            d["v" + c] = rng.normal(size=n) * 0.3
        out.append(d)
    return out


def fill_derivs(ens, seed=3):
    g = torch.Generator().manual_seed(seed)
    for k in ("ax", "ay", "az", "jx", "jy", "jz"):
        getattr(ens.ps, k).copy_(torch.randn(ens.ps.n, generator=g, dtype=torch.float64))


def per_cluster(ens, name, fn):
    bounds = np.concatenate([[0], np.cumsum(ens.counts)])
    res = []
    for a, b in zip(bounds[:-1], bounds[1:]):
        res.append(fn(a, b))
    return res


@pytest.mark.parametrize("name", list(OUTS))
def test_fp64_segmented_equals_single_set(mods, name):
    ensemble, extensions = mods
    ens = ensemble.Ensemble(clusters(), prec="float64")
    fill_derivs(ens)
    getattr(ens, name)()
    torch.cuda.synchronize()
    got = np.stack([getattr(ens.ps, k).cpu().numpy() for k in OUTS[name]])
    kern = {"phi": extensions.Phi, "acc": extensions.Acc, "acc_jerk": extensions.AccJerk,
            "snap_crackle": extensions.SnapCrackle}[name]("CUDA", "float64")
    bounds = np.concatenate([[0], np.cumsum(ens.counts)])
    for a, b in zip(bounds[:-1], bounds[1:]):
        if b == a:
            continue
        sub = ens.ps[int(a):int(b)]
        out = kern.calc(sub, sub)
        want = np.stack([o.cpu().numpy() for o in out])
        assert np.array_equal(got[:, a:b], want), (name, a, b)


@pytest.mark.parametrize("name", list(OUTS))
def test_ds32_segmented_against_oracle(mods, name):
    ensemble, _ = mods
    from oracle.oracle import Oracle
    orc = Oracle()
    ens = ensemble.Ensemble(clusters(), prec="ds32")
    fill_derivs(ens)
    getattr(ens, name)()
    torch.cuda.synchronize()
    got = np.stack([getattr(ens.ps, k).cpu().numpy() for k in OUTS[name]])
    host = ens.ps.to_numpy()
    bounds = np.concatenate([[0], np.cumsum(ens.counts)])
    for a, b in zip(bounds[:-1], bounds[1:]):
        if b == a:
            continue
        sub = {k: host[k][a:b] for k in host}
        want = np.stack(orc.calc(name, sub, sub, nthreads=4))
        groups = [(0,)] if name == "phi" else [(0, 1, 2), (3, 4, 5)][: len(OUTS[name]) // 3]
        for g in groups:
            d = np.sqrt(((got[list(g), a:b] - want[list(g)]) ** 2).sum(0))
            n = np.sqrt((want[list(g)] ** 2).sum(0))
            ok = n > 0
            assert np.all(d[ok] / n[ok] <= TOL[name]), (name, a, b)


def test_ds32_segmented_is_deterministic_after_tuning(mods):
    ensemble, _ = mods
    ens = ensemble.Ensemble(clusters(), prec="ds32")
    ens.acc_jerk()          # first call tunes
    ens.acc_jerk()
    a = ens.ps.ax.clone(), ens.ps.jz.clone()
    ens.acc_jerk()
    assert torch.equal(a[0], ens.ps.ax) and torch.equal(a[1], ens.ps.jz)


def test_graph_captured_hermite6_step_matches_eager(mods):
    """FP64, so both ensembles run identical kernels (no per-object tuning)."""
    ensemble, _ = mods
    cl = clusters(11)
    eager = ensemble.Ensemble(cl, prec="float64")
    graph = ensemble.Ensemble(cl, prec="float64")
    tau = 1.0 / 1024
    for _ in range(3):
        eager.hermite_step(tau)
    graph.capture(tau)          # one eager warm-up step; the captured step does not run
    graph.replay(2)
    torch.cuda.synchronize()
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        assert torch.equal(getattr(eager.ps, k), getattr(graph.ps, k)), k


def test_overlapping_segments_are_rejected(mods):
    ensemble, _ = mods
    from tupan_gb300 import _native
    with pytest.raises(_native.TupanGB300Error):
        ensemble.Segments([0, 5], [10, 10])
