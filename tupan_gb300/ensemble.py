"""Ensembles of independent clusters advanced together on one GPU.

All clusters live in one structure-of-arrays particle set; a segment table
(`tg_segments_create`) says which contiguous range belongs to which cluster.
Each force evaluation is one segmented launch over every cluster's pairs
(in split FP32: one stream-K launch whose units span all clusters, with the
tile shape and grid picked by the library's first-call autotuner).  A 6th
(or 4th) order Hermite step with a shared step size needs no host
synchronisation, so it can be captured once in a CUDA graph and replayed.
"""
import ctypes

import numpy as np
import torch

from . import _native
from .integrator.hermite import DERIV, RV
from .particles import ParticleSystem

PREC = {"float64": _native.PREC_FP64, "ds32": _native.PREC_DS32}

_lib = _native.lib
_lib.tg_segments_create.restype = ctypes.c_void_p
_lib.tg_segments_create.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_longlong),
                                    ctypes.POINTER(ctypes.c_longlong)]
_lib.tg_segments_destroy.restype = None
_lib.tg_segments_destroy.argtypes = [ctypes.c_void_p]
for _name, _np in (("tg_phi_segmented", 6), ("tg_acc_segmented", 8), ("tg_acc_jerk_segmented", 14),
                   ("tg_snap_crackle_segmented", 20)):
    _fn = getattr(_lib, _name)
    _fn.restype = ctypes.c_int
    _fn.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * _np + [ctypes.c_int, ctypes.c_void_p]

P5 = ("mass", "rx", "ry", "rz", "eps2")
P8 = P5 + ("vx", "vy", "vz")
P14 = P8 + ("ax", "ay", "az", "jx", "jy", "jz")


class Segments(object):
    """Owner of a library segment table."""

    def __init__(self, starts, counts):
        s = (ctypes.c_longlong * len(starts))(*[int(x) for x in starts])
        c = (ctypes.c_longlong * len(counts))(*[int(x) for x in counts])
        self.handle = _lib.tg_segments_create(len(starts), s, c)
        if not self.handle:
            raise _native.TupanGB300Error("tg_segments_create: " + _native.last_error())
        self.starts = np.asarray(starts, dtype=np.int64)
        self.counts = np.asarray(counts, dtype=np.int64)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            _lib.tg_segments_destroy(h)
            self.handle = None


class Ensemble(object):
    """Independent clusters (list of attribute dicts) in one particle set."""

    def __init__(self, clusters, prec="ds32", device=None):
        counts = [len(c["mass"]) for c in clusters]
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
        cat = {k: np.concatenate([c[k] for c in clusters]) for k in P8}
        self.ps = ParticleSystem.from_arrays(device=device, **cat)
        for name in ("ax", "ay", "az", "jx", "jy", "jz", "sx", "sy", "sz", "cx", "cy", "cz", "phi"):
            self.ps.register_auxiliary_attribute(name, "real")
        self.segments = Segments(starts, counts)
        self.prec = PREC[prec]
        self.counts = np.array(counts)
        self.interactions = int((self.counts.astype(np.int64) ** 2).sum())
        self.graph = None

    @staticmethod
    def _stream():
        return _native.current_stream()

    def _call(self, name, ps, inputs, outputs):
        fn = getattr(_lib, name)
        rc = fn(self.segments.handle, *[getattr(ps, k).data_ptr() for k in inputs],
                *[getattr(ps, k).data_ptr() for k in outputs], self.prec, self._stream())
        _native.check(rc, name)

    def phi(self, ps=None):
        ps = ps or self.ps
        self._call("tg_phi_segmented", ps, P5, ("phi",))

    def acc(self, ps=None):
        ps = ps or self.ps
        self._call("tg_acc_segmented", ps, P5, ("ax", "ay", "az"))

    def acc_jerk(self, ps=None):
        ps = ps or self.ps
        self._call("tg_acc_jerk_segmented", ps, P8, ("ax", "ay", "az", "jx", "jy", "jz"))

    def snap_crackle(self, ps=None):
        ps = ps or self.ps
        self._call("tg_snap_crackle_segmented", ps, P14, ("sx", "sy", "sz", "cx", "cy", "cz"))

    def derivatives(self, ps, order):
        if order == 2:
            self.acc(ps)
        else:
            self.acc_jerk(ps)
            if order >= 6:
                self.snap_crackle(ps)

    # --- shared-step Hermite (hermite.py:56-67) ---------------------------
    def _predict(self, ps1, ps0, tau, order):
        rv = _native.ptr_array([getattr(ps1, k) for k in RV])
        der = _native.ptr_array([getattr(ps0, k) for k in DERIV[order]])
        _native.check(_lib.tg_hermite_predict(order, ps1.n, float(tau), rv, der, self._stream()),
                      "tg_hermite_predict")

    def _correct(self, ps1, ps0, tau, order):
        rv0 = _native.ptr_array([getattr(ps0, k) for k in RV])
        d0 = _native.ptr_array([getattr(ps0, k) for k in DERIV[order]])
        d1 = _native.ptr_array([getattr(ps1, k) for k in DERIV[order]])
        rv1 = _native.ptr_array([getattr(ps1, k) for k in RV])
        _native.check(_lib.tg_hermite_correct(order, ps1.n, float(tau), rv0, d0, d1, rv1, self._stream()),
                      "tg_hermite_correct")

    def hermite_step(self, tau, order=6):
        """One epec(2) step of every cluster with the shared step tau.
        The start-state copy lives in a persistent buffer so the step can be
        captured in a CUDA graph."""
        ps = self.ps
        if not hasattr(self, "_ps0"):
            self._ps0 = ps.copy()
        ps0 = self._ps0
        for k, v in ps._arrays().items():
            getattr(ps0, k).copy_(v)
        self.derivatives(ps0, order)
        self._predict(ps, ps0, tau, order)
        for _ in range(2):
            self.derivatives(ps, order)
            self._correct(ps, ps0, tau, order)
        ps.time += tau
        ps.nstep += 1

    def capture(self, tau, order=6):
        """Capture one Hermite step in a CUDA graph (after a warm-up step, so
        the library's autotuning and workspace growth happen outside)."""
        self.hermite_step(tau, order)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.hermite_step(tau, order)
        self.graph = g
        return g

    def replay(self, steps=1):
        for _ in range(steps):
            self.graph.replay()

    def energy(self):
        """Per-cluster total energy K + U (FP64 Phi)."""
        saved = self.prec
        self.prec = PREC["float64"]
        self.phi()
        self.prec = saved
        ps = self.ps
        k = 0.5 * ps.mass * (ps.vx ** 2 + ps.vy ** 2 + ps.vz ** 2)
        u = 0.5 * ps.mass * ps.phi
        e = (k + u).cpu().numpy()
        bounds = np.concatenate([[0], np.cumsum(self.counts)])
        return np.array([e[a:b].sum() for a, b in zip(bounds[:-1], bounds[1:])])


def random_ensemble(nclusters=512, nmin=64, nmax=8192, eps=0.01, base_seed=512):
    """Clusters with N log-uniform in [nmin, nmax], each a Plummer sphere
    seeded with base_seed + cluster index."""
    from .ics import plummer_arrays
    out = []
    for c in range(nclusters):
        rng = np.random.default_rng(base_seed + c)
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        out.append(plummer_arrays(n, eps, seed=base_seed + c))
    return out
