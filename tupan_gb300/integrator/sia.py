"""Shared-step SIA21 leapfrog (tupan/integrator/sia.py, SIA21 only).

sia21s.kdk / sia21s.dkd use the fixed step; sia21a.* take the power-of-two
block step from the Tstep kernel.  As in the reference driver
(sia.py:1032-1123), a step of size tau applies the slow/fast bridge with
every particle slow: evolve(tau/2), (no slow-fast kick), evolve(tau/2), where
evolve is kdk(h) = kick(h/2) drift(h) kick(h/2) or dkd(h) = drift(h/2)
kick(h) drift(h/2) (sia.py:300-337), and each kick re-evaluates the
accelerations.  The hierarchical sia21h.* split and the other SIA orders are
not part of this backend.
"""
import torch

from .. import _native
from ..lib import extensions
from . import Base

COEFS = ([1.0], [0.5])      # SIA21 coefficients (sia.py:300-303)


def _stream():
    return torch.cuda.current_stream().cuda_stream


def drift(ps, tau):
    _native.check(_native.lib.tg_drift(ps.n, ps.rx.data_ptr(), ps.ry.data_ptr(), ps.rz.data_ptr(),
                                       ps.vx.data_ptr(), ps.vy.data_ptr(), ps.vz.data_ptr(),
                                       float(tau), _stream()), "tg_drift")
    return ps


def kick(ps, tau):
    extensions.acc.calc(ps, ps)
    _native.check(_native.lib.tg_kick(ps.n, ps.vx.data_ptr(), ps.vy.data_ptr(), ps.vz.data_ptr(),
                                      ps.ax.data_ptr(), ps.ay.data_ptr(), ps.az.data_ptr(),
                                      float(tau), _stream()), "tg_kick")
    return ps


def kdk(ps, tau):
    d, k = COEFS
    ps = kick(ps, k[0] * tau)
    ps = drift(ps, d[0] * tau)
    ps = kick(ps, k[0] * tau)
    return ps


def dkd(ps, tau):
    k, d = COEFS
    ps = drift(ps, d[0] * tau)
    ps = kick(ps, k[0] * tau)
    ps = drift(ps, d[0] * tau)
    return ps


class SIA(Base):
    PROVIDED_METHODS = ("sia21s.kdk", "sia21s.dkd", "sia21a.kdk", "sia21a.dkd")

    def __init__(self, eta, time, ps, method, **kwargs):
        super(SIA, self).__init__(eta, time, ps, **kwargs)
        if method not in self.PROVIDED_METHODS:
            raise ValueError("Unexpected method: %r" % method)
        self.method = method
        self.evolve = kdk if method.endswith("kdk") else dkd

    def do_step(self, ps, tau):
        if ps.n <= 2:
            raise NotImplementedError("few-body (n <= 2) steps use the Kepler pair solver, "
                                      "which this backend does not provide")
        if "a." in self.method:
            ps.set_tstep(ps, self.eta)
            tau = self.get_min_block_tstep(ps, tau)
            if bool((ps.tstep.abs() <= abs(tau)).any()):
                raise NotImplementedError("a slow/fast split is needed; only the shared step is provided")
        k, d = COEFS
        ps = self.evolve(ps, d[0] * tau)        # sf_drift (slow part)
        ps = self.evolve(ps, d[0] * tau)        # sf_kick is empty: no fast particles
        self.advance_time(ps, tau)
        return ps
