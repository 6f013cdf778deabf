"""Hermite predictor-corrector integrators (tupan/integrator/hermite.py).

hermite2/4/6/8 use a shared step; ahermite2/4/6/8 take the power-of-two
block step from the pairwise Tstep kernel (hermite.py:343-349).  One step is
epec(2): predict from the start state's derivatives, then twice re-evaluate
the derivatives at the new state and correct (hermite.py:56-67, 390-410).
The predictor and corrector are the fused FP64 kernels tg_hermite_predict /
tg_hermite_correct; the derivatives come from AccJerk (and SnapCrackle for
orders 6 and 8, Acc for order 2).
"""

from .. import _native
from ..lib import extensions
from . import Base

DERIV = {2: ("ax", "ay", "az"), 4: ("ax", "ay", "az", "jx", "jy", "jz"),
         6: ("ax", "ay", "az", "jx", "jy", "jz", "sx", "sy", "sz"),
         8: ("ax", "ay", "az", "jx", "jy", "jz", "sx", "sy", "sz", "cx", "cy", "cz")}
RV = ("rx", "ry", "rz", "vx", "vy", "vz")


def set_derivatives(ps, order):
    if order == 2:
        extensions.acc.calc(ps, ps)
    else:
        extensions.acc_jerk.calc(ps, ps)
        if order >= 6:
            extensions.snap_crackle.calc(ps, ps)


def _stream():
    return _native.current_stream()


def predict(ps1, ps0, tau, order):
    rv = _native.ptr_array([getattr(ps1, k) for k in RV])
    der = _native.ptr_array([getattr(ps0, k) for k in DERIV[order]])
    _native.check(_native.lib.tg_hermite_predict(order, ps1.n, float(tau), rv, der, _stream()),
                  "tg_hermite_predict")


def correct(ps1, ps0, tau, order):
    rv0 = _native.ptr_array([getattr(ps0, k) for k in RV])
    d0 = _native.ptr_array([getattr(ps0, k) for k in DERIV[order]])
    d1 = _native.ptr_array([getattr(ps1, k) for k in DERIV[order]])
    rv1 = _native.ptr_array([getattr(ps1, k) for k in RV])
    _native.check(_native.lib.tg_hermite_correct(order, ps1.n, float(tau), rv0, d0, d1, rv1, _stream()),
                  "tg_hermite_correct")


def epec(n, ps, tau, order):
    ps0 = ps.copy()
    set_derivatives(ps0, order)
    ps1 = ps
    predict(ps1, ps0, tau, order)
    for _ in range(n):
        set_derivatives(ps1, order)
        correct(ps1, ps0, tau, order)
    return ps1


class Hermite(Base):
    PROVIDED_METHODS = ("hermite2", "ahermite2", "hermite4", "ahermite4",
                        "hermite6", "ahermite6", "hermite8", "ahermite8")

    def __init__(self, eta, time, ps, method, **kwargs):
        super(Hermite, self).__init__(eta, time, ps, **kwargs)
        self.method = method
        self.order = int(method[-1])

    def get_hermite_tstep(self, ps, eta, tau):
        ps.set_tstep(ps, eta)
        return self.get_min_block_tstep(ps, tau)

    def do_step(self, ps, tau):
        if "ahermite" in self.method:
            tau = self.get_hermite_tstep(ps, self.eta, tau)
        ps = epec(2, ps, tau, self.order)
        self.advance_time(ps, tau)
        return ps
