"""Sakura integrator (tupan/integrator/sakura.py).

sakura_step (sakura.py:22-50): half drift, pairwise Kepler drifts with
flag -1 then +1 over tau/2 each (the Sakura kernel returns the increments
dr, dv, added by tg_add_increments), half drift.  asakura takes the step
from the Tstep kernel's sum and max criteria (sakura.py:100-117).
"""

from .. import _native
from ..lib import extensions
from . import Base
from .sia import drift


def _stream():
    return _native.current_stream()


def apply_increments(ps):
    _native.check(_native.lib.tg_add_increments(
        ps.n, ps.rx.data_ptr(), ps.ry.data_ptr(), ps.rz.data_ptr(),
        ps.vx.data_ptr(), ps.vy.data_ptr(), ps.vz.data_ptr(),
        ps.drx.data_ptr(), ps.dry.data_ptr(), ps.drz.data_ptr(),
        ps.dvx.data_ptr(), ps.dvy.data_ptr(), ps.dvz.data_ptr(), _stream()), "tg_add_increments")


def sakura_step(ps, tau):
    drift(ps, tau / 2)
    extensions.sakura.calc(ps, ps, tau / 2, -1)
    apply_increments(ps)
    extensions.sakura.calc(ps, ps, tau / 2, 1)
    apply_increments(ps)
    drift(ps, tau / 2)
    return ps


class Sakura(Base):
    PROVIDED_METHODS = ("sakura", "asakura")

    def __init__(self, eta, time, ps, method, **kwargs):
        super(Sakura, self).__init__(eta, time, ps, **kwargs)
        self.method = method

    def get_sakura_tstep(self, ps, eta, tau):
        ps.set_tstep(ps, eta)
        iw2_a = (eta / ps.tstep) ** 2
        iw2_b = (eta / ps.tstepij) ** 2
        w2_sakura = float((iw2_a - iw2_b).max())
        dt_sakura = eta / (1 + w2_sakura) ** 0.5
        ps.tstep.fill_(dt_sakura)
        return self.get_min_block_tstep(ps, tau)

    def do_step(self, ps, tau):
        if "asakura" in self.method:
            tau = self.get_sakura_tstep(ps, self.eta, tau)
        ps = sakura_step(ps, tau)
        self.advance_time(ps, tau)
        return ps
