"""Algorithmic-regularisation leapfrog (tupan/integrator/nreg.py).

The NREG integrator (methods "nreg" and "anreg") advances the system in a
fictitious time: the position step nreg_x moves every particle by dt = h/W
relative to the others (NREG_X kernel: r_i <- sum_j m_j (r_ij + v_ij dt)
/ M, the same pass also returning the accelerations and the potential sum
U), and the velocity step nreg_v kicks by h/U (NREG_V kernel:
v_i <- sum_j m_j (v_ij + a_ij dt) / M, with the kinetic sum for W = K - E0).
The physical time advances by the position steps' dt (nreg.py:22-63);
"nreg" composes two half steps with the extended-phase-space variable S
(nreg.py:79-88).

The state the reference keeps as class attributes of the particle type
(E0, W, U, S, t_curr) lives on the ParticleSystem instance here.  All
reductions use tg_sum (numpy's order) and r = mr / M is an IEEE division
per element (tg_div3), so FP64 trajectories equal the reference's.
"""

from .. import _native
from .._native import psum
from ..lib import extensions
from . import Base


def _div3(x, y, z, mx, my, mz, d):
    _native.check(_native.lib.tg_div3(x.numel(), x.data_ptr(), y.data_ptr(), z.data_ptr(), mx.data_ptr(),
                                      my.data_ptr(), mz.data_ptr(), float(d),
                                      _native.current_stream()), "tg_div3")


def nreg_x(ps, dt):
    """nreg.py:22-34"""
    mtot = ps.total_mass
    extensions.nreg_x.calc(ps, ps, dt)
    _div3(ps.rx, ps.ry, ps.rz, ps.mrx, ps.mry, ps.mrz, mtot)
    ps.U = 0.5 * psum(ps.u)
    ps.t_curr += dt
    return ps


def nreg_v(ps, dt):
    """nreg.py:45-63"""
    mtot = ps.total_mass
    extensions.nreg_v.calc(ps, ps, dt)
    _div3(ps.vx, ps.vy, ps.vz, ps.mvx, ps.mvy, ps.mvz, mtot)
    K = 0.25 * psum(ps.mk) / mtot
    ps.W = K - ps.E0
    return ps


def anreg_step(ps, h):
    """nreg.py:67-76"""
    ps = nreg_x(ps, 0.5 * (h / ps.W))
    ps = nreg_v(ps, (h / ps.U))
    ps = nreg_x(ps, 0.5 * (h / ps.W))
    return ps


def nreg_step(ps, h):
    """nreg.py:79-88"""
    ps = anreg_step(ps, 0.5 * (h * ps.S))
    ps.S = 1 / (2 / ps.W - 1 / ps.S)
    ps = anreg_step(ps, 0.5 * (h * ps.S))
    return ps


class NREG(Base):
    PROVIDED_METHODS = ("nreg", "anreg")

    def __init__(self, eta, time, ps, method, **kwargs):
        super(NREG, self).__init__(eta, time, ps, **kwargs)
        self.method = method

    def initialize(self, t_end):
        """nreg.py:105-122"""
        ps = self.ps
        ps.t_curr = self.t_curr
        ps.E0 = ps.kinetic_energy + ps.potential_energy
        ps.W = -ps.potential_energy
        ps.U = -ps.potential_energy
        ps.S = -ps.potential_energy
        super(NREG, self).initialize(t_end)

    def do_step(self, ps, tau):
        """nreg.py:138-165: the step is measured in physical time."""
        t0 = ps.t_curr
        if "anreg" in self.method:
            ps = anreg_step(ps, tau / 2)
        else:
            ps = nreg_step(ps, tau)
        dt = ps.t_curr - t0
        ps.tstep.fill_(dt)
        ps.time += tau
        ps.nstep += 1
        self.t_curr = ps.t_curr
        self.record(ps, tau)
        return ps
