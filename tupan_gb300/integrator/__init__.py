"""Integrators driving the GPU kernels, mirroring tupan/integrator.

Base and Integrator follow tupan/integrator/__init__.py:13-157 (base time
step, power-of-two block step commensurate with the current time,
evolve_step); Hermite (hermite2..8, ahermite2..8), SIA21 (sia21s/sia21a,
kdk/dkd), NREG (nreg, anreg) and Sakura (sakura, asakura) are in the
submodules.  All particle
state stays on the GPU; the element-wise updates are the fused FP64 kernels
of libtupan_gb300 (tg_drift, tg_kick, tg_hermite_predict, ...), evaluated in
the reference's operation order.
"""
import math
import sys

import numpy as np
import torch

from ..lib import extensions


class Base(object):
    def __init__(self, eta, time, ps, **kwargs):
        self.eta = eta
        self.ps = ps
        self.t_curr = float(time)
        ps.t_curr = self.t_curr
        self.is_initialized = False
        pn_order = kwargs.pop("pn_order", 0)
        clight = kwargs.pop("clight", None)
        if pn_order > 0:
            if clight is None:
                raise TypeError("'clight' is not defined. Please set the speed of light "
                                "argument 'clight' when using 'pn_order' > 0.")
            extensions.clight.pn_order = pn_order
            extensions.clight.clight = clight
        self.reporter = kwargs.pop("reporter", None)
        self.viewer = kwargs.pop("viewer", None)
        self.dumpper = kwargs.pop("dumpper", None)
        self.dump_freq = kwargs.pop("dump_freq", 1)
        self.gl_freq = kwargs.pop("gl_freq", 1)
        self.wl = None
        if kwargs:
            raise TypeError("%s.__init__ received unexpected keyword arguments: %s."
                            % (type(self).__name__, ", ".join(kwargs.keys())))

    def initialize(self, t_end):
        """The report, worldline dump and viewer event of the initial state
        (hermite.py:318-327 and the same lines of sia.py, sakura.py, nreg.py)."""
        if self.reporter:
            self.reporter.diagnostic_report(self.ps)
        if self.dumpper:
            self.dumpper.dump_worldline(self.ps)
        if self.viewer:
            self.viewer.show_event(self.ps)
        self.is_initialized = True

    def finalize(self, t_end):
        pass

    def get_base_tstep(self, t_end):
        """integrator/__init__.py:49-57"""
        dt = min(abs(t_end) - abs(self.t_curr), abs(self.eta))
        dt = max(dt, abs(t_end) * (2 * sys.float_info.epsilon))
        return math.copysign(dt, self.eta)

    def get_min_block_tstep(self, ps, tau):
        """Power-of-two step not above the smallest particle step and
        commensurate with the current time (integrator/__init__.py:59-78)."""
        min_ts = ps.min_tstep()
        power = int(np.log2(min_ts) - 1)
        min_bts = 2.0 ** power
        t_next = self.t_curr + min_bts
        while t_next % min_bts != 0:
            min_bts /= 2
        min_bts = math.copysign(min_bts, tau)
        if abs(min_bts) > abs(tau):
            min_bts = tau
        return min_bts

    def advance_time(self, ps, tau):
        self.t_curr += tau
        ps.t_curr = self.t_curr
        ps.tstep.fill_(tau)
        ps.time += tau
        ps.nstep += 1
        self.record(ps, tau)

    def record(self, ps, tau):
        """Particles whose time is a multiple of dump_freq * tau join the
        step's worldline, those at a multiple of gl_freq * tau go to the
        viewer (hermite.py:402-409).  fmod is exact, and it is zero exactly
        where the reference's numpy remainder is.  Selecting reads one flag
        back to the host, and only when a dumpper or a viewer is set."""
        if self.dumpper and self.wl is not None:
            slc = torch.fmod(ps.time, self.dump_freq * tau) == 0
            if bool(slc.any()):
                self.wl.append(ps[slc])
        if self.viewer:
            slc = torch.fmod(ps.time, self.gl_freq * tau) == 0
            if bool(slc.any()):
                self.viewer.show_event(ps[slc])

    def evolve_step(self, t_end):
        if not self.is_initialized:
            self.initialize(t_end)
        ps = self.ps
        self.wl = ps[0:0]          # this step's worldline (integrator/__init__.py:89)
        tau = self.get_base_tstep(t_end)
        self.ps = self.do_step(ps, tau)
        if self.reporter:
            self.reporter.diagnostic_report(self.ps)
        if self.dumpper:
            self.dumpper.dump_worldline(self.wl)


from . import hermite, nreg, sakura, sia  # noqa: E402


class Integrator(object):
    """Method dispatcher (integrator/__init__.py:108-157)."""
    PROVIDED_METHODS = (sia.SIA.PROVIDED_METHODS + nreg.NREG.PROVIDED_METHODS
                        + sakura.Sakura.PROVIDED_METHODS + hermite.Hermite.PROVIDED_METHODS)

    def __init__(self, eta, time, ps, **kwargs):
        method = kwargs.pop("method", None)
        if method in sia.SIA.PROVIDED_METHODS:
            self.integrator = sia.SIA(eta, time, ps, method, **kwargs)
        elif method in nreg.NREG.PROVIDED_METHODS:
            self.integrator = nreg.NREG(eta, time, ps, method, **kwargs)
        elif method in sakura.Sakura.PROVIDED_METHODS:
            self.integrator = sakura.Sakura(eta, time, ps, method, **kwargs)
        elif method in hermite.Hermite.PROVIDED_METHODS:
            self.integrator = hermite.Hermite(eta, time, ps, method, **kwargs)
        else:
            raise ValueError("Unexpected integration method: %r. Provided methods: %s"
                             % (method, list(self.PROVIDED_METHODS)))

    def initialize(self, t_end):
        self.integrator.initialize(t_end)

    def finalize(self, t_end):
        self.integrator.finalize(t_end)

    def evolve_step(self, t_end):
        self.integrator.evolve_step(t_end)

    @property
    def time(self):
        return self.integrator.t_curr

    @property
    def particle_system(self):
        return self.integrator.ps
