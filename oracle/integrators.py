"""CPU restatement of the reference integrators used on the hot path.

TEST INFRASTRUCTURE ONLY (the checker for tupan_gb300.integrator).  numpy
arrays, the kernels of oracle/tupan_oracle.c, and the reference's time-step
logic and update expressions in numpy's evaluation order:

  Base.get_base_tstep / get_min_block_tstep   tupan/integrator/__init__.py:49-78
  Hermite H2/H4/H6/H8 epredict/ecorrect/epec  tupan/integrator/hermite.py:20-283, 387-410
  SIA21 kdk/dkd with the shared-step bridge   tupan/integrator/sia.py:64-86, 193-230, 300-352, 1032-1123
  sakura_step / asakura step                  tupan/integrator/sakura.py:22-50, 100-159

With the FP64 oracle kernels (bit-identical to the reference C backend) the
trajectories are bit-identical to the reference integrators; pinned in
tests/test_integrators_oracle.py.
"""
import math
import sys

import numpy as np

from .oracle import Oracle

FIELDS = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")


class PS(dict):
    """A particle set: dict of float64 arrays with the reference names."""

    @property
    def n(self):
        return len(self["mass"])

    def copy(self):
        return PS({k: v.copy() for k, v in self.items()})


def make_ps(d):
    ps = PS({k: np.array(d[k], dtype=np.float64) for k in FIELDS})
    ps["time"] = np.zeros(ps.n)
    ps["tstep"] = np.zeros(ps.n)
    ps["nstep"] = np.zeros(ps.n, dtype=np.int64)
    return ps


class Kernels(object):
    def __init__(self, nthreads=4):
        self.o = Oracle()
        self.nthreads = nthreads

    def acc(self, ps):
        ps["ax"], ps["ay"], ps["az"] = self.o.calc("acc", ps, ps, nthreads=self.nthreads)

    def acc_jerk(self, ps):
        r = self.o.calc("acc_jerk", ps, ps, nthreads=self.nthreads)
        for k, v in zip(("ax", "ay", "az", "jx", "jy", "jz"), r):
            ps[k] = v

    def snap_crackle(self, ps):
        r = self.o.calc("snap_crackle", ps, ps, nthreads=self.nthreads)
        for k, v in zip(("sx", "sy", "sz", "cx", "cy", "cz"), r):
            ps[k] = v

    def tstep(self, ps, eta):
        ps["tstep"], ps["tstepij"] = self.o.calc("tstep", ps, ps, eta, nthreads=self.nthreads)

    def sakura(self, ps, dt, flag):
        r = self.o.calc("sakura", ps, ps, dt, flag, nthreads=self.nthreads)
        for k, v in zip(("drx", "dry", "drz", "dvx", "dvy", "dvz"), r):
            ps[k] = v


class Base(object):
    def __init__(self, eta, time, ps, kernels):
        self.eta = eta
        self.t_curr = float(time)
        self.ps = ps
        self.k = kernels

    def get_base_tstep(self, t_end):
        dt = min(abs(t_end) - abs(self.t_curr), abs(self.eta))
        dt = max(dt, abs(t_end) * (2 * sys.float_info.epsilon))
        return math.copysign(dt, self.eta)

    def get_min_block_tstep(self, ps, tau):
        min_ts = abs(ps["tstep"]).min()
        power = int(np.log2(min_ts) - 1)
        min_bts = 2.0 ** power
        t_next = self.t_curr + min_bts
        while t_next % min_bts != 0:
            min_bts /= 2
        min_bts = math.copysign(min_bts, tau)
        if abs(min_bts) > abs(tau):
            min_bts = tau
        return min_bts

    def finish(self, ps, tau):
        self.t_curr += tau
        ps["tstep"][...] = tau
        ps["time"] += tau
        ps["nstep"] += 1

    def evolve_step(self, t_end):
        tau = self.get_base_tstep(t_end)
        self.ps = self.do_step(self.ps, tau)

    def run(self, t_end):
        while abs(self.t_curr) < abs(t_end):
            self.evolve_step(t_end)
        return self.ps


# --- Hermite -------------------------------------------------------------
def _derivs(ps, order):
    keys = ("a", "j", "s", "c")[:order // 2]
    return [[ps[k + c] for c in "xyz"] for k in keys]


def hermite_predict(ps1, ps0, tau, order):
    """rx += ((((d_m tau/(m+1) + ...) + a) tau/2 + v) tau; same for v."""
    m = order // 2
    d = _derivs(ps0, order)
    for c, axis in enumerate("xyz"):
        v0 = ps0["v" + axis]
        acc = d[m - 1][c]
        for q in range(m - 2, -1, -1):
            acc = acc * tau / (q + 3) + d[q][c]
        ps1["r" + axis] += (acc * tau / 2 + v0) * tau
        bcc = d[m - 1][c]
        for q in range(m - 2, -1, -1):
            bcc = bcc * tau / (q + 2) + d[q][c]
        ps1["v" + axis] += bcc * tau


def hermite_correct(ps1, ps0, tau, order):
    for axis in "xyz":
        a0, a1 = ps0["a" + axis], ps1["a" + axis]
        r0, v0 = ps0["r" + axis], ps0["v" + axis]
        if order == 2:
            v1 = (a0 + a1) * tau / 2 + v0
            r1 = (v0 + v1) * tau / 2 + r0
        elif order == 4:
            j0, j1 = ps0["j" + axis], ps1["j" + axis]
            v1 = ((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + v0
            r1 = ((a0 - a1) * tau / 6 + (v0 + v1)) * tau / 2 + r0
        elif order == 6:
            j0, j1 = ps0["j" + axis], ps1["j" + axis]
            s0, s1 = ps0["s" + axis], ps1["s" + axis]
            v1 = (((s0 + s1) * tau / 12 + (j0 - j1)) * tau / 5 + (a0 + a1)) * tau / 2 + v0
            r1 = (((j0 + j1) * tau / 12 + (a0 - a1)) * tau / 5 + (v0 + v1)) * tau / 2 + r0
        else:
            j0, j1 = ps0["j" + axis], ps1["j" + axis]
            s0, s1 = ps0["s" + axis], ps1["s" + axis]
            c0, c1 = ps0["c" + axis], ps1["c" + axis]
            v1 = ((((c0 - c1) * tau / 20 + (s0 + s1)) * tau / 3 + 3 * (j0 - j1)) * tau / 14
                  + (a0 + a1)) * tau / 2 + v0
            r1 = ((((s0 - s1) * tau / 20 + (j0 + j1)) * tau / 3 + 3 * (a0 - a1)) * tau / 14
                  + (v0 + v1)) * tau / 2 + r0
        ps1["v" + axis][...] = v1
        ps1["r" + axis][...] = r1


class Hermite(Base):
    def __init__(self, eta, time, ps, method, kernels):
        super(Hermite, self).__init__(eta, time, ps, kernels)
        self.method = method
        self.order = int(method[-1])

    def derivatives(self, ps):
        if self.order == 2:
            self.k.acc(ps)
        else:
            self.k.acc_jerk(ps)
            if self.order >= 6:
                self.k.snap_crackle(ps)

    def do_step(self, ps, tau):
        if "ahermite" in self.method:
            self.k.tstep(ps, self.eta)
            tau = self.get_min_block_tstep(ps, tau)
        ps0 = ps.copy()
        self.derivatives(ps0)
        ps1 = ps
        hermite_predict(ps1, ps0, tau, self.order)
        for _ in range(2):
            self.derivatives(ps1)
            hermite_correct(ps1, ps0, tau, self.order)
        self.finish(ps1, tau)
        return ps1


# --- SIA21 ---------------------------------------------------------------
class SIA21(Base):
    def __init__(self, eta, time, ps, method, kernels):
        super(SIA21, self).__init__(eta, time, ps, kernels)
        self.method = method

    def drift(self, ps, tau):
        for a in "xyz":
            ps["r" + a] += ps["v" + a] * tau

    def kick(self, ps, tau):
        self.k.acc(ps)
        for a in "xyz":
            ps["v" + a] += ps["a" + a] * tau

    def evolve(self, ps, tau):
        if self.method.endswith("kdk"):
            self.kick(ps, 0.5 * tau)
            self.drift(ps, 1.0 * tau)
            self.kick(ps, 0.5 * tau)
        else:
            self.drift(ps, 0.5 * tau)
            self.kick(ps, 1.0 * tau)
            self.drift(ps, 0.5 * tau)

    def do_step(self, ps, tau):
        if "a." in self.method:
            self.k.tstep(ps, self.eta)
            tau = self.get_min_block_tstep(ps, tau)
        self.evolve(ps, 0.5 * tau)
        self.evolve(ps, 0.5 * tau)
        self.finish(ps, tau)
        return ps


# --- Sakura --------------------------------------------------------------
class Sakura(Base):
    def __init__(self, eta, time, ps, method, kernels):
        super(Sakura, self).__init__(eta, time, ps, kernels)
        self.method = method

    def step(self, ps, tau):
        for a in "xyz":
            ps["r" + a] += ps["v" + a] * tau / 2
        for flag in (-1, 1):
            self.k.sakura(ps, tau / 2, flag)
            for a in "xyz":
                ps["r" + a] += ps["dr" + a]
                ps["v" + a] += ps["dv" + a]
        for a in "xyz":
            ps["r" + a] += ps["v" + a] * tau / 2

    def do_step(self, ps, tau):
        if "asakura" in self.method:
            self.k.tstep(ps, self.eta)
            iw2_a = (self.eta / ps["tstep"]) ** 2
            iw2_b = (self.eta / ps["tstepij"]) ** 2
            w2 = (iw2_a - iw2_b).max()
            ps["tstep"][...] = self.eta / (1 + w2) ** 0.5
            tau = self.get_min_block_tstep(ps, tau)
        self.step(ps, tau)
        self.finish(ps, tau)
        return ps


def integrator(method, eta, ps, kernels=None, time=0.0):
    kernels = kernels or Kernels()
    if "hermite" in method:
        return Hermite(eta, time, ps, method, kernels)
    if method.startswith("sia21"):
        return SIA21(eta, time, ps, method, kernels)
    if "sakura" in method:
        return Sakura(eta, time, ps, method, kernels)
    raise ValueError(method)
