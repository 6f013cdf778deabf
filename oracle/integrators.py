"""CPU restatement of the reference integrators used on the hot path.

TEST INFRASTRUCTURE ONLY (the checker for tupan_gb300.integrator).  numpy
arrays, the kernels of oracle/tupan_oracle.c, and the reference's time-step
logic and update expressions in numpy's evaluation order:

  Base.get_base_tstep / get_min_block_tstep   tupan/integrator/__init__.py:49-78
  Hermite H2/H4/H6/H8 epredict/ecorrect/epec  tupan/integrator/hermite.py:20-283, 387-410
  SIA21..SIA69 kdk/dkd, s./a./h. modes with   tupan/integrator/sia.py:24-86, 186-230, 300-961, 1032-1123
  the slow/fast split and FewBody             tupan/integrator/fewbody.py:13-57
  sakura_step / asakura step                  tupan/integrator/sakura.py:22-50, 100-159
  NREG nreg_x/nreg_v/anreg_step/nreg_step     tupan/integrator/nreg.py:22-165
  worldline rows (dump_freq)                  tupan/integrator/__init__.py:86-97, hermite.py:318-327, 402-405

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
    ps["id"] = np.arange(ps.n, dtype=np.int64)
    return ps


class Kernels(object):
    def __init__(self, nthreads=4):
        self.o = Oracle()
        self.nthreads = nthreads

    def acc(self, ps, jps=None):
        ps["ax"], ps["ay"], ps["az"] = self.o.calc("acc", ps, ps if jps is None else jps,
                                                   nthreads=self.nthreads)

    def kepler(self, ps, dt):
        r = self.o.kepler(ps, dt)
        for k, v in zip(("rx", "ry", "rz", "vx", "vy", "vz"), r):
            ps[k] = v

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

    def phi(self, ps):
        ps["phi"], = self.o.calc("phi", ps, ps, nthreads=self.nthreads)

    def nreg_x(self, ps, dt):
        r = self.o.calc("nreg_x", ps, ps, dt, nthreads=self.nthreads)
        for k, v in zip(("mrx", "mry", "mrz", "ax", "ay", "az", "u"), r):
            ps[k] = v

    def nreg_v(self, ps, dt):
        r = self.o.calc("nreg_v", ps, ps, dt, nthreads=self.nthreads)
        for k, v in zip(("mvx", "mvy", "mvz", "mk"), r):
            ps[k] = v

    def sakura(self, ps, dt, flag):
        r = self.o.calc("sakura", ps, ps, dt, flag, nthreads=self.nthreads)
        for k, v in zip(("drx", "dry", "drz", "dvx", "dvy", "dvz"), r):
            ps[k] = v


class Base(object):
    def __init__(self, eta, time, ps, kernels, dump_freq=None):
        self.eta = eta
        self.t_curr = float(time)
        self.ps = ps
        self.k = kernels
        # with dump_freq set, `worldline` collects the rows the reference's
        # dumpper receives: the whole set once before the first step, then
        # the particles whose time is a multiple of dump_freq * tau
        self.dump_freq = dump_freq
        self.worldline = []
        self.started = False

    def record(self, ps, tau):
        if self.dump_freq is not None:
            slc = ps["time"] % (self.dump_freq * tau) == 0
            if any(slc):
                self.worldline.append(ps_select(ps, slc))

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
        self.record(ps, tau)

    def evolve_step(self, t_end):
        if not self.started:
            self.started = True
            if self.dump_freq is not None:
                self.worldline.append(self.ps.copy())
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


# --- SIA ------------------------------------------------------------------
SIA_COEFS = {
    "sia21": ([1.0], [0.5]),
    "sia22": ([0.5], [0.1931833275037836, 0.6136333449924328]),
    "sia43": ([1.3512071919596575, -1.7024143839193150],
              [0.6756035959798288, -0.17560359597982877]),
    "sia44": ([0.7123418310626056, -0.21234183106260562],
              [0.1786178958448091, -0.06626458266981843, 0.7752933736500186]),
    "sia45": ([-0.0844296195070715, 0.354900057157426, 0.459059124699291],
              [0.2750081212332419, -0.1347950099106792, 0.35978688867743724]),
    "sia46": ([0.209515106613362, -0.143851773179818, 0.434336666566456],
              [0.0792036964311957, 0.353172906049774, -0.0420650803577195, 0.21937695575349958]),
    "sia67": ([0.7845136104775573, 0.23557321335935813, -1.177679984178871, 1.3151863206839112],
              [0.39225680523877865, 0.5100434119184577, -0.47105338540975644, 0.06875316825252015]),
    "sia69": ([0.39103020330868477, 0.334037289611136, -0.7062272811875614, 0.08187754964805945,
               0.7985644772393624],
              [0.19551510165434238, 0.3625337464599104, -0.1860949957882127, -0.31217486576975095,
               0.44022101344371095]),
}


def sia_sequence(first, second):
    """The symmetric operator sequence of one SIA propagator (sia.py:300-961):
    operator 0 with the coefficients `second` opens and closes it and
    alternates with operator 1 (coefficients `first`)."""
    half = []
    for i in range(len(first)):
        half += [(0, second[i]), (1, first[i])]
    if len(second) == len(first) + 1:
        half.append((0, second[-1]))
    return half + half[:-1][::-1]


def ps_select(ps, mask):
    return PS({k: v[mask] for k, v in ps.items()})


def ps_join(slow, fast):
    if not fast.n:
        return slow
    if not slow.n:
        return fast
    out = PS()
    for k in set(slow) | set(fast):
        a = slow.get(k, np.zeros(slow.n, dtype=fast[k].dtype if k in fast else np.float64))
        b = fast.get(k, np.zeros(fast.n, dtype=a.dtype))
        out[k] = np.concatenate((a, b))
    return out


class SIA(Base):
    def __init__(self, eta, time, ps, method, kernels):
        super(SIA, self).__init__(eta, time, ps, kernels)
        self.method = method
        self.ops = sia_sequence(*SIA_COEFS[method[:5]])
        mode = method[5]
        self.update_tstep = mode in "ah"
        self.shared_tstep = mode in "sa"
        self.kdk = method.endswith("kdk")

    def drift(self, ps, tau):
        for a in "xyz":
            ps["r" + a] += ps["v" + a] * tau

    def kick_n(self, ps, tau):
        for a in "xyz":
            ps["v" + a] += ps["a" + a] * tau

    def kick(self, ps, tau):
        self.k.acc(ps)
        self.kick_n(ps, tau)

    def fewbody(self, ps, tau):
        if ps.n == 1:
            self.drift(ps, tau)
        elif ps.n == 2:
            self.k.kepler(ps, tau)
        return ps

    def evolve(self, ps, tau):
        if ps.n <= 2:
            return self.fewbody(ps, tau)
        for op, c in self.ops:
            if (op == 0) == self.kdk:
                self.kick(ps, c * tau)
            else:
                self.drift(ps, c * tau)
        return ps

    def sf_kick(self, slow, fast, tau):
        if slow.n and fast.n:
            self.k.acc(slow, fast)
            self.k.acc(fast, slow)
            self.kick_n(slow, tau)
            self.kick_n(fast, tau)

    def bridge(self, slow, fast, tau):
        for op, c in self.ops:
            if op == 0:
                slow = self.evolve(slow, c * tau)
                fast = self.recurse(fast, c * tau)
            else:
                self.sf_kick(slow, fast, c * tau)
        return slow, fast

    def recurse(self, ps, tau):
        if not ps.n:
            return ps
        flag = -1
        if self.update_tstep:
            flag = 1
            self.k.tstep(ps, self.eta)
            if self.shared_tstep:
                tau = self.get_min_block_tstep(ps, tau)
        if ps.n <= 2:
            slow, fast = ps, PS({k: v[:0] for k, v in ps.items()})
        else:
            cond = np.abs(ps["tstep"]) > flag * abs(tau)
            slow, fast = ps_select(ps, cond), ps_select(ps, ~cond)
        slow, fast = self.bridge(slow, fast, tau)
        if fast.n == 0:
            self.t_curr += tau
        if slow.n:
            slow["tstep"][...] = tau
            slow["time"] += tau
            slow["nstep"] += 1
            self.record(slow, tau)
        return ps_join(slow, fast)

    def do_step(self, ps, tau):
        return self.recurse(ps, tau)


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


# --- NREG ----------------------------------------------------------------
class NREG(Base):
    """Algorithmic regularisation (nreg.py:22-165): positions move by h/W and
    velocities by h/U in a fictitious time; the physical time is the sum of
    the position steps.  E0, W, U, S are the reference's class attributes of
    the particle type."""

    def __init__(self, eta, time, ps, method, kernels):
        super(NREG, self).__init__(eta, time, ps, kernels)
        self.method = method
        self.initialised = False

    def energies(self, ps):
        ke = float((0.5 * ps["mass"] * (ps["vx"] ** 2 + ps["vy"] ** 2 + ps["vz"] ** 2)).sum())
        self.k.phi(ps)
        pe = 0.5 * float((ps["mass"] * ps["phi"]).sum())
        return ke, pe

    def initialise(self, ps):
        ke, pe = self.energies(ps)
        self.E0 = ke + pe
        self.W = self.U = self.S = -pe
        self.initialised = True

    def nreg_x(self, ps, dt):
        mtot = float(ps["mass"].sum())
        self.k.nreg_x(ps, dt)
        for a in "xyz":
            ps["r" + a][...] = ps["mr" + a] / mtot
        self.U = 0.5 * ps["u"].sum()
        self.t_curr += dt

    def nreg_v(self, ps, dt):
        mtot = float(ps["mass"].sum())
        self.k.nreg_v(ps, dt)
        for a in "xyz":
            ps["v" + a][...] = ps["mv" + a] / mtot
        K = 0.25 * ps["mk"].sum() / mtot
        self.W = K - self.E0

    def anreg_step(self, ps, h):
        self.nreg_x(ps, 0.5 * (h / self.W))
        self.nreg_v(ps, (h / self.U))
        self.nreg_x(ps, 0.5 * (h / self.W))

    def nreg_step(self, ps, h):
        self.anreg_step(ps, 0.5 * (h * self.S))
        self.S = 1 / (2 / self.W - 1 / self.S)
        self.anreg_step(ps, 0.5 * (h * self.S))

    def do_step(self, ps, tau):
        if not self.initialised:
            self.initialise(ps)
        t0 = self.t_curr
        if "anreg" in self.method:
            self.anreg_step(ps, tau / 2)
        else:
            self.nreg_step(ps, tau)
        ps["tstep"][...] = self.t_curr - t0
        ps["time"] += tau
        ps["nstep"] += 1
        self.record(ps, tau)
        return ps


def integrator(method, eta, ps, kernels=None, time=0.0, dump_freq=None):
    kernels = kernels or Kernels()
    if method in ("nreg", "anreg"):
        it = NREG(eta, time, ps, method, kernels)
    elif "hermite" in method:
        it = Hermite(eta, time, ps, method, kernels)
    elif method.startswith("sia"):
        it = SIA(eta, time, ps, method, kernels)
    elif "sakura" in method:
        it = Sakura(eta, time, ps, method, kernels)
    else:
        raise ValueError(method)
    it.dump_freq = dump_freq
    return it
