"""Symplectic integrators with the slow/fast split (tupan/integrator/sia.py).

Methods "sia<NM><mode>.<form>": the eight coefficient sets SIA21, SIA22,
SIA43, SIA44, SIA45, SIA46, SIA67, SIA69 (sia.py:300-961; Yoshida 1990 and
Omelyan, Mryglod & Folk 2003), the forms kdk and dkd, and the modes

  s.  shared fixed step (all particles slow);
  a.  shared power-of-two block step from the Tstep kernel;
  h.  hierarchical: at every level the particles whose pairwise time step
      is not above the level's step form the "fast" subsystem, which is
      advanced recursively with the same scheme at the bridge's sub-steps,
      while the slow subsystem takes one step and slow<->fast cross kicks
      couple them (sia.py:24-57, 186-230, 1072-1123).

Every scheme is a symmetric composition, written here as a palindrome of
coefficients: kdk alternates kick/drift starting with a kick whose
coefficients are the scheme's second list, dkd alternates drift/kick
starting with a drift whose coefficients are the second list, and the
bridge alternates slow/fast drift (second list) with cross kicks (first
list).  Subsystems of at most two particles are advanced by FewBody
(fewbody.py:13-57): a free drift for one particle, the Kepler pair solver
for two.

All particle state stays on the GPU: subsystems are boolean-mask selections
of the particle set (order preserved) and joining concatenates slow then
fast, as the reference does, so the particle order after an h. step is the
reference's.  Post-Newtonian SIA (sia.py:88-160) is not provided: the
reference's PN bridge calls particle methods that do not exist.

The h. modes run the recursion natively (tg_sia_h_step): on a small
cluster a step is about a thousand levels of a few particles each, and a
level driven from Python costs more than its arithmetic.  The native step
makes the same kernel calls in the same order with the same arguments, so
its FP64 trajectories equal this module's recursion bit for bit;
`SIA.native_h = False` selects the Python recursion below.
"""
import ctypes
import warnings

import torch

from .. import _native
from ..lib import extensions
from . import Base

# (first list, second list) per scheme, sia.py:300-961
COEFS = {
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


def palindrome(first, second):
    """Operator sequence [(0 | 1, coef)] of a symmetric composition: operator
    0 takes the coefficients `second` (and opens and closes the sequence),
    operator 1 takes `first`; the middle element is the last coefficient of
    the longer list."""
    seq = []
    for i in range(len(first)):
        seq.append((0, second[i]))
        seq.append((1, first[i]))
    if len(second) == len(first) + 1:
        seq.append((0, second[-1]))
    return seq + seq[:-1][::-1]


def _stream():
    return _native.current_stream()


def drift(ps, tau):
    """r += v * tau (drift_n, sia.py:61-70)"""
    if ps.n:
        _native.check(_native.lib.tg_drift(ps.n, ps.rx.data_ptr(), ps.ry.data_ptr(), ps.rz.data_ptr(),
                                           ps.vx.data_ptr(), ps.vy.data_ptr(), ps.vz.data_ptr(),
                                           float(tau), _stream()), "tg_drift")
    return ps


def kick_n(ps, tau):
    """v += a * tau (kick_n, sia.py:73-82)"""
    if ps.n:
        _native.check(_native.lib.tg_kick(ps.n, ps.vx.data_ptr(), ps.vy.data_ptr(), ps.vz.data_ptr(),
                                          ps.ax.data_ptr(), ps.ay.data_ptr(), ps.az.data_ptr(),
                                          float(tau), _stream()), "tg_kick")
    return ps


def kick(ps, tau):
    """sia.py:175-184"""
    extensions.acc.calc(ps, ps)
    return kick_n(ps, tau)


class FewBody(object):
    """fewbody.py:13-57"""

    @staticmethod
    def evolve(ps, tau):
        if ps.n == 0:
            return ps
        if ps.n == 1:
            return drift(ps, tau)
        extensions.kepler.calc(ps, ps, tau)
        return ps


def split(ps, condition):
    """sia.py:24-43: (slow, fast); a set of at most two particles stays whole.
    Each part keeps the particles' order; the partition takes one host
    synchronisation (the count), the stable sort and gathers none."""
    if ps.n <= 2:
        return ps, type(ps)(0)
    order = torch.argsort((~condition).to(torch.int8), stable=True)
    k = int(condition.sum())
    return ps.take(order[:k]), ps.take(order[k:])


def join(slow, fast):
    """sia.py:46-57: slow followed by fast."""
    if not fast.n:
        return slow
    if not slow.n:
        return fast
    slow.append(fast)
    return slow


def sf_kick(slow, fast, tau):
    """Slow<->fast cross kick (sia.py:200-230, Newtonian branch)."""
    if slow.n and fast.n:
        extensions.acc.calc(slow, fast)
        extensions.acc.calc(fast, slow)
        kick_n(slow, tau)
        kick_n(fast, tau)
    return slow, fast


class Scheme(object):
    """One coefficient set with its kdk, dkd and bridge propagators."""

    def __init__(self, name):
        # op 0: kick (kdk), drift (dkd) or slow/fast drift (bridge)
        self.ops = palindrome(*COEFS[name])

    def kdk(self, ps, tau):
        if ps.n <= 2:
            return FewBody.evolve(ps, tau)
        for op, c in self.ops:
            ps = kick(ps, c * tau) if op == 0 else drift(ps, c * tau)
        return ps

    def dkd(self, ps, tau):
        if ps.n <= 2:
            return FewBody.evolve(ps, tau)
        for op, c in self.ops:
            ps = drift(ps, c * tau) if op == 0 else kick(ps, c * tau)
        return ps

    def bridge(self, slow, fast, tau, evolve, recurse):
        for op, c in self.ops:
            if op == 0:
                slow = evolve(slow, c * tau)
                fast = recurse(fast, c * tau, evolve, self.bridge)
            else:
                slow, fast = sf_kick(slow, fast, c * tau)
        return slow, fast


# attribute rows tg_sia_h_step reads and permutes, in TG_SIA_ROW_* order
# (the last one, nstep, is in the int64 block)
NATIVE_ROWS = ("mass", "eps2", "rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep", "tstepij",
               "ax", "ay", "az", "nstep")
KEPLER_CAP = 2   # TG_ST_KEPLER_CAP


class SIA(Base):
    PROVIDED_METHODS = tuple("%s%s.%s" % (s, m, f) for s in sorted(COEFS)
                             for m in ("s", "a", "h") for f in ("dkd", "kdk"))
    native_h = True

    def __init__(self, eta, time, ps, method, **kwargs):
        if kwargs.get("pn_order", 0):
            raise NotImplementedError("post-Newtonian SIA is not provided")
        super(SIA, self).__init__(eta, time, ps, **kwargs)
        if method not in self.PROVIDED_METHODS:
            raise ValueError("Unexpected method: %r" % method)
        self.method = method
        self.scheme = Scheme(method[:5])
        mode = method[5]
        self.update_tstep = mode in "ah"
        self.shared_tstep = mode in "sa"
        self.kdk = method.endswith("kdk")
        self.evolve = self.scheme.kdk if self.kdk else self.scheme.dkd
        nops = len(self.scheme.ops)
        self._op_kind = (ctypes.c_int * nops)(*[op for op, _ in self.scheme.ops])
        self._op_coef = (ctypes.c_double * nops)(*[c for _, c in self.scheme.ops])

    def recurse(self, ps, tau, evolve, bridge):
        """sia.py:1092-1123"""
        if not ps.n:
            return ps
        flag = -1
        if self.update_tstep:
            flag = 1
            ps.set_tstep(ps, self.eta)
            if self.shared_tstep:
                tau = self.get_min_block_tstep(ps, tau)
        if self.update_tstep:
            slow, fast = split(ps, ps.tstep.abs() > flag * abs(tau))
        else:
            # |tstep| > -|tau| holds for every particle: all slow, no copy
            slow, fast = ps, type(ps)(0)
        slow, fast = bridge(slow, fast, tau, evolve, self.recurse)
        if fast.n == 0:
            self.t_curr += tau
            ps.t_curr = self.t_curr
        if slow.n:
            slow.tstep.fill_(tau)
            slow.time += tau
            slow.nstep += 1
            self.record(slow, tau)
        return join(slow, fast)

    def do_step(self, ps, tau):
        # the native recursion has no per-level worldline or viewer hook
        if (self.native_h and self.update_tstep and not self.shared_tstep
                and not self.dumpper and not self.viewer):
            return self.native_step(ps, tau)
        return self.recurse(ps, tau, self.evolve, self.scheme.bridge)

    def native_step(self, ps, tau):
        """One h. step by tg_sia_h_step: the particles of `ps` are advanced
        and reordered in place (slow before fast at every level, the order
        recurse() returns), and t_curr advances as recurse() advances it.
        Kepler pairs that reach their retry bound are reported once per
        step."""
        if not ps.n:
            return ps
        for name in ("tstepij", "ax", "ay", "az"):
            if name not in ps._layout:
                ps.register_auxiliary_attribute(name, "real")
        real, ints = ps._real, ps._int
        if real.stride(1) != 1 or ints.stride(1) != 1:
            raise ValueError("particle blocks must have contiguous rows")
        rows = (ctypes.c_int * len(NATIVE_ROWS))(*[ps._layout[k][1] for k in NATIVE_ROWS])
        t = ctypes.c_double(self.t_curr)
        stream = _stream()
        prec = extensions.PRECISIONS
        _native.check(_native.lib.tg_sia_h_step(
            len(self._op_kind), self._op_kind, self._op_coef, int(self.kdk), float(self.eta), float(tau),
            prec[extensions.acc.kernel.prec], prec[extensions.tstep.kernel.prec], ps.n,
            real.data_ptr(), real.stride(0), len(ps._rnames), ints.data_ptr(), ints.stride(0), len(ps._inames),
            rows, ctypes.byref(t), stream), "tg_sia_h_step")
        self.t_curr = t.value
        ps.t_curr = self.t_curr
        st = _native.sync_status(stream)
        if st & KEPLER_CAP:
            warnings.warn("kepler_solver: retry bound reached for some pairs (status %d); "
                          "the last iterate was kept" % st, RuntimeWarning)
        return ps
