"""Run diagnostics of a GPU-resident particle system, as the reference's
`Diagnostic` reports them (tupan/simulation.py:39-129).

Every `report_freq`-th call of `diagnostic_report(ps)` writes one line with
the reference's columns: time, time since the previous report, kinetic,
potential and total energy, virial energy 2K + U, the relative energy error
eerr = (E - E0) / (-U), its running root mean square geerr, and the drifts
|com_r - com_r0|, |com_v - com_v0|, |P - P0| and |L - L0| of the centre of
mass and of the linear and angular momenta, then the wall-clock time since
the first report.  `fname` is a file, or '<stdout>' / '<stderr>' (the
reference's `myprint`, simulation.py:29-36).

The reductions run on the GPU in FP64 (tupan_gb300.particles): numpy-order
sums for K, U and the centre of mass, and the potential from the FP64 Phi
kernel, which makes each report one O(N^2) pairwise evaluation.  The values
of the last report are kept in `last` for callers that want them unprinted.
"""
import math
import sys
import timeit

COLUMNS = ("#00:time", "#01:dtime", "#02:ke", "#03:pe", "#04:te", "#05:virial", "#06:eerr",
           "#07:geerr", "#08:com_r", "#09:com_v", "#10:lmom", "#11:amom", "#12:wct")
HEADER_FMT = ("{0:13s} {1:10s} {2:10s} {3:10s} {4:15s} {5:10s} {6:10s} {7:10s} "
              "{8:10s} {9:10s} {10:10s} {11:10s} {12:13s}")
LINE_FMT = ("{time:< 13.6e} {dtime:< 10.3e} {ke:< 10.3e} {pe:< 10.3e} {te:< 15.8e} "
            "{virial:< 10.3e} {eerr:< 10.3e} {geerr:< 10.3e} {com_r:< 10.3e} {com_v:< 10.3e} "
            "{lmom:< 10.3e} {amom:< 10.3e} {wct:< 13.6e}")


def _write(text, fname, mode):
    if fname == "<stdout>":
        print(text, file=sys.stdout)
    elif fname == "<stderr>":
        print(text, file=sys.stderr)
    else:
        with open(fname, mode) as f:
            print(text, file=f)


def _norm(a, b):
    return math.sqrt(sum((float(x) - float(y)) ** 2 for x, y in zip(a, b)))


class Diagnostic(object):
    """Energy and momentum report of a run (simulation.py:39-129)."""

    def __init__(self, fname, time, ps, report_freq=4, pn_order=0):
        self.fname = fname
        self.time = time
        self.report_freq = report_freq
        self.include_pn_corrections = bool(pn_order)
        self.nreport = 0
        self.is_initialized = False
        self.last = None

    def initialize(self, ps):
        self.ke0 = ps.kinetic_energy
        self.pe0 = ps.potential_energy
        self.te0 = self.ke0 + self.pe0
        self.com_r0 = ps.com_r
        self.com_v0 = ps.com_v
        self.lmom0 = ps.linear_momentum
        self.amom0 = ps.angular_momentum
        self.count = 0
        self.ceerr = 0.0
        self.tic = timeit.default_timer()
        _write(HEADER_FMT.format(*COLUMNS), self.fname, "w")
        self.is_initialized = True

    def diagnostic_report(self, ps):
        if not self.is_initialized:
            self.initialize(ps)
        t_curr = getattr(ps, "t_curr", self.time)
        if self.nreport % self.report_freq == 0:
            self.print_diagnostic(t_curr, t_curr - self.time, ps)
        self.nreport += 1

    def print_diagnostic(self, time, dtime, ps):
        self.time = time
        ke = ps.kinetic_energy
        pe = ps.potential_energy
        te = ke + pe
        virial = 2 * ke + pe
        eerr = (te - self.te0) / (-pe)
        self.count += 1
        self.ceerr += eerr ** 2
        geerr = math.sqrt(self.ceerr / self.count)
        rec = dict(time=time, dtime=dtime, ke=ke, pe=pe, te=te, virial=virial, eerr=eerr, geerr=geerr,
                   com_r=_norm(ps.com_r, self.com_r0), com_v=_norm(ps.com_v, self.com_v0),
                   lmom=_norm(ps.linear_momentum, self.lmom0), amom=_norm(ps.angular_momentum, self.amom0),
                   wct=timeit.default_timer() - self.tic)
        self.last = rec
        _write(LINE_FMT.format(**rec), self.fname, "a")
