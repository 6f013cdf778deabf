"""High-level kernel interface, mirroring tupan/lib/extensions.py.

Same class names (Phi, Acc, AccJerk, SnapCrackle, Tstep, PNAcc, Sakura,
NREG_X, NREG_V, Kepler), the same `calc(ips, jps, *args)` call, the same
output attribute names registered on `ips` through
`ips.register_auxiliary_attribute(name, "real")`, the same module singletons
and the same `clight` object (extensions.py:30-60, 94-97, 100-651, 654-666).  The only backend is "CUDA": the GB300 library
libtupan_gb300.so, reached through a Kernel object with the reference's
protocol (cty, set_gsize, set_args, map_buffers, run; cffi_backend.py:90-126).

Precision ("prec") is "float64" (FP64 kernels, bit-identical to the reference
for Phi/Acc/AccJerk/SnapCrackle/Tstep), "ds32" (split FP32; "float32" is
accepted as an alias) or "ds32x" (double-single arithmetic, ~1e-12, for Acc
and AccJerk; the other kernels run it as "ds32").  The default is "ds32" when `--use_sp` is on the
command line (as the reference selects single precision), else
TUPAN_GB300_PREC, else float64; `--use_cl` (the reference's OpenCL switch)
selects nothing: the only backend is CUDA.

Particle arrays may be float64 CUDA torch tensors (used in place, no copies)
or numpy arrays (copied to the GPU, results copied back into the registered
numpy outputs, like the reference's OpenCL backend, opencl_backend.py:117-164).
"""
import os
import sys
import warnings
from collections import namedtuple

import numpy as np
import torch

from .. import _native

__all__ = ["Phi", "phi",
           "Acc", "acc",
           "AccJerk", "acc_jerk",
           "SnapCrackle", "snap_crackle",
           "Tstep", "tstep",
           "PNAcc", "pnacc",
           "Sakura", "sakura",
           "NREG_X", "nreg_x",
           "NREG_V", "nreg_v",
           "Kepler", "kepler",
           "Clight", "clight", "get_kernel"]

PRECISIONS = {"float64": _native.PREC_FP64, "ds32": _native.PREC_DS32,
              "float32": _native.PREC_DS32, "ds32x": _native.PREC_DS32X}
# kernels with a double-single form; the others run "ds32x" as "ds32"
DS32X_KERNELS = ("acc", "acc_jerk")


def kernel_precision(name, prec):
    """The TG_PREC_* code a kernel runs a precision name at."""
    if prec == "ds32x" and name not in DS32X_KERNELS:
        return _native.PREC_DS32
    return PRECISIONS[prec]


class Clight(object):
    """PN order, speed of light and its inverse powers (extensions.py:30-60)."""

    def __init__(self):
        self._pn_order = 0
        self._clight = None
        for k in range(1, 8):
            setattr(self, "inv%d" % k, 0.0)

    @property
    def pn_order(self):
        return self._pn_order

    @pn_order.setter
    def pn_order(self, value):
        self._pn_order = int(value)

    @property
    def clight(self):
        return self._clight

    @clight.setter
    def clight(self, value):
        self._clight = float(value)
        self.inv1 = 1.0 / self._clight
        self.inv2 = self.inv1 ** 2
        self.inv3 = self.inv1 ** 3
        self.inv4 = self.inv1 ** 4
        self.inv5 = self.inv1 ** 5
        self.inv6 = self.inv1 ** 6
        self.inv7 = self.inv1 ** 7


class _DeviceArg(object):
    """A float64 device buffer standing for one kernel array argument."""
    __slots__ = ("tensor", "host", "writeback")

    def __init__(self, tensor, host=None, writeback=None):
        self.tensor = tensor
        self.host = host            # numpy array to copy results into
        self.writeback = writeback  # torch tensor to copy results into

    @property
    def ptr(self):
        return self.tensor.data_ptr()


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("tupan_gb300 needs a CUDA device; none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def _ptr(arg):
    """Device address of a converted array argument."""
    return arg.data_ptr() if isinstance(arg, torch.Tensor) else arg.ptr


def _to_device_arg(x, output):
    """Convert one array argument (numpy or torch): a float64 contiguous CUDA
    tensor is used as it is, anything else becomes a _DeviceArg staging
    copy."""
    if isinstance(x, torch.Tensor):
        if x.is_cuda and x.dtype == torch.float64 and x.is_contiguous():
            return x
        t = x.detach().to(device=_device(), dtype=torch.float64).contiguous()
        return _DeviceArg(t, writeback=x if output else None)
    a = np.asarray(x)
    if output:
        t = torch.empty(a.shape[0], dtype=torch.float64, device=_device())
        return _DeviceArg(t, host=a)
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(_device(), non_blocking=False)
    return _DeviceArg(t)


class CUDAKernel(object):
    """Kernel object with the reference backend protocol (cffi_backend.py:90-126)."""

    def __init__(self, prec, name):
        if prec not in PRECISIONS:
            raise ValueError("Inappropriate 'prec': %r. Supported: %s" % (prec, sorted(PRECISIONS)))
        self.prec = prec
        host = {v: k for k, v in _native.HOST_SYMBOLS.items()}
        self.name = host.get(name, name[:-len("_kernel")] if name.endswith("_kernel") else name)
        if self.name not in _native.SPECS and self.name != "kepler_solver":
            raise ValueError("unknown kernel %r" % name)
        types = namedtuple("Types", ["c_int", "c_int_p", "c_uint", "c_uint_p", "c_real", "c_real_p"])
        self.cty = types(c_int=int, c_int_p=None, c_uint=int, c_uint_p=None, c_real=float,
                         c_real_p=lambda x: _to_device_arg(x, output=False))
        self.c_real_out = lambda x: _to_device_arg(x, output=True)
        self.args = None
        self.ni = self.nj = 0

    def set_gsize(self, ni, nj):
        self.ni, self.nj = int(ni), int(nj)

    def allocate_local_memory(self, numbufs, sctype):
        return []

    def set_args(self, args, start=0):
        self.args = list(args)

    def run(self):
        if self.name == "kepler_solver":
            return self._run_kepler()
        fields, scal, outs = _native.SPECS[self.name]
        nf, ns, no = len(fields), len(scal), len(outs)
        a = self.args
        ni = int(a[0])
        iptr = [_ptr(x) for x in a[1:1 + nf]]
        nj = int(a[1 + nf])
        jptr = [_ptr(x) for x in a[2 + nf:2 + 2 * nf]]
        sc = a[2 + 2 * nf:2 + 2 * nf + ns]
        optr = [_ptr(x) for x in a[2 + 2 * nf + ns:]]
        assert len(optr) == no
        stream = _native.current_stream()
        _native.call_device(self.name, ni, iptr, nj, jptr, sc, optr, kernel_precision(self.name, self.prec), stream)
        if self.name == "sakura":
            st = _native.sync_status(stream)
            if st:
                warnings.warn("sakura: Kepler retry bound reached for some pairs (status %d); "
                              "the last iterate was kept" % st, RuntimeWarning)

    def _run_kepler(self):
        # args: m, rx, ry, rz, e2, vx, vy, vz, dt, then the six outputs
        a = self.args
        n = (a[0] if isinstance(a[0], torch.Tensor) else a[0].tensor).numel()
        if n % 2:
            raise ValueError("kepler_solver: the particle set must hold whole pairs (n = %d)" % n)
        stream = _native.current_stream()
        rc = _native.lib.tg_kepler_solver(n // 2, *[_ptr(x) for x in a[:8]], float(a[8]),
                                          *[_ptr(x) for x in a[9:15]], stream)
        _native.check(rc, "tg_kepler_solver")
        st = _native.sync_status(stream)
        if st:
            warnings.warn("kepler_solver: retry bound reached for some pairs (status %d); "
                          "the last iterate was kept" % st, RuntimeWarning)

    def map_buffers(self, arrays, buffers):
        for arr, buf in zip(arrays, buffers):
            if isinstance(buf, torch.Tensor):   # written in place
                continue
            if buf.host is not None:
                buf.host[...] = buf.tensor.cpu().numpy()
            elif buf.writeback is not None:
                buf.writeback.copy_(buf.tensor)
        return arrays


def default_precision():
    """Precision of kernels made without an explicit `prec`: "ds32" when
    `--use_sp` is on the command line (the reference's single-precision
    switch, tupan/lib/utils/ctype.py:13-18), else TUPAN_GB300_PREC, else
    "float64"."""
    if "--use_sp" in sys.argv:
        return "ds32"
    return os.environ.get("TUPAN_GB300_PREC", "float64")


def get_kernel(name, backend="CUDA", prec=None):
    if backend not in ("CUDA", "C", "CL"):
        raise ValueError("Inappropriate 'backend': %s. Supported values: ['CUDA']" % backend)
    if prec is None:
        prec = default_precision()
    return CUDAKernel(prec, name)


def prepare_args(args, argtypes):
    return [argtype(arg) for (arg, argtype) in zip(args, argtypes)]


def _register(ips, names):
    for n in names:
        if not hasattr(ips, n):
            ips.register_auxiliary_attribute(n, "real")


class AbstractExtension(object):
    name = None
    outputs = ()

    def __init__(self, backend="CUDA", prec=None):
        self.kernel = get_kernel(self.name, backend, prec)
        fields, scal, outs = _native.SPECS[self.kernel.name]
        cty = self.kernel.cty
        self.argtypes = ((cty.c_uint,) + (cty.c_real_p,) * len(fields)) * 2
        self.restypes = (self.kernel.c_real_out,) * len(outs)

    def _fields(self, ps):
        fields = _native.SPECS[self.kernel.name][0]
        return tuple(getattr(ps, f) for f in fields)

    def set_args(self, ips, jps, *args):
        ni, nj = ips.n, jps.n
        self.kernel.set_gsize(ni, nj)
        _register(ips, self.outputs)
        self._inargs = (ni,) + self._fields(ips) + (nj,) + self._fields(jps)
        self._scalars = tuple(args)
        self._outargs = tuple(getattr(ips, n) for n in self.outputs)
        self.inargs = prepare_args(self._inargs, self.argtypes)
        self.outargs = prepare_args(self._outargs, self.restypes)
        self.kernel.set_args(self.inargs + list(self._scalars) + self.outargs)

    def run(self):
        self.kernel.run()

    def get_result(self):
        return self.kernel.map_buffers(self._outargs, self.outargs)

    def calc(self, ips, jps, *args):
        self.set_args(ips, jps, *args)
        self.run()
        return self.get_result()


class Phi(AbstractExtension):
    """Gravitational potential (extensions.py:100-160)."""
    name = "phi_kernel"
    outputs = ("phi",)


class Acc(AbstractExtension):
    """Gravitational acceleration (extensions.py:163-235)."""
    name = "acc_kernel"
    outputs = ("ax", "ay", "az")


class AccJerk(AbstractExtension):
    """Acceleration and jerk (extensions.py:238-283)."""
    name = "acc_jerk_kernel"
    outputs = ("ax", "ay", "az", "jx", "jy", "jz")


class SnapCrackle(AbstractExtension):
    """Snap and crackle (extensions.py:286-339)."""
    name = "snap_crackle_kernel"
    outputs = ("sx", "sy", "sz", "cx", "cy", "cz")


class Tstep(AbstractExtension):
    """Pairwise time-step criterion (extensions.py:342-382): calc(ips, jps, eta)."""
    name = "tstep_kernel"
    outputs = ("tstep", "tstepij")

    def set_args(self, ips, jps, eta):
        super(Tstep, self).set_args(ips, jps, float(eta))


class PNAcc(AbstractExtension):
    """Post-Newtonian acceleration (extensions.py:385-436); reads `clight`."""
    name = "pnacc_kernel"
    outputs = ("pnax", "pnay", "pnaz")

    def set_args(self, ips, jps):
        c = clight
        super(PNAcc, self).set_args(ips, jps, int(c.pn_order), c.inv1, c.inv2, c.inv3,
                                    c.inv4, c.inv5, c.inv6, c.inv7)


class Sakura(AbstractExtension):
    """Sakura pairwise Kepler drift (extensions.py:439-507): calc(ips, jps, dt, flag)."""
    name = "sakura_kernel"
    outputs = ("drx", "dry", "drz", "dvx", "dvy", "dvz")

    def set_args(self, ips, jps, dt, flag):
        super(Sakura, self).set_args(ips, jps, float(dt), int(flag))


class NREG_X(AbstractExtension):
    """NREG position step (extensions.py:510-566): calc(ips, jps, dt) ->
    (mrx, mry, mrz, ax, ay, az, u).  Always FP64."""
    name = "nreg_Xkernel"
    outputs = ("mrx", "mry", "mrz", "ax", "ay", "az", "u")

    def set_args(self, ips, jps, dt):
        super(NREG_X, self).set_args(ips, jps, float(dt))


class NREG_V(AbstractExtension):
    """NREG velocity step (extensions.py:569-617): calc(ips, jps, dt) ->
    (mvx, mvy, mvz, mk).  Always FP64."""
    name = "nreg_Vkernel"
    outputs = ("mvx", "mvy", "mvz", "mk")

    def set_args(self, ips, jps, dt):
        super(NREG_V, self).set_args(ips, jps, float(dt))


class Kepler(object):
    """Kepler pair solver (extensions.py:620-651): calc(ips, jps, dt) moves
    the particles of `ips` in place; every consecutive pair (2p, 2p+1) is
    one two-body problem (the reference passes exactly one pair).  `jps` is
    unused, as in the reference.  FP64."""
    name = "kepler_solver_kernel"
    fields = ("mass", "rx", "ry", "rz", "eps2", "vx", "vy", "vz")
    outputs = ("rx", "ry", "rz", "vx", "vy", "vz")

    def __init__(self, backend="CUDA", prec=None):
        self.kernel = get_kernel(self.name, backend, prec)
        self.argtypes = (self.kernel.cty.c_real_p,) * len(self.fields)
        self.restypes = (self.kernel.c_real_out,) * len(self.outputs)

    def set_args(self, ips, jps, dt):
        self._inargs = tuple(getattr(ips, f) for f in self.fields)
        self._outargs = tuple(getattr(ips, f) for f in self.outputs)
        self.inargs = prepare_args(self._inargs, self.argtypes)
        self.outargs = prepare_args(self._outargs, self.restypes)
        self.kernel.set_args(self.inargs + [float(dt)] + self.outargs)

    def run(self):
        self.kernel.run()

    def get_result(self):
        return self.kernel.map_buffers(self._outargs, self.outargs)

    def calc(self, ips, jps, dt):
        self.set_args(ips, jps, dt)
        self.run()
        return self.get_result()


backend = "CUDA"

clight = Clight()
phi = Phi(backend)
acc = Acc(backend)
acc_jerk = AccJerk(backend)
snap_crackle = SnapCrackle(backend)
tstep = Tstep(backend)
pnacc = PNAcc(backend)
sakura = Sakura(backend)
nreg_x = NREG_X(backend)
nreg_v = NREG_V(backend)
kepler = Kepler(backend)


def set_precision(prec):
    """Switch every module singleton to `prec` ("float64" or "ds32").  The
    Sakura, NREG and Kepler kernels compute in FP64 either way."""
    global phi, acc, acc_jerk, snap_crackle, tstep, pnacc, sakura
    phi = Phi(backend, prec)
    acc = Acc(backend, prec)
    acc_jerk = AccJerk(backend, prec)
    snap_crackle = SnapCrackle(backend, prec)
    tstep = Tstep(backend, prec)
    pnacc = PNAcc(backend, prec)
    sakura = Sakura(backend, prec)
