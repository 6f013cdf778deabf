"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the cpu_baseline / reference legs of bench.py as the checker.  The product
package (tupan_gb300) never imports this module.

Two CPU implementations share one calling convention here:

* ``Oracle()``      -- oracle/tupan_oracle.c, the restatement of the reference
                       algorithm (built by oracle/Makefile into oracle/_build/);
                       multi-threaded over i-slices.
* ``ReferenceLib()`` -- the reference's own C backend compiled unmodified from
                       its sources by oracle/ref.mk into oracle/_ref/ (only
                       where the reference tree is mounted).

Both take particle sets as mappings of float64 numpy arrays with the
reference attribute names (tupan/particles/body.py:26-39: mass, rx, ry, rz,
eps2, vx, vy, vz; plus ax..az, jx..jz for SnapCrackle) and return a tuple of
float64 output arrays in the reference output order
(tupan/lib/extensions.py:100-507).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

P5 = ("mass", "rx", "ry", "rz", "eps2")
P8 = P5 + ("vx", "vy", "vz")
P14 = P8 + ("ax", "ay", "az", "jx", "jy", "jz")

# name -> (particle fields, scalar kinds, output names); libtupan.h:2-246
SPECS = {
    "phi": (P5, (), ("phi",)),
    "acc": (P5, (), ("ax", "ay", "az")),
    "acc_jerk": (P8, (), ("ax", "ay", "az", "jx", "jy", "jz")),
    "snap_crackle": (P14, (), ("sx", "sy", "sz", "cx", "cy", "cz")),
    "tstep": (P8, ("real",), ("tstep", "tstepij")),
    "pnacc": (P8, ("uint",) + ("real",) * 7, ("pnax", "pnay", "pnaz")),
    "sakura": (P8, ("real", "int"), ("drx", "dry", "drz", "dvx", "dvy", "dvz")),
    "nreg_x": (P8, ("real",), ("mrx", "mry", "mrz", "ax", "ay", "az", "u")),
    "nreg_v": (("mass", "vx", "vy", "vz", "ax", "ay", "az"), ("real",), ("mvx", "mvy", "mvz", "mk")),
}
# kernels whose reference symbol is not <name>_kernel (libtupan.h:152-201)
REF_SYMBOLS = {"nreg_x": "nreg_Xkernel", "nreg_v": "nreg_Vkernel"}
KEPLER_OUT = ("rx", "ry", "rz", "vx", "vy", "vz")

_DP = ctypes.POINTER(ctypes.c_double)


def build(quiet=True):
    """Compile oracle/_build/liboracle.so with make (gcc)."""
    out = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "_build", "liboracle.so")


def _as_f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


class _CLib:
    prefix = ""
    threaded = False

    def __init__(self, path):
        self.lib = ctypes.CDLL(path)

    def _scalar(self, kind, value):
        if kind == "real":
            return ctypes.c_double(float(value))
        if kind == "uint":
            return ctypes.c_ulong(int(value))
        return ctypes.c_long(int(value))

    def calc(self, name, ips, jps, *scalars, nthreads=1):
        fields, kinds, outs = SPECS[name]
        if len(scalars) != len(kinds):
            raise TypeError("%s expects %d scalar arguments" % (name, len(kinds)))
        ni = len(ips["mass"])
        nj = len(jps["mass"])
        keep = []

        def ptr(a):
            a = _as_f64(a)
            keep.append(a)
            return a.ctypes.data_as(_DP)

        args = [ctypes.c_size_t(ni)] + [ptr(ips[f]) for f in fields]
        args += [ctypes.c_size_t(nj)] + [ptr(jps[f]) for f in fields]
        args += [self._scalar(k, v) for k, v in zip(kinds, scalars)]
        res = tuple(np.zeros(ni) for _ in outs)
        args += [r.ctypes.data_as(_DP) for r in res]
        if self.threaded:
            args.append(ctypes.c_int(int(nthreads)))
        fn = getattr(self.lib, self.symbol(name))
        fn.restype = None
        fn(*args)
        return res

    def symbol(self, name):
        return self.prefix + name + self.suffix

    def _kepler_args(self, ps, dt, npairs):
        keep, res = [], tuple(np.zeros(2 * npairs) for _ in KEPLER_OUT)
        for f in P8:
            a = _as_f64(ps[f])
            if a.shape != (2 * npairs,):
                raise ValueError("kepler: %s must hold 2 x npairs values" % f)
            keep.append(a)
        args = [a.ctypes.data_as(_DP) for a in keep] + [ctypes.c_double(float(dt))]
        args += [r.ctypes.data_as(_DP) for r in res]
        return keep, res, args


class Oracle(_CLib):
    """The restated algorithm (oracle/tupan_oracle.c)."""
    prefix = "orc_"
    suffix = ""
    threaded = True

    def kepler(self, ps, dt, nthreads=1, capped=None):
        """Kepler pair solver over consecutive pairs (2p, 2p+1) of `ps`;
        returns (rx, ry, rz, vx, vy, vz) after dt
        (kepler_solver_kernel_common.h:8-81).  If `capped` is a list, it
        receives one flag per pair: True where a retry bound was reached."""
        npairs = len(ps["mass"]) // 2
        keep, res, args = self._kepler_args(ps, dt, npairs)
        flags = np.zeros(npairs, dtype=np.intc)
        fn = self.lib.orc_kepler_solver
        fn.restype = None
        fn(ctypes.c_size_t(npairs), *args, flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
           ctypes.c_int(int(nthreads)))
        if capped is not None:
            capped[:] = [bool(x) for x in flags]
        return res

    def __init__(self, path=None):
        if path is None:
            path = os.path.join(HERE, "_build", "liboracle.so")
            if not os.path.exists(path):
                path = build()
        super().__init__(path)


class ReferenceLib(_CLib):
    """The reference's C backend, built from its sources by oracle/ref.mk."""
    prefix = ""
    suffix = "_kernel"
    threaded = False

    def __init__(self, path=None):
        if path is None:
            path = os.path.join(HERE, "_ref", "libtupan_ref_f64.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        super().__init__(path)

    def _scalar(self, kind, value):
        # FP64 build of the reference: UINT = unsigned long, INT = long
        return super()._scalar(kind, value)

    def symbol(self, name):
        return REF_SYMBOLS.get(name, name + self.suffix)

    def kepler(self, ps, dt, nthreads=1):
        """The reference kepler_solver_kernel, one call per pair."""
        npairs = len(ps["mass"]) // 2
        res = tuple(np.zeros(2 * npairs) for _ in KEPLER_OUT)
        fn = self.lib.kepler_solver_kernel
        fn.restype = None
        for p in range(npairs):
            sub = {f: _as_f64(ps[f])[2 * p:2 * p + 2].copy() for f in P8}
            _, out, args = self._kepler_args(sub, dt, 1)
            fn(*args)
            for r, o in zip(res, out):
                r[2 * p:2 * p + 2] = o
        return res


def reference_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libtupan_ref_f64.so"))
