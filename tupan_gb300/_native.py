"""ctypes binding of libtupan_gb300.so (include/tupan_gb300.h).

The library is the only compute path: importing this module without the
built library raises ImportError with the build command, and there is no
CPU fallback anywhere in the package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("TUPAN_GB300_LIB") or os.path.join(HERE, "_lib", "libtupan_gb300.so")

PREC_FP64 = 0
PREC_DS32 = 1
PREC_DS32X = 2   # double-single arithmetic: Acc, AccJerk, the Acc adjoint

OK = 0
EINVAL = -1
ECUDA = -2
ENOMEM = -3
ENODEV = -4

ST_MBAR_TIMEOUT = 1
ST_KEPLER_CAP = 2

P5 = ("mass", "rx", "ry", "rz", "eps2")
P8 = P5 + ("vx", "vy", "vz")
P14 = P8 + ("ax", "ay", "az", "jx", "jy", "jz")

# kernel -> (particle fields, scalar ctypes, output names); libtupan.h:2-246
SPECS = {
    "phi": (P5, (), ("phi",)),
    "acc": (P5, (), ("ax", "ay", "az")),
    "acc_jerk": (P8, (), ("ax", "ay", "az", "jx", "jy", "jz")),
    "snap_crackle": (P14, (), ("sx", "sy", "sz", "cx", "cy", "cz")),
    "tstep": (P8, (ctypes.c_double,), ("tstep", "tstepij")),
    "pnacc": (P8, (ctypes.c_ulong,) + (ctypes.c_double,) * 7, ("pnax", "pnay", "pnaz")),
    "sakura": (P8, (ctypes.c_double, ctypes.c_long), ("drx", "dry", "drz", "dvx", "dvy", "dvz")),
    "nreg_x": (P8, (ctypes.c_double,), ("mrx", "mry", "mrz", "ax", "ay", "az", "u")),
    "nreg_v": (("mass", "vx", "vy", "vz", "ax", "ay", "az"), (ctypes.c_double,), ("mvx", "mvy", "mvz", "mk")),
}
# drop-in host symbols that are not <name>_kernel (libtupan.h:152-201)
HOST_SYMBOLS = {"nreg_x": "nreg_Xkernel", "nreg_v": "nreg_Vkernel"}
# the Kepler pair solver's fields, in argument order (libtupan.h:231-246)
KEPLER_FIELDS = P8
KEPLER_OUT = ("rx", "ry", "rz", "vx", "vy", "vz")

_DP = ctypes.c_void_p


class TupanGB300Error(RuntimeError):
    """A call into libtupan_gb300 returned an error code."""


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libtupan_gb300.so is not built (%s); run `python -m tupan_gb300.build` "
            "or __graft_entry__.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (fields, scal, outs) in SPECS.items():
        for prefix in ("tg_", ""):
            fn = getattr(lib, "tg_" + name if prefix else HOST_SYMBOLS.get(name, name + "_kernel"))
            args = [ctypes.c_size_t if prefix else ctypes.c_ulong] + [_DP] * len(fields)
            args += [ctypes.c_size_t if prefix else ctypes.c_ulong] + [_DP] * len(fields)
            args += list(scal) + [_DP] * len(outs)
            if prefix:
                args += [ctypes.c_int, _DP]
                fn.restype = ctypes.c_int
            else:
                fn.restype = None
            fn.argtypes = args
    lib.tg_version.restype = ctypes.c_char_p
    lib.tg_last_error.restype = ctypes.c_char_p
    lib.tg_sync_status.restype = ctypes.c_int
    lib.tg_sync_status.argtypes = [_DP]
    lib.tg_set_host_precision.argtypes = [ctypes.c_int]
    lib.tg_set_host_precision.restype = ctypes.c_int
    lib.tg_get_host_precision.restype = ctypes.c_int
    lib.tg_device_sms.restype = ctypes.c_int
    for nm in ("tg_drift", "tg_kick"):
        getattr(lib, nm).restype = ctypes.c_int
        getattr(lib, nm).argtypes = [ctypes.c_size_t] + [_DP] * 6 + [ctypes.c_double, _DP]
    lib.tg_add_increments.restype = ctypes.c_int
    lib.tg_add_increments.argtypes = [ctypes.c_size_t] + [_DP] * 12 + [_DP]
    PP = ctypes.POINTER(ctypes.c_void_p)
    lib.tg_hermite_predict.restype = ctypes.c_int
    lib.tg_hermite_predict.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_double, PP, PP, _DP]
    lib.tg_hermite_correct.restype = ctypes.c_int
    lib.tg_hermite_correct.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_double, PP, PP, PP, PP, _DP]
    lib.tg_acc_vjp.restype = ctypes.c_int
    lib.tg_acc_vjp.argtypes = [ctypes.c_size_t] + [_DP] * 12 + [ctypes.c_int, _DP]
    lib.tg_probe_fma_tflops.restype = ctypes.c_double
    lib.tg_probe_fma_tflops.argtypes = [ctypes.c_int, ctypes.c_int, _DP]
    lib.tg_set_recompute_threshold.restype = ctypes.c_double
    lib.tg_set_recompute_threshold.argtypes = [ctypes.c_double]
    lib.tg_time_pair_kernel.restype = ctypes.c_int
    lib.tg_time_pair_kernel.argtypes = [ctypes.c_int]
    lib.tg_pair_kernel_time.restype = ctypes.c_int
    lib.tg_pair_kernel_time.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_longlong)]
    lib.tg_set_sakura_split.restype = ctypes.c_int
    lib.tg_set_sakura_split.argtypes = [ctypes.c_int]
    lib.tg_check_bounded_wait.restype = ctypes.c_int
    lib.tg_check_bounded_wait.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.tg_div3.restype = ctypes.c_int
    lib.tg_div3.argtypes = [ctypes.c_size_t] + [_DP] * 6 + [ctypes.c_double, _DP]
    lib.tg_sum.restype = ctypes.c_int
    lib.tg_sum.argtypes = [ctypes.c_size_t, _DP, _DP, _DP]
    lib.tg_kepler_solver.restype = ctypes.c_int
    lib.tg_kepler_solver.argtypes = [ctypes.c_size_t] + [_DP] * 8 + [ctypes.c_double] + [_DP] * 6 + [_DP]
    lib.tg_sia_h_step.restype = ctypes.c_int
    lib.tg_sia_h_step.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_size_t, _DP, ctypes.c_size_t, ctypes.c_int, _DP, ctypes.c_size_t,
                                  ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), _DP]
    lib.kepler_solver_kernel.restype = None
    lib.kepler_solver_kernel.argtypes = [_DP] * 8 + [ctypes.c_double] + [_DP] * 6
    return lib


lib = _load()


def last_error():
    return lib.tg_last_error().decode()


def check(rc, what):
    if rc != OK:
        raise TupanGB300Error("%s failed (code %d): %s" % (what, rc, last_error()))
    return rc


def call_device(name, ni, iptrs, nj, jptrs, scalars, optrs, prec, stream):
    """Call tg_<name> with raw device pointers (ints); raises on error."""
    fn = getattr(lib, "tg_" + name)
    rc = fn(ni, *iptrs, nj, *jptrs, *scalars, *optrs, int(prec), stream)
    return check(rc, "tg_" + name)


KERNEL_ACC = 1
KERNEL_ACC_JERK = 2


def pair_kernel_time(kernel):
    """(total ms, launches) of the ordered pairwise kernel of `kernel`
    (KERNEL_ACC or KERNEL_ACC_JERK) recorded while tg_time_pair_kernel was on."""
    ms, n = ctypes.c_double(), ctypes.c_longlong()
    check(lib.tg_pair_kernel_time(kernel, ctypes.byref(ms), ctypes.byref(n)), "tg_pair_kernel_time")
    return ms.value, n.value


def set_recompute_threshold(tau):
    """Split-FP32 Acc/AccJerk accuracy control (tg_set_recompute_threshold):
    returns the previous threshold; raises on a value outside [1, 1e6]."""
    prev = lib.tg_set_recompute_threshold(float(tau))
    if prev < 0:
        raise ValueError("recompute threshold must lie in [1, 1e6], got %r" % (tau,))
    return prev


def sync_status(stream=None):
    rc = lib.tg_sync_status(stream)
    if rc < 0:
        raise TupanGB300Error("tg_sync_status failed: %s" % last_error())
    return rc


def current_stream():
    """Handle of torch's current CUDA stream on the current device: the
    value of torch.cuda.current_stream().cuda_stream, without building the
    Stream object (the integrators ask for it before every launch)."""
    import torch
    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:
        return raw(torch.cuda.current_device())
    return torch.cuda.current_stream().cuda_stream


def psum(t):
    """float(sum of a float64 CUDA tensor) in numpy's pairwise order (tg_sum),
    so the value equals numpy.sum of the same array bit for bit."""
    import torch
    t = t.contiguous()
    if not (t.is_cuda and t.dtype == torch.float64):
        raise TypeError("psum expects a float64 CUDA tensor")
    out = torch.empty(1, dtype=torch.float64, device=t.device)
    check(lib.tg_sum(t.numel(), t.data_ptr(), out.data_ptr(), current_stream()),
          "tg_sum")
    return float(out.item())


def ptr_array(tensors):
    """A host array of device pointers (for the tg_hermite_* entry points)."""
    arr = (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])
    return arr
