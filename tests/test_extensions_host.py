"""Host-side logic of the extensions layer, without a GPU: precision
selection as the reference makes it (`--use_sp` on the command line,
tupan/lib/utils/ctype.py:13-18), the backend names the reference passes, and
kernel-name resolution (libtupan.h symbols and short names)."""
import sys

import pytest


@pytest.fixture()
def ext(monkeypatch):
    monkeypatch.delenv("TUPAN_GB300_PREC", raising=False)
    from tupan_gb300.lib import extensions
    return extensions


def test_default_precision_is_fp64(ext, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["prog"])
    assert ext.default_precision() == "float64"
    assert ext.get_kernel("acc").prec == "float64"


def test_use_sp_selects_split_fp32(ext, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["prog", "--use_sp"])
    assert ext.get_kernel("acc_jerk").prec == "ds32"
    assert ext.AccJerk("C").kernel.prec == "ds32"


def test_environment_precision(ext, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["prog"])
    monkeypatch.setenv("TUPAN_GB300_PREC", "ds32")
    assert ext.get_kernel("phi").prec == "ds32"


def test_reference_backend_names_and_symbols(ext):
    for backend in ("C", "CL", "CUDA"):
        assert ext.get_kernel("acc_kernel", backend, "float64").name == "acc"
    assert ext.get_kernel("nreg_Xkernel", "C", "float64").name == "nreg_x"
    with pytest.raises(ValueError):
        ext.get_kernel("acc", "OCL")
    with pytest.raises(ValueError):
        ext.get_kernel("acc", "C", "float16")
    with pytest.raises(ValueError):
        ext.get_kernel("no_such_kernel", "C", "float64")


def test_ds32x_maps_to_double_single_only_where_it_exists(ext):
    from tupan_gb300 import _native
    assert ext.get_kernel("acc", "C", "ds32x").prec == "ds32x"
    assert ext.kernel_precision("acc", "ds32x") == _native.PREC_DS32X
    assert ext.kernel_precision("acc_jerk", "ds32x") == _native.PREC_DS32X
    for name in ("phi", "snap_crackle", "tstep", "pnacc"):
        assert ext.kernel_precision(name, "ds32x") == _native.PREC_DS32
    assert ext.kernel_precision("phi", "float64") == _native.PREC_FP64
