"""The C ABI library loads without a GPU and exports every symbol include/*.h declares,
and the Python binding covers the same set."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(qsv_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    from qip_gb300 import _native, build

    path = build.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_native.SIGNATURES) == syms


def test_status_strings_without_a_device():
    from qip_gb300 import _native

    lib = _native.load()
    assert lib.qsv_status_string(0) == b"ok"
    assert lib.qsv_status_string(1) == b"invalid argument"
    assert lib.qsv_launch_count() >= 0


def test_library_is_sm103a_only():
    from qip_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_state_size_and_dtype_limits_without_a_device():
    """qsv_create rejects n outside [1, 34] and unknown dtypes before any device call;
    the Python layer raises the reference's ValueError for them."""
    import numpy
    import pytest

    from qip_gb300 import GpuBackend, _native

    lib = _native.load()
    h = ctypes.c_void_p()
    for n, dtype in ((0, 1), (35, 0), (10, 7)):
        assert lib.qsv_create(n, dtype, ctypes.byref(h)) == 1  # QSV_ERR_INVALID
        assert lib.qsv_last_error(None)
        assert not h.value
    with pytest.raises(ValueError):
        GpuBackend.make_state(35, [], [], statetype=numpy.complex64)


def test_normal_build_is_not_the_bounds_checked_one():
    """qsv_bounds_report answers only in libqsv_checked.so; the normal build says so
    without touching a device."""
    from qip_gb300 import _native

    count, first = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    assert _native.load().qsv_bounds_report(ctypes.byref(count), ctypes.byref(first)) == _native.QSV_ERR_UNSUPPORTED


def test_adjoint_plan_queries_check_their_arguments_without_a_device():
    """The adjoint plan's host-side queries reject a null plan or output before any
    device call (the scratch size of a null plan is 0)."""
    from qip_gb300 import _native

    lib = _native.load()
    out = ctypes.c_int(-1)
    assert lib.qsv_adjoint_plan_fused_blocks(None, ctypes.byref(out)) == _native.QSV_ERR_INVALID
    assert out.value == -1
    assert lib.qsv_adjoint_scratch_bytes(None, 64) == 0
    bad = ctypes.c_void_p()
    # Too many blocks for one walk launch (grid y <= 65535) or none at all.
    assert lib.qsv_adjoint_plan_create(24, 0, None, None, None, ctypes.byref(bad)) == _native.QSV_ERR_INVALID
    assert lib.qsv_adjoint_plan_create(24, 65536, None, None, None, ctypes.byref(bad)) == _native.QSV_ERR_INVALID
    assert not bad.value
