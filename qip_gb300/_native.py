"""ctypes binding of libqsv.so (the C ABI declared in include/qsv.h).

The library is built in-tree by ``qip_gb300.build``.  Loading never falls back to a
CPU implementation: if the library cannot be loaded, every backend call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy

from . import build as _build

QSV_C64 = 0
QSV_C128 = 1

QSV_OK = 0
QSV_ERR_INVALID = 1
QSV_ERR_OOM = 2
QSV_ERR_CUDA = 3
QSV_ERR_TIMEOUT = 4
QSV_ERR_UNSUPPORTED = 5

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int64_p = ctypes.POINTER(ctypes.c_int64)
_handle = ctypes.c_void_p

# name -> (restype, argtypes); mirrors include/qsv.h
SIGNATURES = {
    "qsv_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "qsv_destroy": (ctypes.c_int, [_handle]),
    "qsv_trim": (ctypes.c_int, []),
    "qsv_bounds_report": (ctypes.c_int, [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong)]),
    "qsv_set_stream": (ctypes.c_int, [_handle, ctypes.c_void_p]),
    "qsv_synchronize": (ctypes.c_int, [_handle]),
    "qsv_num_qubits": (ctypes.c_int, [_handle]),
    "qsv_dtype": (ctypes.c_int, [_handle]),
    "qsv_device_ptr": (ctypes.c_void_p, [_handle]),
    "qsv_last_error": (ctypes.c_char_p, [_handle]),
    "qsv_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "qsv_launch_count": (ctypes.c_ulonglong, []),
    "qsv_set_product_state": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, _c_int_p, _c_double_p]),
    "qsv_write_range": (ctypes.c_int, [_handle, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64]),
    "qsv_add_range": (ctypes.c_int, [_handle, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64]),
    "qsv_read_range": (ctypes.c_int, [_handle, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64]),
    "qsv_apply_matrix": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, ctypes.c_int, _c_int_p, _c_double_p]),
    "qsv_apply_diagonal": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, ctypes.c_int, _c_int_p, _c_double_p]),
    "qsv_apply_monomial": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, ctypes.c_int, _c_int_p, _c_int_p,
                                          _c_double_p]),
    "qsv_apply_swap": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, _c_int_p, ctypes.c_int, _c_int_p]),
    "qsv_trace_push": (ctypes.c_int, [ctypes.c_char_p]),
    "qsv_trace_pop": (ctypes.c_int, []),
    "qsv_host_alloc": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    "qsv_host_free": (ctypes.c_int, [ctypes.c_void_p]),
    "qsv_batch_segment_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  _c_int_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p]),
    "qsv_batch_segment_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_int, _c_int_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                  ctypes.c_void_p]),
    "qsv_fusion_plan": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, _c_double_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, _c_int_p, _c_int_p, _c_int_p, _c_int_p]),
    "qsv_block_matrices": (ctypes.c_int, [ctypes.c_int, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p,
                                           _c_double_p, _c_double_p]),
    "qsv_tune_blocks": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, _c_int_p, ctypes.c_int, _c_double_p, _c_int_p]),
    "qsv_set_block_mode": (ctypes.c_int, [_handle, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "qsv_apply_blocks": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, _c_int_p, _c_double_p]),
    "qsv_probabilities": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, _c_double_p]),
    "qsv_norm2": (ctypes.c_int, [_handle, _c_double_p]),
    "qsv_qubit_marginals": (ctypes.c_int, [_handle, _c_double_p, _c_double_p]),
    "qsv_collapse": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, ctypes.c_uint64, ctypes.c_double]),
    "qsv_reduce": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, ctypes.c_uint64, ctypes.c_double]),
    "qsv_plan_create": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, _c_int_p, _c_double_p,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "qsv_plan_launch": (ctypes.c_int, [_handle, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "qsv_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "qsv_inject_block_stall": (ctypes.c_int, [_handle, ctypes.c_uint64]),
    "qsv_adjoint_plan_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "qsv_adjoint_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "qsv_adjoint_scratch_bytes": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_int]),
    "qsv_adjoint_plan_fused_blocks": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "qsv_adjoint_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "qsv_adjoint_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "qsv_adjoint_status": (ctypes.c_int, [ctypes.c_void_p]),
    "qsv_batch_rotation_matrices": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p]),
    "qsv_probabilities_static": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_int_p,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "qsv_inner_product": (ctypes.c_int, [_handle, _handle, _c_double_p, _c_double_p]),
    "qsv_batch_reset": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "qsv_batch_apply_1q": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "qsv_batch_observable_sumz": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                 ctypes.c_void_p]),
    "qsv_batch_adjoint_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_size_t, ctypes.c_void_p]),
    "qsv_circuits_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "qsv_circuits_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "qsv_circuits_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "qsv_circuits_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "qsv_circuits_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "qsv_func_apply": (ctypes.c_int, [_handle, ctypes.c_int, _c_int_p, ctypes.c_int, _c_int_p, _c_int64_p]),
}

_lib = None
_lock = threading.Lock()


class QsvError(RuntimeError):
    """A libqsv call failed (CUDA error, device timeout, unsupported request)."""


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libqsv.so (building it first when it is missing).  Raises on failure."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        # QSV_BOUNDS_CHECK=1 selects the bounds-checked library (tests of the kernels'
        # indexing); it must have been built (qip_gb300.build.build(checked=True)).
        checked = os.environ.get("QSV_BOUNDS_CHECK", "0") not in ("", "0")
        path = _build.LIB_CHECKED if checked else _build.LIB
        if not os.path.exists(path):
            if not build_if_missing or checked:
                raise OSError(f"{path} is missing; run qip_gb300.build.build(checked={checked})")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, handle=None, what: str = "") -> None:
    """Map a status code to the reference's exception types."""
    if status == QSV_OK:
        return
    lib = load()
    msg = lib.qsv_last_error(handle).decode(errors="replace") if True else ""
    text = f"{what}: {msg}" if what else msg
    if status == QSV_ERR_INVALID:
        raise ValueError(text)
    if status == QSV_ERR_OOM:
        raise MemoryError(text)
    raise QsvError(f"{lib.qsv_status_string(status).decode()}: {text}")


def int_array(values) -> numpy.ndarray:
    return numpy.ascontiguousarray(numpy.asarray(values, dtype=numpy.int32).reshape(-1))


def ip(a: numpy.ndarray):
    return a.ctypes.data_as(_c_int_p) if a.size else None


def dp(a: numpy.ndarray):
    return a.ctypes.data_as(_c_double_p)


def c128(mat) -> numpy.ndarray:
    """Contiguous complex128 copy viewed as interleaved doubles."""
    m = numpy.ascontiguousarray(numpy.asarray(mat, dtype=numpy.complex128))
    return m.view(numpy.float64).reshape(-1)


def launch_count() -> int:
    return int(load().qsv_launch_count())
